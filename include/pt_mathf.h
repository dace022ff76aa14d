/*
 * pt_mathf.h — the float transcendentals of the path tracer, identical on
 * the GPU (nvcc, device code) and on the CPU (any C99/C++ compiler).
 *
 * The shader's arithmetic is float +, -, *, / and sqrt (correctly rounded
 * everywhere) plus sin, cos, exp, log, pow and acos, whose last bits differ
 * between math libraries.  The reference's cone-sampling pdf
 * (1 - cos^2 thetaMax, src/shader.comp:1027) cancels catastrophically, so a
 * one-ulp difference in a sine three bounces earlier can move a sample's XYZ
 * by 0.5%.  With these functions on both sides a path computes the same bits
 * on the GPU and on the CPU restatement, given -fmad=false / -ffp-contract=off
 * and fma written out where it is meant.
 *
 * Methods (all float, fused multiply-add written explicitly):
 *   sin/cos  Cody & Waite reduction by pi/2 (three-part constant), minimax
 *            polynomials on [-pi/4, pi/4]; quadrant from k mod 4.
 *   exp      k = rint(x/ln2), two-part ln2 reduction, minimax e^r, exact
 *            scaling by 2^k (two steps near the range ends).
 *   log      x = 2^e * m, m in [sqrt(1/2), sqrt(2)], s = f/(2+f),
 *            log(1+f) = f - s*(f - s^2*R(s^2)) with R minimax.
 *   pow      binary powering for integral |y| <= 32 (the shader's 7, 5, -5),
 *            else exp(y*log|x|) with the product's rounding error fed back.
 *   acos     via asin: x + x^3*A(x^2) on [0, 1/2]; 2*asin(sqrt((1-|x|)/2)) above.
 * Coefficients: Lawson-weighted minimax fits made by
 * pathtracer_gb300/csrc/kernel/gen_pt_mathf.py.  Measured errors (tests):
 * sin/cos <= 2 ulp for |x| < 2^16, exp/log <= 2 ulp, acos <= 2 ulp,
 * pow <= 8 ulp on the exponent range the shader uses.
 */
#ifndef PT_MATHF_H
#define PT_MATHF_H

#if !defined(__CUDACC_RTC__)
#include <stdint.h>
#endif

/* PTM_FN: inlined everywhere.  PTM_CALL: the larger functions; a GPU
 * translation unit that defines PTM_OUTLINE before including this header
 * calls them instead of inlining them at every call site (smaller hot loops,
 * fewer instruction-cache misses).  The arithmetic is the same either way. */
#if defined(__CUDACC__)
#define PTM_FN static __device__ __forceinline__
#if defined(PTM_OUTLINE)
#define PTM_CALL static __device__ __noinline__
#else
#define PTM_CALL static __device__ __forceinline__
#endif
#define PTM_FMA(a, b, c) __fmaf_rn((a), (b), (c))
PTM_FN uint32_t ptm_bits(float f) { return __float_as_uint(f); }
PTM_FN float ptm_from_bits(uint32_t u) { return __uint_as_float(u); }
#else
#include <math.h>
#include <string.h>
#define PTM_FN static inline
#define PTM_CALL static inline
#define PTM_FMA(a, b, c) fmaf((a), (b), (c))
PTM_FN uint32_t ptm_bits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
PTM_FN float ptm_from_bits(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}
#endif

#define PTM_INF ptm_from_bits(0x7f800000u)
#define PTM_NAN ptm_from_bits(0x7fc00000u)

/* pi/2, pi and ln2 as sums of three floats. */
#define PTM_PIO2_1 1.570796371e+00f
#define PTM_PIO2_2 -4.371138829e-08f
#define PTM_PIO2_3 -1.715124510e-15f
#define PTM_PI_1 3.141592741e+00f
#define PTM_PI_2 -8.742277657e-08f
#define PTM_LN2_1 6.931471825e-01f
#define PTM_LN2_2 -1.904654212e-09f
#define PTM_2_OVER_PI 6.366197467e-01f
#define PTM_LOG2E 1.442695022e+00f

/* Minimax coefficients (lowest order first). */
#define PTM_S0 -1.666666716e-01f
#define PTM_S1 8.333329111e-03f
#define PTM_S2 -1.983931288e-04f
#define PTM_S3 2.718121550e-06f
#define PTM_C0 4.166666791e-02f
#define PTM_C1 -1.388888340e-03f
#define PTM_C2 2.479945942e-05f
#define PTM_C3 -2.720575480e-07f
#define PTM_E0 5.000000000e-01f
#define PTM_E1 1.666666567e-01f
#define PTM_E2 4.166629538e-02f
#define PTM_E3 8.333496749e-03f
#define PTM_E4 1.394464867e-03f
#define PTM_E5 1.979035296e-04f
#define PTM_L0 6.666666269e-01f
#define PTM_L1 4.000033438e-01f
#define PTM_L2 2.853734791e-01f
#define PTM_L3 2.358147204e-01f
#define PTM_A0 1.666666716e-01f
#define PTM_A1 7.499948889e-02f
#define PTM_A2 4.465997219e-02f
#define PTM_A3 3.011252545e-02f
#define PTM_A4 2.460470796e-02f
#define PTM_A5 7.509485353e-03f
#define PTM_A6 3.464631364e-02f
#define PTM_T0 -3.333329856e-01f
#define PTM_T1 1.999854892e-01f
#define PTM_T2 -1.426424235e-01f
#define PTM_T3 1.095218584e-01f
#define PTM_T4 -8.403450996e-02f
#define PTM_T5 5.795760080e-02f
#define PTM_T6 -3.117785044e-02f
#define PTM_T7 1.091460884e-02f
#define PTM_T8 -1.793622272e-03f

typedef struct ptm_sc {
    float s, c;
} ptm_sc;

/* sin and cos of x together. */
PTM_FN ptm_sc ptm_sincos_inline(float x) {
    ptm_sc out;
    if (!(x - x == 0.0f)) { /* inf or NaN */
        out.s = PTM_NAN;
        out.c = PTM_NAN;
        return out;
    }
    const float k = rintf(x * PTM_2_OVER_PI);
    float r = PTM_FMA(-k, PTM_PIO2_1, x);
    r = PTM_FMA(-k, PTM_PIO2_2, r);
    r = PTM_FMA(-k, PTM_PIO2_3, r);
    /* k mod 4, exact for every finite k */
    const int q = (int)(k - 4.0f * floorf(k * 0.25f));
    const float z = r * r;
    float p = PTM_FMA(PTM_FMA(PTM_FMA(PTM_S3, z, PTM_S2), z, PTM_S1), z, PTM_S0);
    const float sr = PTM_FMA(r * z, p, r);
    float qc = PTM_FMA(PTM_FMA(PTM_FMA(PTM_C3, z, PTM_C2), z, PTM_C1), z, PTM_C0);
    const float cr = PTM_FMA(z * z, qc, PTM_FMA(-0.5f, z, 1.0f));
    float s, c;
    if (q == 0) {
        s = sr;
        c = cr;
    } else if (q == 1) {
        s = cr;
        c = -sr;
    } else if (q == 2) {
        s = -sr;
        c = -cr;
    } else {
        s = -cr;
        c = sr;
    }
    out.s = s;
    out.c = c;
    return out;
}

PTM_CALL ptm_sc ptm_sincos_v(float x) { return ptm_sincos_inline(x); }

PTM_FN float ptm_sinf_inline(float x) { return ptm_sincos_inline(x).s; }

PTM_FN void ptm_sincosf(float x, float* s_out, float* c_out) {
    const ptm_sc r = ptm_sincos_v(x);
    *s_out = r.s;
    *c_out = r.c;
}

PTM_FN float ptm_sinf(float x) {
    float s, c;
    ptm_sincosf(x, &s, &c);
    return s;
}

PTM_FN float ptm_cosf(float x) {
    float s, c;
    ptm_sincosf(x, &s, &c);
    return c;
}

/* y * 2^k for integral k in [-300, 300], exact unless the result is subnormal. */
PTM_FN float ptm_scale2(float y, int k) {
    if (k > 127) {
        y *= ptm_from_bits(0x7f000000u); /* 2^127 */
        k -= 127;
        if (k > 127) k = 127;
    } else if (k < -126) {
        y *= ptm_from_bits(0x00800000u); /* 2^-126 */
        k += 126;
        if (k < -126) k = -126;
    }
    return y * ptm_from_bits((uint32_t)(k + 127) << 23);
}

PTM_CALL float ptm_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283936f) return PTM_INF;
    if (x < -103.9720840f) return 0.0f;
    const float k = rintf(x * PTM_LOG2E);
    float r = PTM_FMA(-k, PTM_LN2_1, x);
    r = PTM_FMA(-k, PTM_LN2_2, r);
    const float p =
        PTM_FMA(PTM_FMA(PTM_FMA(PTM_FMA(PTM_FMA(PTM_E5, r, PTM_E4), r, PTM_E3), r, PTM_E2), r, PTM_E1), r, PTM_E0);
    const float em1 = PTM_FMA(r * r, p, r); /* e^r - 1 */
    return ptm_scale2(1.0f + em1, (int)k);
}

/* log(1+f) for f = m - 1, m in [sqrt(1/2), sqrt(2)]. */
PTM_FN float ptm_log1p_reduced(float f) {
    const float s = f / (2.0f + f);
    const float z = s * s;
    const float R = PTM_FMA(PTM_FMA(PTM_FMA(PTM_L3, z, PTM_L2), z, PTM_L1), z, PTM_L0);
    const float t = PTM_FMA(-z, R, f);
    return PTM_FMA(-s, t, f);
}

/* Splits finite x > 0 into 2^e * m, m in [sqrt(1/2), sqrt(2)). */
PTM_FN float ptm_frexp_sqrt2(float x, int* e_out) {
    uint32_t u = ptm_bits(x);
    int e = 0;
    if (u < 0x00800000u) { /* subnormal */
        x *= 8388608.0f;
        u = ptm_bits(x);
        e = -23;
    }
    e += (int)(u >> 23) - 127;
    float m = ptm_from_bits((u & 0x007fffffu) | 0x3f800000u);
    if (m > 1.414213538f) {
        m *= 0.5f;
        e += 1;
    }
    *e_out = e;
    return m;
}

PTM_FN float ptm_logf_inline(float x) {
    if (x != x) return x;
    if (x < 0.0f) return PTM_NAN;
    if (x == 0.0f) return -PTM_INF;
    if (x == PTM_INF) return x;
    int e;
    const float m = ptm_frexp_sqrt2(x, &e);
    const float l1p = ptm_log1p_reduced(m - 1.0f);
    const float ef = (float)e;
    return PTM_FMA(ef, PTM_LN2_1, PTM_FMA(ef, PTM_LN2_2, l1p));
}

PTM_CALL float ptm_logf(float x) { return ptm_logf_inline(x); }

/* |x|^y through exp(y*log|x|), the product's rounding error fed back. */
PTM_CALL float ptm_pow_exp_log(float ax, float y) {
    const float L = ptm_logf(ax);
    const float p = y * L;
    const float perr = PTM_FMA(y, L, -p);
    const float e = ptm_expf(p);
    return PTM_FMA(e, perr, e);
}

PTM_FN float ptm_powf(float x, float y) {
    if (y == 0.0f || x == 1.0f) return 1.0f;
    if (x != x || y != y) return PTM_NAN;
    const float ay = fabsf(y);
    const int y_int = (ay < 16777216.0f) ? (floorf(ay) == ay) : 1;
    const int y_odd = y_int && ay < 16777216.0f && ((int)(ay - 2.0f * floorf(ay * 0.5f)) == 1);
    const float ax = fabsf(x);
    const int neg = (x < 0.0f) && y_odd;
    if (x < 0.0f && !y_int) return PTM_NAN;
    if (ax == 0.0f) {
        const float r = (y > 0.0f) ? 0.0f : PTM_INF;
        return neg ? -r : r;
    }
    if (ax == PTM_INF) {
        const float r = (y > 0.0f) ? PTM_INF : 0.0f;
        return neg ? -r : r;
    }
    float r;
    if (y_int && ay <= 32.0f) {
        int n = (int)ay;
        float b = ax;
        r = 1.0f;
        while (n) {
            if (n & 1) r *= b;
            n >>= 1;
            if (n) b *= b;
        }
        if (y < 0.0f) r = 1.0f / r;
    } else {
        r = ptm_pow_exp_log(ax, y);
    }
    return neg ? -r : r;
}

PTM_FN float ptm_asin_poly(float x, float z) {
    const float A = PTM_FMA(
        PTM_FMA(PTM_FMA(PTM_FMA(PTM_FMA(PTM_FMA(PTM_A6, z, PTM_A5), z, PTM_A4), z, PTM_A3), z, PTM_A2), z, PTM_A1), z,
        PTM_A0);
    return PTM_FMA(x * z, A, x);
}

PTM_CALL float ptm_acosf(float x) {
    if (x != x) return x;
    const float ax = fabsf(x);
    if (ax > 1.0f) return PTM_NAN;
    if (ax <= 0.5f) {
        const float as = ptm_asin_poly(x, x * x);
        return PTM_PIO2_1 - (as - PTM_PIO2_2);
    }
    const float z = (1.0f - ax) * 0.5f;
    const float s = sqrtf(z);
    const float as2 = 2.0f * ptm_asin_poly(s, z);
    if (x > 0.0f) return as2;
    return PTM_PI_1 - (as2 - PTM_PI_2);
}

/* asin(x): the polynomial on |x| <= 1/2, else pi/2 - 2 asin(sqrt((1-|x|)/2)). */
PTM_CALL float ptm_asinf(float x) {
    if (x != x) return x;
    const float ax = fabsf(x);
    if (ax > 1.0f) return PTM_NAN;
    float r;
    if (ax <= 0.5f) {
        r = ptm_asin_poly(ax, ax * ax);
    } else {
        const float z = (1.0f - ax) * 0.5f;
        const float s = sqrtf(z);
        r = PTM_PIO2_1 - (2.0f * ptm_asin_poly(s, z) - PTM_PIO2_2);
    }
    return (ptm_bits(x) >> 31) ? -r : r;
}

/* atan(r) for r in [0, 1]: r + r^3 * T(r^2). */
PTM_FN float ptm_atan_poly(float r) {
    const float z = r * r;
    float t = PTM_FMA(PTM_T8, z, PTM_T7);
    t = PTM_FMA(t, z, PTM_T6);
    t = PTM_FMA(t, z, PTM_T5);
    t = PTM_FMA(t, z, PTM_T4);
    t = PTM_FMA(t, z, PTM_T3);
    t = PTM_FMA(t, z, PTM_T2);
    t = PTM_FMA(t, z, PTM_T1);
    t = PTM_FMA(t, z, PTM_T0);
    return PTM_FMA(r * z, t, r);
}

/* atan(x): |x| > 1 through pi/2 - atan(1/|x|). */
PTM_CALL float ptm_atanf(float x) {
    if (x != x) return x;
    const float a = fabsf(x);
    float r;
    if (a > 1.0f) {
        const float p = ptm_atan_poly(1.0f / a);
        r = PTM_PIO2_1 - (p - PTM_PIO2_2);
    } else {
        r = ptm_atan_poly(a);
    }
    return (ptm_bits(x) >> 31) ? -r : r;
}

/* atan2(y, x), the angle of (x, y) in [-pi, pi], with the IEEE conventions
 * for zeros and infinities; NaN in, NaN out. */
PTM_CALL float ptm_atan2f(float y, float x) {
    if (x != x || y != y) return PTM_NAN;
    const float ax = fabsf(x), ay = fabsf(y);
    const int xneg = (int)(ptm_bits(x) >> 31);
    float r;
    if (ax == PTM_INF && ay == PTM_INF) {
        r = PTM_PIO2_1 * 0.5f; /* pi/4 */
        if (xneg) r = PTM_PI_1 - (r - PTM_PI_2);
    } else if (ay == 0.0f) {
        r = xneg ? PTM_PI_1 : 0.0f;
    } else {
        const int swap = ay > ax;
        const float t = swap ? ax / ay : ay / ax;
        const float p = ptm_atan_poly(t);
        r = swap ? PTM_PIO2_1 - (p - PTM_PIO2_2) : p;
        if (xneg) r = PTM_PI_1 - (r - PTM_PI_2);
    }
    return (ptm_bits(y) >> 31) ? -r : r;
}

/* 2^x: x = k + f with k integral and |f| <= 1/2, 2^f = e^(f ln2) by the
 * exponential's polynomial. */
PTM_CALL float ptm_exp2f(float x) {
    if (x != x) return x;
    if (x > 128.0f) return PTM_INF;
    if (x < -150.0f) return 0.0f;
    const float k = rintf(x);
    const float f = x - k;
    const float r = PTM_FMA(f, PTM_LN2_1, f * PTM_LN2_2);
    const float p =
        PTM_FMA(PTM_FMA(PTM_FMA(PTM_FMA(PTM_FMA(PTM_E5, r, PTM_E4), r, PTM_E3), r, PTM_E2), r, PTM_E1), r, PTM_E0);
    const float em1 = PTM_FMA(r * r, p, r);
    return ptm_scale2(1.0f + em1, (int)k);
}

/* log2(x) = log(x) * log2(e). */
PTM_CALL float ptm_log2f(float x) { return ptm_logf(x) * PTM_LOG2E; }

#endif /* PT_MATHF_H */
