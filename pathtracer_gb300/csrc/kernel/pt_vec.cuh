// pt_vec.cuh — GLSL value semantics for the sm_103a kernels.
//
// The kernels are compiled with -fmad=false so that every a*b+c stays two
// correctly rounded operations, exactly as written; __fmaf_rn appears only
// where src/shader.comp writes fma().  Built-ins follow the GLSL
// specification: mix(x,y,a) = x*(1-a) + y*a, mod(x,y) = x - y*floor(x/y),
// normalize(v) = v * (1/sqrt(v.v)), inversesqrt(x) = 1/sqrt(x) (IEEE sqrt and
// division, never the approximate rsqrt), min/max = IEEE minNum/maxNum.
// sin, cos, exp, log, pow and acos are the pt_mathf functions, which compute
// the same bits on the GPU and on a CPU.
//
// The path arithmetic is written once for a scalar type R (float: the
// shader's method, bit for bit; double: the FP64 reference renderer).  Every
// helper here exists for float and double vectors; the m_* functions are the
// scalar built-ins of either precision (float: the exact functions the FP32
// kernels have always called; double: CUDA's double-precision ones).
#pragma once

#if !defined(__CUDACC_RTC__)
#include <cuda_runtime.h>
#include <stdint.h>
#endif

#include "../../../include/pt_mathf.h"

#define PT_DI __device__ __forceinline__

PT_DI float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
PT_DI float4 f4(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
PT_DI float4 f4s(float s) { return make_float4(s, s, s, s); }

// Vector types of a scalar type, and generic constructors (v3<R>(x, y, z)).
template <typename R> struct VecT;
template <> struct VecT<float> {
    using v2 = float2;
    using v3 = float3;
    using v4 = float4;
};
template <> struct VecT<double> {
    using v2 = double2;
    using v3 = double3;
    using v4 = double4_16a;
};
template <typename R> using V2 = typename VecT<R>::v2;
template <typename R> using V3 = typename VecT<R>::v3;
template <typename R> using V4 = typename VecT<R>::v4;
// The scalar type of a vector type.
template <typename V> struct ScalarOf { using type = decltype(V{}.x); };
template <typename V> using SOf = typename ScalarOf<V>::type;
template <typename R> PT_DI V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <typename R> PT_DI V4<R> v4(R x, R y, R z, R w) { return V4<R>{x, y, z, w}; }
template <typename R> PT_DI V4<R> v4s(R s) { return V4<R>{s, s, s, s}; }
template <typename R> PT_DI V2<R> v2(R x, R y) { return V2<R>{x, y}; }
// A literal of the shader's (float) constant in precision R: the float
// value itself for float, the decimal's double value for double.
#define PT_LIT(R, x) ((R)(sizeof(R) == 4 ? (double)(x##f) : (x)))

// Scalar built-ins by precision.
PT_DI float m_sqrt(float x) { return sqrtf(x); }
PT_DI double m_sqrt(double x) { return sqrt(x); }
PT_DI float m_fabs(float x) { return fabsf(x); }
PT_DI double m_fabs(double x) { return fabs(x); }
PT_DI float m_fmin(float a, float b) { return fminf(a, b); }
PT_DI double m_fmin(double a, double b) { return fmin(a, b); }
PT_DI float m_fmax(float a, float b) { return fmaxf(a, b); }
PT_DI double m_fmax(double a, double b) { return fmax(a, b); }
PT_DI float m_floor(float x) { return floorf(x); }
PT_DI double m_floor(double x) { return floor(x); }
PT_DI float m_ceil(float x) { return ceilf(x); }
PT_DI double m_ceil(double x) { return ceil(x); }
PT_DI float m_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
PT_DI double m_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
PT_DI float m_exp(float x) { return ptm_expf(x); }
PT_DI double m_exp(double x) { return exp(x); }
PT_DI float m_log(float x) { return ptm_logf(x); }
PT_DI double m_log(double x) { return log(x); }
PT_DI float m_pow(float x, float y) { return ptm_powf(x, y); }
PT_DI double m_pow(double x, double y) { return pow(x, y); }
PT_DI float m_acos(float x) { return ptm_acosf(x); }
PT_DI double m_acos(double x) { return acos(x); }
PT_DI void m_sincos(float x, float* s, float* c) { ptm_sincosf(x, s, c); }
PT_DI void m_sincos(double x, double* s, double* c) { sincos(x, s, c); }
PT_DI float m_sin(float x) { return ptm_sinf(x); }
PT_DI double m_sin(double x) { return sin(x); }
PT_DI float m_cos(float x) { return ptm_cosf(x); }
PT_DI double m_cos(double x) { return cos(x); }
// The inlined forms the SDF plug-ins' hot loops call.
PT_DI float m_log_inline(float x) { return ptm_logf_inline(x); }
PT_DI double m_log_inline(double x) { return log(x); }
PT_DI float m_sin_inline(float x) { return ptm_sinf_inline(x); }
PT_DI double m_sin_inline(double x) { return sin(x); }

PT_DI float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
PT_DI float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
PT_DI float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
PT_DI float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
PT_DI float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
PT_DI float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }

PT_DI float4 operator+(float4 a, float4 b) { return f4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
PT_DI float4 operator*(float4 a, float4 b) { return f4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
PT_DI float4 operator*(float4 a, float s) { return f4(a.x * s, a.y * s, a.z * s, a.w * s); }
PT_DI float4 operator/(float4 a, float s) { return f4(a.x / s, a.y / s, a.z / s, a.w / s); }

// The same operators for double vectors (the FP64 reference renderer).
PT_DI double3 operator+(double3 a, double3 b) { return double3{a.x + b.x, a.y + b.y, a.z + b.z}; }
PT_DI double3 operator-(double3 a, double3 b) { return double3{a.x - b.x, a.y - b.y, a.z - b.z}; }
PT_DI double3 operator*(double3 a, double3 b) { return double3{a.x * b.x, a.y * b.y, a.z * b.z}; }
PT_DI double3 operator/(double3 a, double3 b) { return double3{a.x / b.x, a.y / b.y, a.z / b.z}; }
PT_DI double3 operator*(double3 a, double s) { return double3{a.x * s, a.y * s, a.z * s}; }
PT_DI double3 operator-(double3 a) { return double3{-a.x, -a.y, -a.z}; }
PT_DI double4_16a operator+(double4_16a a, double4_16a b) { return double4_16a{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
PT_DI double4_16a operator*(double4_16a a, double4_16a b) { return double4_16a{a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
PT_DI double4_16a operator*(double4_16a a, double s) { return double4_16a{a.x * s, a.y * s, a.z * s, a.w * s}; }
PT_DI double4_16a operator/(double4_16a a, double s) { return double4_16a{a.x / s, a.y / s, a.z / s, a.w / s}; }

template <typename V> PT_DI auto dot3(V a, V b) -> decltype(a.x) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename V> PT_DI auto length3(V a) -> decltype(a.x) { return m_sqrt(dot3(a, a)); }
template <typename V> PT_DI V normalize3(V a) {
    const auto inv = decltype(a.x)(1) / m_sqrt(dot3(a, a));
    return a * inv;
}
template <typename V> PT_DI V fma3(V a, V b, V c) {
    return V{m_fma(a.x, b.x, c.x), m_fma(a.y, b.y, c.y), m_fma(a.z, b.z, c.z)};
}
// fma(v, vec3(t), o) — the shader's ray-point form.
template <typename V> PT_DI V fma3s(V a, decltype(a.x) t, V c) {
    return V{m_fma(a.x, t, c.x), m_fma(a.y, t, c.y), m_fma(a.z, t, c.z)};
}
template <typename V> PT_DI V abs3(V a) { return V{m_fabs(a.x), m_fabs(a.y), m_fabs(a.z)}; }
template <typename V> PT_DI V min3(V a, V b) { return V{m_fmin(a.x, b.x), m_fmin(a.y, b.y), m_fmin(a.z, b.z)}; }
template <typename V> PT_DI V max3(V a, V b) { return V{m_fmax(a.x, b.x), m_fmax(a.y, b.y), m_fmax(a.z, b.z)}; }

template <typename R> PT_DI R sign_glsl(R x) { return (x > R(0)) ? R(1) : ((x < R(0)) ? R(-1) : R(0)); }
template <typename R> PT_DI R step_glsl(R edge, R x) { return (x < edge) ? R(0) : R(1); }
template <typename R> PT_DI R mix_glsl(R x, R y, R a) { return x * (R(1) - a) + y * a; }
template <typename R> PT_DI R mod_glsl(R x, R y) { return x - y * m_floor(x / y); }

// pow(x, N) for a positive integer constant N: ptm_powf's binary powering
// (include/pt_mathf.h) unrolled, without its checks for 1, 0, inf, NaN and
// negative x, which the products get right by themselves; only a NaN x gives
// another NaN payload than ptm_powf, so callers use it where the result is
// consumed by arithmetic that makes any NaN canonical (or x is never NaN).
template <int N, typename R>
PT_DI R pow_pos_int(R x) {
    static_assert(N > 0, "positive exponent");
    R r = R(0), b = x;
    bool have = false;
#pragma unroll
    for (int n = N; n != 0; n >>= 1) {
        if (n & 1) {
            r = have ? r * b : b;
            have = true;
        }
        if (n >> 1) b = b * b;
    }
    return r;
}

// mat3 as three columns.
template <typename R> struct M3 {
    V3<R> c0, c1, c2;
};
using m3 = M3<float>;
// mat3 * vec3
template <typename R> PT_DI V3<R> mul_mv(const M3<R>& m, V3<R> v) {
    return v3<R>(m.c0.x * v.x + m.c1.x * v.y + m.c2.x * v.z, m.c0.y * v.x + m.c1.y * v.y + m.c2.y * v.z,
                 m.c0.z * v.x + m.c1.z * v.y + m.c2.z * v.z);
}
// vec3 * mat3
template <typename R> PT_DI V3<R> mul_vm(V3<R> v, const M3<R>& m) {
    return v3<R>(dot3(v, m.c0), dot3(v, m.c1), dot3(v, m.c2));
}
template <typename R> PT_DI M3<R> mul_mm(const M3<R>& a, const M3<R>& b) {
    return M3<R>{mul_mv(a, b.c0), mul_mv(a, b.c1), mul_mv(a, b.c2)};
}

// refract(I, N, eta) per the GLSL specification.
template <typename V> PT_DI V refract3(V I, V N, decltype(I.x) eta) {
    using R = decltype(I.x);
    const R d = dot3(N, I);
    const R k = R(1) - eta * eta * (R(1) - d * d);
    if (k < R(0)) return V{R(0), R(0), R(0)};
    return I * eta - N * (eta * d + m_sqrt(k));
}

// RotationMatrix (src/shader.comp:143-152): mX * mY * mZ from degrees.
template <typename V, typename R = SOf<V>> PT_DI M3<R> rotation_matrix(V angle) {
    angle = angle * PT_LIT(R, 0.0174532925199);
    R sx, sy, sz, cx, cy, cz;
    m_sincos(angle.x, &sx, &cx);
    m_sincos(angle.y, &sy, &cy);
    m_sincos(angle.z, &sz, &cz);
    const R o = R(1), z = R(0);
    const M3<R> mX{v3<R>(o, z, z), v3<R>(z, cx, -sx), v3<R>(z, sx, cx)};
    const M3<R> mY{v3<R>(cy, z, sy), v3<R>(z, o, z), v3<R>(-sy, z, cy)};
    const M3<R> mZ{v3<R>(cz, -sz, z), v3<R>(sz, cz, z), v3<R>(z, z, o)};
    return mul_mm(mul_mm(mX, mY), mZ);
}
