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

PT_DI float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PT_DI float length3(float3 a) { return sqrtf(dot3(a, a)); }
PT_DI float3 normalize3(float3 a) {
    const float inv = 1.0f / sqrtf(dot3(a, a));
    return a * inv;
}
PT_DI float3 fma3(float3 a, float3 b, float3 c) {
    return f3(__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y), __fmaf_rn(a.z, b.z, c.z));
}
// fma(v, vec3(t), o) — the shader's ray-point form.
PT_DI float3 fma3s(float3 a, float t, float3 c) {
    return f3(__fmaf_rn(a.x, t, c.x), __fmaf_rn(a.y, t, c.y), __fmaf_rn(a.z, t, c.z));
}
PT_DI float3 abs3(float3 a) { return f3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
PT_DI float3 min3(float3 a, float3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
PT_DI float3 max3(float3 a, float3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }

PT_DI float sign_glsl(float x) { return (x > 0.0f) ? 1.0f : ((x < 0.0f) ? -1.0f : 0.0f); }
PT_DI float step_glsl(float edge, float x) { return (x < edge) ? 0.0f : 1.0f; }
PT_DI float mix_glsl(float x, float y, float a) { return x * (1.0f - a) + y * a; }
PT_DI float mod_glsl(float x, float y) { return x - y * floorf(x / y); }

// pow(x, N) for a positive integer constant N: ptm_powf's binary powering
// (include/pt_mathf.h) unrolled, without its checks for 1, 0, inf, NaN and
// negative x, which the products get right by themselves; only a NaN x gives
// another NaN payload than ptm_powf, so callers use it where the result is
// consumed by arithmetic that makes any NaN canonical (or x is never NaN).
template <int N>
PT_DI float pow_pos_int(float x) {
    static_assert(N > 0, "positive exponent");
    float r = 0.0f, b = x;
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
struct m3 {
    float3 c0, c1, c2;
};
// mat3 * vec3
PT_DI float3 mul_mv(const m3& m, float3 v) {
    return f3(m.c0.x * v.x + m.c1.x * v.y + m.c2.x * v.z, m.c0.y * v.x + m.c1.y * v.y + m.c2.y * v.z,
              m.c0.z * v.x + m.c1.z * v.y + m.c2.z * v.z);
}
// vec3 * mat3
PT_DI float3 mul_vm(float3 v, const m3& m) { return f3(dot3(v, m.c0), dot3(v, m.c1), dot3(v, m.c2)); }
PT_DI m3 mul_mm(const m3& a, const m3& b) { return m3{mul_mv(a, b.c0), mul_mv(a, b.c1), mul_mv(a, b.c2)}; }

// refract(I, N, eta) per the GLSL specification.
PT_DI float3 refract3(float3 I, float3 N, float eta) {
    const float d = dot3(N, I);
    const float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return f3(0.0f, 0.0f, 0.0f);
    return I * eta - N * (eta * d + sqrtf(k));
}

// RotationMatrix (src/shader.comp:143-152): mX * mY * mZ from degrees.
PT_DI m3 rotation_matrix(float3 angle) {
    angle = angle * 0.0174532925199f;
    float sx, sy, sz, cx, cy, cz;
    ptm_sincosf(angle.x, &sx, &cx);
    ptm_sincosf(angle.y, &sy, &cy);
    ptm_sincosf(angle.z, &sz, &cz);
    const m3 mX{f3(1.0f, 0.0f, 0.0f), f3(0.0f, cx, -sx), f3(0.0f, sx, cx)};
    const m3 mY{f3(cy, 0.0f, sy), f3(0.0f, 1.0f, 0.0f), f3(-sy, 0.0f, cy)};
    const m3 mZ{f3(cz, -sz, 0.0f), f3(sz, cz, 0.0f), f3(0.0f, 0.0f, 1.0f)};
    return mul_mm(mul_mm(mX, mY), mZ);
}
