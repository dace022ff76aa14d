// pt_glsl_shim.h — the part of GLSL that scene SDF snippets use, as C++ for
// the runtime-compiled kernels (NVRTC) and for the host (g++), with the same
// float arithmetic on both: IEEE +, -, *, / and sqrt, fma written out, and
// pt_mathf for the transcendentals.  Snippets reach it through
// pt_glsl_translate (pt_glsl.cpp), which rewrites float literals, swizzles and
// parameter qualifiers into this vocabulary.
//
// Covered: float/int/uint/bool, vec2/vec3/vec4 (constructors, component
// access, read swizzles as member calls, swizzle assignment through set_<sw>
// members, arithmetic with vectors and scalars), uvec2/ivec2 and
// uvec3, bvec2/bvec3/bvec4 (constructors, components), mat2/mat3 (constructors
// from columns or scalars, matrix * vector, mat3 * mat3), vector indexing
// v[i], structs (declared in the snippet), and the built-ins
// abs sign floor ceil fract round trunc mod min max clamp mix step
// smoothstep sqrt inversesqrt pow exp exp2 log log2 sin cos tan asin acos
// atan (one and two arguments) length distance dot cross normalize reflect
// fma radians degrees faceforward refract, plus the shader's smin for floats
// and vec2.
#pragma once

#if defined(__CUDACC__)
#define PTG_FN static __device__ __forceinline__
#define PTG_M __device__ __forceinline__
#else
#define PTG_FN static inline
#define PTG_M inline
#endif

#include "../../../include/pt_mathf.h"

// The scalar functions the vocabulary is built on.  The FP64 reference
// renderer compiles the same snippet text with every GLSL float a double:
// its program defines PTG_DOUBLE and `float` as `double` around this header
// and the snippets, and the functions below become CUDA's double-precision
// ones (literals stay the float values the text writes).
#if defined(PTG_DOUBLE)
#define PTG_ABS(a) ::fabs(a)
#define PTG_FLOOR(a) ::floor(a)
#define PTG_CEIL(a) ::ceil(a)
#define PTG_SQRT(a) ::sqrt(a)
#define PTG_ROUND(a) ::round(a)
#define PTG_TRUNC(a) ::trunc(a)
#define PTG_MIN(a, b) ::fmin((double)(a), (double)(b))
#define PTG_MAX(a, b) ::fmax((double)(a), (double)(b))
#define PTG_FMA(a, b, c) ::fma((double)(a), (double)(b), (double)(c))
#define PTG_EXP(a) ::exp(a)
#define PTG_LOG(a) ::log(a)
#define PTG_SIN(a) ::sin(a)
#define PTG_COS(a) ::cos(a)
#define PTG_SINCOS(a, s, c) ::sincos((a), (s), (c))
#define PTG_ACOS(a) ::acos(a)
#define PTG_ASIN(a) ::asin(a)
#define PTG_ATAN(a) ::atan(a)
#define PTG_ATAN2(y, x) ::atan2((double)(y), (double)(x))
#define PTG_EXP2(a) ::exp2(a)
#define PTG_LOG2(a) ::log2(a)
#define PTG_POW(a, b) ::pow((double)(a), (double)(b))
#else
#define PTG_ABS(a) fabsf(a)
#define PTG_FLOOR(a) floorf(a)
#define PTG_CEIL(a) ceilf(a)
#define PTG_SQRT(a) sqrtf(a)
#define PTG_ROUND(a) roundf(a)
#define PTG_TRUNC(a) truncf(a)
#define PTG_MIN(a, b) fminf((a), (b))
#define PTG_MAX(a, b) fmaxf((a), (b))
#define PTG_FMA(a, b, c) PTM_FMA((a), (b), (c))
#define PTG_EXP(a) ptm_expf(a)
#define PTG_LOG(a) ptm_logf(a)
#define PTG_SIN(a) ptm_sinf(a)
#define PTG_COS(a) ptm_cosf(a)
#define PTG_SINCOS(a, s, c) ptm_sincosf((a), (s), (c))
#define PTG_ACOS(a) ptm_acosf(a)
#define PTG_ASIN(a) ptm_asinf(a)
#define PTG_ATAN(a) ptm_atanf(a)
#define PTG_ATAN2(y, x) ptm_atan2f((y), (x))
#define PTG_EXP2(a) ptm_exp2f(a)
#define PTG_LOG2(a) ptm_log2f(a)
#define PTG_POW(a, b) ptm_powf((a), (b))
#endif

namespace ptg {

typedef unsigned int uint;

struct vec2;
struct vec3;
struct vec4;

struct vec2 {
    float x, y;
    PTG_M float& operator[](int i) { return i == 0 ? x : y; }
    PTG_M float operator[](int i) const { return i == 0 ? x : y; }
    PTG_M vec2() : x(0.0f), y(0.0f) {}
    PTG_M explicit vec2(float s) : x(s), y(s) {}
    PTG_M vec2(float a, float b) : x(a), y(b) {}
    PTG_M void set_xy(vec2 v);
    PTG_M void set_yx(vec2 v);
    PTG_M explicit vec2(const struct uvec2& v);  // vec2(uvec2): component conversion
    PTG_M vec2 xx() const { return vec2(x, x); }
    PTG_M vec2 xy() const { return vec2(x, y); }
    PTG_M vec2 yx() const { return vec2(y, x); }
    PTG_M vec2 yy() const { return vec2(y, y); }
#define PTG_V2S3(A, B, C) PTG_M vec3 A##B##C() const;
    PTG_V2S3(x, x, x) PTG_V2S3(x, x, y) PTG_V2S3(x, y, x) PTG_V2S3(x, y, y) PTG_V2S3(y, x, x) PTG_V2S3(y, x, y)
    PTG_V2S3(y, y, x) PTG_V2S3(y, y, y)
#undef PTG_V2S3
};

struct vec3 {
    float x, y, z;
    PTG_M float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    PTG_M float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    PTG_M vec3() : x(0.0f), y(0.0f), z(0.0f) {}
    PTG_M explicit vec3(float s) : x(s), y(s), z(s) {}
    PTG_M vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    PTG_M vec3(vec2 a, float c) : x(a.x), y(a.y), z(c) {}
    PTG_M vec3(float a, vec2 b) : x(a), y(b.x), z(b.y) {}
#define PTG_S2(A, B) \
    PTG_M vec2 A##B() const { return vec2(A, B); }
    PTG_S2(x, x) PTG_S2(x, y) PTG_S2(x, z) PTG_S2(y, x) PTG_S2(y, y) PTG_S2(y, z) PTG_S2(z, x) PTG_S2(z, y)
    PTG_S2(z, z)
#define PTG_S3(A, B, C) \
    PTG_M vec3 A##B##C() const { return vec3(A, B, C); }
#define PTG_S3B(A, B) PTG_S3(A, B, x) PTG_S3(A, B, y) PTG_S3(A, B, z)
#define PTG_S3A(A) PTG_S3B(A, x) PTG_S3B(A, y) PTG_S3B(A, z)
    PTG_S3A(x) PTG_S3A(y) PTG_S3A(z)
#define PTG_SET2(A, B) \
    PTG_M void set_##A##B(vec2 v) { A = v.x; B = v.y; }
    PTG_SET2(x, y) PTG_SET2(x, z) PTG_SET2(y, x) PTG_SET2(y, z) PTG_SET2(z, x) PTG_SET2(z, y)
};

struct vec4 {
    float x, y, z, w;
    PTG_M float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    PTG_M float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    PTG_M vec4() : x(0.0f), y(0.0f), z(0.0f), w(0.0f) {}
    PTG_M explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    PTG_M vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    PTG_M vec4(vec3 a, float d) : x(a.x), y(a.y), z(a.z), w(d) {}
    PTG_M vec4(vec2 a, vec2 b) : x(a.x), y(a.y), z(b.x), w(b.y) {}
    PTG_M vec3 xyz() const { return vec3(x, y, z); }
    PTG_M vec2 xy() const { return vec2(x, y); }
    PTG_M vec2 zw() const { return vec2(z, w); }
    PTG_M void set_xy(vec2 v) { x = v.x; y = v.y; }
    PTG_M void set_zw(vec2 v) { z = v.x; w = v.y; }
    PTG_M void set_xyz(vec3 v) { x = v.x; y = v.y; z = v.z; }
};
PTG_M void vec2::set_xy(vec2 v) { x = v.x; y = v.y; }
PTG_M void vec2::set_yx(vec2 v) { y = v.x; x = v.y; }
#define PTG_V2S3(A, B, C) \
    PTG_M vec3 vec2::A##B##C() const { return vec3(A, B, C); }
PTG_V2S3(x, x, x) PTG_V2S3(x, x, y) PTG_V2S3(x, y, x) PTG_V2S3(x, y, y) PTG_V2S3(y, x, x) PTG_V2S3(y, x, y)
PTG_V2S3(y, y, x) PTG_V2S3(y, y, y)
#undef PTG_V2S3

// Integer and boolean vectors: constructors and components (GLSL's
// arithmetic on them is not covered).
struct uvec2 {
    uint x, y;
    PTG_M uvec2() : x(0u), y(0u) {}
    PTG_M explicit uvec2(uint s) : x(s), y(s) {}
    PTG_M uvec2(uint a, uint b) : x(a), y(b) {}
};
PTG_M vec2::vec2(const uvec2& v) : x((float)v.x), y((float)v.y) {}
struct uvec3 {
    uint x, y, z;
    PTG_M uvec3() : x(0u), y(0u), z(0u) {}
    PTG_M explicit uvec3(uint s) : x(s), y(s), z(s) {}
    PTG_M uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};
struct ivec2 {
    int x, y;
    PTG_M ivec2() : x(0), y(0) {}
    PTG_M explicit ivec2(int s) : x(s), y(s) {}
    PTG_M ivec2(int a, int b) : x(a), y(b) {}
};
struct bvec2 {
    bool x, y;
    PTG_M bvec2() : x(false), y(false) {}
    PTG_M explicit bvec2(bool s) : x(s), y(s) {}
    PTG_M bvec2(bool a, bool b) : x(a), y(b) {}
};
struct bvec3 {
    bool x, y, z;
    PTG_M bool operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    PTG_M bvec3() : x(false), y(false), z(false) {}
    PTG_M explicit bvec3(bool s) : x(s), y(s), z(s) {}
    PTG_M bvec3(bool a, bool b, bool c) : x(a), y(b), z(c) {}
};
struct bvec4 {
    bool x, y, z, w;
    PTG_M bool operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    PTG_M bvec4() : x(false), y(false), z(false), w(false) {}
    PTG_M explicit bvec4(bool s) : x(s), y(s), z(s), w(s) {}
    PTG_M bvec4(bool a, bool b, bool c, bool d) : x(a), y(b), z(c), w(d) {}
    PTG_M bvec2 xy() const { return bvec2(x, y); }
    PTG_M bvec2 zw() const { return bvec2(z, w); }
    PTG_M void set_xy(bvec2 v) { x = v.x; y = v.y; }
    PTG_M void set_zw(bvec2 v) { z = v.x; w = v.y; }
};

// Component-wise arithmetic.
#define PTG_VV(OP)                                                                                      \
    PTG_FN vec2 operator OP(vec2 a, vec2 b) { return vec2(a.x OP b.x, a.y OP b.y); }                  \
    PTG_FN vec3 operator OP(vec3 a, vec3 b) { return vec3(a.x OP b.x, a.y OP b.y, a.z OP b.z); }      \
    PTG_FN vec4 operator OP(vec4 a, vec4 b) { return vec4(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w); }
PTG_VV(+)
PTG_VV(-)
PTG_VV(*)
#undef PTG_VV
PTG_FN vec2 operator/(vec2 a, vec2 b) { return vec2(a.x / b.x, a.y / b.y); }
PTG_FN vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
PTG_FN vec4 operator/(vec4 a, vec4 b) { return vec4(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w); }
// With a scalar on either side, and the assignment forms.
#define PTG_OPS(V)                                                                             \
    PTG_FN V operator+(V a, float s) { return a + V(s); }                                      \
    PTG_FN V operator-(V a, float s) { return a - V(s); }                                      \
    PTG_FN V operator*(V a, float s) { return a * V(s); }                                      \
    PTG_FN V operator/(V a, float s) { return a / V(s); }                                      \
    PTG_FN V operator+(float s, V a) { return V(s) + a; }                                      \
    PTG_FN V operator-(float s, V a) { return V(s) - a; }                                      \
    PTG_FN V operator*(float s, V a) { return V(s) * a; }                                      \
    PTG_FN V operator/(float s, V a) { return V(s) / a; }                                      \
    PTG_FN V& operator+=(V& a, V b) { return a = a + b; }                                      \
    PTG_FN V& operator-=(V& a, V b) { return a = a - b; }                                      \
    PTG_FN V& operator*=(V& a, V b) { return a = a * b; }                                      \
    PTG_FN V& operator/=(V& a, V b) { return a = a / b; }                                      \
    PTG_FN V& operator+=(V& a, float s) { return a = a + s; }                                  \
    PTG_FN V& operator-=(V& a, float s) { return a = a - s; }                                  \
    PTG_FN V& operator*=(V& a, float s) { return a = a * s; }                                  \
    PTG_FN V& operator/=(V& a, float s) { return a = a / s; }
PTG_OPS(vec2)
PTG_OPS(vec3)
PTG_OPS(vec4)

// Negation flips signs (-(+0) is -0, unlike 0 - a).
PTG_FN vec2 operator-(vec2 a) { return vec2(-a.x, -a.y); }
PTG_FN vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
PTG_FN vec4 operator-(vec4 a) { return vec4(-a.x, -a.y, -a.z, -a.w); }

// An integer vector in arithmetic with a float vector converts to it.
PTG_FN vec2 to_vec2(ivec2 v) { return vec2((float)v.x, (float)v.y); }
PTG_FN vec2 operator+(vec2 a, ivec2 b) { return a + to_vec2(b); }
PTG_FN vec2 operator-(vec2 a, ivec2 b) { return a - to_vec2(b); }
PTG_FN vec2 operator*(vec2 a, ivec2 b) { return a * to_vec2(b); }
PTG_FN vec2 operator/(vec2 a, ivec2 b) { return a / to_vec2(b); }
PTG_FN vec2& operator+=(vec2& a, ivec2 b) { return a = a + b; }
PTG_FN vec2& operator-=(vec2& a, ivec2 b) { return a = a - b; }
PTG_FN vec2& operator*=(vec2& a, ivec2 b) { return a = a * b; }
PTG_FN vec2& operator/=(vec2& a, ivec2 b) { return a = a / b; }

// Apply a float function component-wise.
#define PTG_MAP1(NAME, F)                                                                       \
    PTG_FN float NAME(float a) { return F(a); }                                                 \
    PTG_FN vec2 NAME(vec2 a) { return vec2(F(a.x), F(a.y)); }                                   \
    PTG_FN vec3 NAME(vec3 a) { return vec3(F(a.x), F(a.y), F(a.z)); }                           \
    PTG_FN vec4 NAME(vec4 a) { return vec4(F(a.x), F(a.y), F(a.z), F(a.w)); }
#define PTG_MAP2(NAME, F)                                                                       \
    PTG_FN float NAME(float a, float b) { return F(a, b); }                                     \
    PTG_FN vec2 NAME(vec2 a, vec2 b) { return vec2(F(a.x, b.x), F(a.y, b.y)); }                 \
    PTG_FN vec3 NAME(vec3 a, vec3 b) { return vec3(F(a.x, b.x), F(a.y, b.y), F(a.z, b.z)); }    \
    PTG_FN vec4 NAME(vec4 a, vec4 b) { return vec4(F(a.x, b.x), F(a.y, b.y), F(a.z, b.z), F(a.w, b.w)); } \
    PTG_FN vec2 NAME(vec2 a, float b) { return NAME(a, vec2(b)); }                              \
    PTG_FN vec3 NAME(vec3 a, float b) { return NAME(a, vec3(b)); }                              \
    PTG_FN vec4 NAME(vec4 a, float b) { return NAME(a, vec4(b)); }

PTG_FN float f_abs(float a) { return PTG_ABS(a); }
PTG_FN float f_sign(float a) { return (a > 0.0f) ? 1.0f : ((a < 0.0f) ? -1.0f : 0.0f); }
PTG_FN float f_floor(float a) { return PTG_FLOOR(a); }
PTG_FN float f_ceil(float a) { return PTG_CEIL(a); }
PTG_FN float f_fract(float a) { return a - PTG_FLOOR(a); }
PTG_FN float f_sqrt(float a) { return PTG_SQRT(a); }
PTG_FN float f_isqrt(float a) { return 1.0f / PTG_SQRT(a); }
PTG_FN float f_exp(float a) { return PTG_EXP(a); }
PTG_FN float f_log(float a) { return PTG_LOG(a); }
PTG_FN float f_sin(float a) { return PTG_SIN(a); }
PTG_FN float f_cos(float a) { return PTG_COS(a); }
PTG_FN float f_acos(float a) { return PTG_ACOS(a); }
PTG_FN float f_asin(float a) { return PTG_ASIN(a); }
PTG_FN float f_atan(float a) { return PTG_ATAN(a); }
PTG_FN float f_atan2(float y, float x) { return PTG_ATAN2(y, x); }
PTG_FN float f_tan(float a) {
    float s, c;
    PTG_SINCOS(a, &s, &c);
    return s / c;
}
PTG_FN float f_exp2(float a) { return PTG_EXP2(a); }
PTG_FN float f_log2(float a) { return PTG_LOG2(a); }
PTG_FN float f_round(float a) { return PTG_ROUND(a); }
PTG_FN float f_trunc(float a) { return PTG_TRUNC(a); }
PTG_FN float f_radians(float a) { return a * 0.01745329252f; }
PTG_FN float f_degrees(float a) { return a * 57.29577951f; }
PTG_FN float f_mod(float a, float b) { return a - b * PTG_FLOOR(a / b); }
PTG_FN float f_min(float a, float b) { return PTG_MIN(a, b); }
PTG_FN float f_max(float a, float b) { return PTG_MAX(a, b); }
PTG_FN float f_pow(float a, float b) { return PTG_POW(a, b); }
PTG_FN float f_step(float edge, float a) { return (a < edge) ? 0.0f : 1.0f; }

PTG_MAP1(abs, f_abs)
PTG_MAP1(sign, f_sign)
PTG_MAP1(floor, f_floor)
PTG_MAP1(ceil, f_ceil)
PTG_MAP1(fract, f_fract)
PTG_MAP1(sqrt, f_sqrt)
PTG_MAP1(inversesqrt, f_isqrt)
PTG_MAP1(exp, f_exp)
PTG_MAP1(log, f_log)
PTG_MAP1(sin, f_sin)
PTG_MAP1(cos, f_cos)
PTG_MAP1(acos, f_acos)
PTG_MAP1(asin, f_asin)
PTG_MAP1(atan, f_atan)
PTG_MAP1(tan, f_tan)
PTG_MAP1(exp2, f_exp2)
PTG_MAP1(log2, f_log2)
PTG_MAP1(round, f_round)
PTG_MAP1(trunc, f_trunc)
PTG_MAP1(radians, f_radians)
PTG_MAP1(degrees, f_degrees)
PTG_MAP2(mod, f_mod)
PTG_MAP2(min, f_min)
PTG_MAP2(max, f_max)
PTG_MAP2(pow, f_pow)
PTG_MAP2(step, f_step)
PTG_MAP2(atan, f_atan2)  // atan(y, x)
PTG_FN vec2 step(float e, vec2 a) { return step(vec2(e), a); }
PTG_FN vec3 step(float e, vec3 a) { return step(vec3(e), a); }

PTG_FN float fma(float a, float b, float c) { return PTG_FMA(a, b, c); }
PTG_FN vec2 fma(vec2 a, vec2 b, vec2 c) { return vec2(PTG_FMA(a.x, b.x, c.x), PTG_FMA(a.y, b.y, c.y)); }
PTG_FN vec3 fma(vec3 a, vec3 b, vec3 c) {
    return vec3(PTG_FMA(a.x, b.x, c.x), PTG_FMA(a.y, b.y, c.y), PTG_FMA(a.z, b.z, c.z));
}
PTG_FN vec4 fma(vec4 a, vec4 b, vec4 c) {
    return vec4(PTG_FMA(a.x, b.x, c.x), PTG_FMA(a.y, b.y, c.y), PTG_FMA(a.z, b.z, c.z), PTG_FMA(a.w, b.w, c.w));
}

template <typename V> PTG_FN V clamp(V a, V lo, V hi) { return min(max(a, lo), hi); }
PTG_FN float clamp(float a, float lo, float hi) { return min(max(a, lo), hi); }
PTG_FN vec2 clamp(vec2 a, float lo, float hi) { return min(max(a, lo), hi); }
PTG_FN vec3 clamp(vec3 a, float lo, float hi) { return min(max(a, lo), hi); }
PTG_FN float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
PTG_FN vec2 mix(vec2 a, vec2 b, float t) { return a * (1.0f - t) + b * t; }
PTG_FN vec3 mix(vec3 a, vec3 b, float t) { return a * (1.0f - t) + b * t; }
PTG_FN vec3 mix(vec3 a, vec3 b, vec3 t) { return a * (1.0f - t) + b * t; }
PTG_FN vec4 mix(vec4 a, vec4 b, float t) { return a * (1.0f - t) + b * t; }
PTG_FN vec4 mix(vec4 a, vec4 b, vec4 t) { return a * (1.0f - t) + b * t; }
PTG_FN float smoothstep(float e0, float e1, float x) {
    const float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

PTG_FN float dot(float a, float b) { return a * b; }
PTG_FN float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
PTG_FN float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PTG_FN float dot(vec4 a, vec4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
template <typename V> PTG_FN float length(V a) { return PTG_SQRT(dot(a, a)); }
PTG_FN float length(float a) { return PTG_ABS(a); }
template <typename V> PTG_FN float distance(V a, V b) { return length(a - b); }
template <typename V> PTG_FN V normalize(V a) { return a * (1.0f / PTG_SQRT(dot(a, a))); }
PTG_FN vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <typename V> PTG_FN V reflect(V i, V n) { return i - 2.0f * dot(n, i) * n; }
template <typename V> PTG_FN V faceforward(V n, V i, V nref) { return dot(nref, i) < 0.0f ? n : -n; }
template <typename V> PTG_FN V refract(V i, V n, float eta) {
    const float d = dot(n, i);
    const float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return V(0.0f);
    return eta * i - (eta * d + PTG_SQRT(k)) * n;
}

struct mat2 {
    vec2 c0, c1;
    PTG_M mat2(vec2 a, vec2 b) : c0(a), c1(b) {}
    PTG_M mat2(float a, float b, float c, float d) : c0(a, b), c1(c, d) {}
};
PTG_FN vec2 operator*(mat2 m, vec2 v) { return vec2(m.c0.x * v.x + m.c1.x * v.y, m.c0.y * v.x + m.c1.y * v.y); }
PTG_FN vec2 operator*(vec2 v, mat2 m) { return vec2(dot(v, m.c0), dot(v, m.c1)); }
struct mat3 {
    vec3 c0, c1, c2;
    PTG_M mat3(vec3 a, vec3 b, vec3 c) : c0(a), c1(b), c2(c) {}
    // column-major, as GLSL fills a matrix from scalars
    PTG_M mat3(float a, float b, float c, float d, float e, float f, float g, float h, float i)
        : c0(a, b, c), c1(d, e, f), c2(g, h, i) {}
    PTG_M vec3& operator[](int j) { return j == 0 ? c0 : (j == 1 ? c1 : c2); }  // column j
    PTG_M vec3 operator[](int j) const { return j == 0 ? c0 : (j == 1 ? c1 : c2); }
};
PTG_FN vec3 operator*(mat3 m, vec3 v) {
    return vec3(m.c0.x * v.x + m.c1.x * v.y + m.c2.x * v.z, m.c0.y * v.x + m.c1.y * v.y + m.c2.y * v.z,
                m.c0.z * v.x + m.c1.z * v.y + m.c2.z * v.z);
}
PTG_FN vec3 operator*(vec3 v, mat3 m) { return vec3(dot(v, m.c0), dot(v, m.c1), dot(v, m.c2)); }
PTG_FN mat3 operator*(mat3 a, mat3 b) { return mat3(a * b.c0, a * b.c1, a * b.c2); }
PTG_FN vec3& operator*=(vec3& v, mat3 m) { return v = v * m; }

// The shader's polynomial smooth minimum (src/shader.comp:686-702), k = 0.02 * 6,
// with its ONEBYTHREE constant (src/shader.comp:10).
PTG_FN float smin(float x, float y) {
    float k = 0.02f;
    k *= 6.0f;
    const float h = PTG_MAX(k - PTG_ABS(x - y), 0.0f) / k;
    const float m = h * h * h * 0.5f;
    const float s = m * k * 0.3333333f;
    return PTG_MIN(x, y) - s;
}
PTG_FN vec2 smin(vec2 x, vec2 y) {
    float k = 0.02f;
    k *= 6.0f;
    const float h = PTG_MAX(k - PTG_ABS(x.x - y.x), 0.0f) / k;
    const float m = h * h * h * 0.5f;
    const float s = m * k * 0.3333333f;
    return (x.x < y.x) ? vec2(x.x - s, x.y + (y.y - x.y) * m) : vec2(y.x - s, x.y + (y.y - x.y) * (1.0f - m));
}

}  // namespace ptg
