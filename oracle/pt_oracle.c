/*
 * pt_oracle.c — scalar CPU restatement of src/shader.comp (phyastro/PathTracer).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle for libpt_cuda.  Each function below
 * cites the shader lines it restates (SC = src/shader.comp) and evaluates the
 * GLSL expressions in the same order, in float, without contraction
 * (compiled with -ffp-contract=off); `fma` is called exactly where the shader
 * writes fma.  GLSL built-ins follow their specification:
 *   mix(x,y,a) = x*(1-a) + y*a        mod(x,y) = x - y*floor(x/y)
 *   normalize(v) = v * (1/sqrt(v.v))  length(v) = sqrt(v.v)
 *   inversesqrt(x) = 1/sqrt(x)        sign, step, faceforward, refract as specified
 *   min/max = IEEE minNum/maxNum (fminf/fmaxf)
 * Transcendentals are the pt_mathf functions (include/pt_mathf.h), the same
 * float algorithms the GPU kernels run, so both sides compute identical bits.
 * Out-of-range reads of the uniform arrays return 0 (robust buffer access).
 *
 * Pinned against the reference's own shader: the reference has no tests or
 * golden vectors and cannot run here as a program (Vulkan/Windows), but its
 * shader builds for the CPU from its source through the repository's GLSL
 * translator (oracle/ref_shader.py), and this restatement agrees with it bit
 * for bit: single functions on seeded inputs, and every sample of the
 * reference's own scene files (tests/test_oracle_reference.py).  Known-answer
 * values derived from the formulas are in tests/test_oracle_kat.py.
 */
#include "pt_oracle.h"
#include "../include/pt_mathf.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_F 3.141592653589792623810034526344f /* SC:9 */
#define ONEBYTHREE 0.3333333f                  /* SC:10 */
#define MAXDIST 1e5f                           /* SC:8 */
#define COUNT(c, k) do { if ((c)->cnt) (c)->cnt[k]++; } while (0)

/* ------------------------------------------------------------------ */
/* GLSL value types and built-ins                                      */
/* ------------------------------------------------------------------ */
typedef struct { float x, y; } vec2;
typedef struct { float x, y, z; } vec3;
typedef struct { float x, y, z, w; } vec4;
typedef struct { vec3 c0, c1, c2; } mat3; /* columns */

static inline vec2 mk2(float x, float y) { vec2 r = {x, y}; return r; }
static inline vec3 mk3(float x, float y, float z) { vec3 r = {x, y, z}; return r; }
static inline vec4 mk4(float x, float y, float z, float w) { vec4 r = {x, y, z, w}; return r; }
static inline vec4 s4(float s) { return mk4(s, s, s, s); }

static inline vec3 add3(vec3 a, vec3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline vec3 sub3(vec3 a, vec3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline vec3 mul3(vec3 a, vec3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline vec3 div3(vec3 a, vec3 b) { return mk3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline vec3 scl3(vec3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
static inline vec3 neg3(vec3 a) { return mk3(-a.x, -a.y, -a.z); }
static inline vec3 fma3(vec3 a, vec3 b, vec3 c) { return mk3(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y), fmaf(a.z, b.z, c.z)); }
static inline vec3 abs3(vec3 a) { return mk3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
static inline vec3 min3(vec3 a, vec3 b) { return mk3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
static inline vec3 max3(vec3 a, vec3 b) { return mk3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
static inline float dot3(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float length3(vec3 a) { return sqrtf(dot3(a, a)); }
static inline vec3 normalize3(vec3 a) { float inv = 1.0f / sqrtf(dot3(a, a)); return scl3(a, inv); }

static inline vec4 add4(vec4 a, vec4 b) { return mk4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline vec4 mul4(vec4 a, vec4 b) { return mk4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
static inline vec4 scl4(vec4 a, float s) { return mk4(a.x * s, a.y * s, a.z * s, a.w * s); }
static inline vec4 div4s(vec4 a, float s) { return mk4(a.x / s, a.y / s, a.z / s, a.w / s); }

static inline float signf_glsl(float x) { return (x > 0.0f) ? 1.0f : ((x < 0.0f) ? -1.0f : 0.0f); }
static inline float stepf_glsl(float edge, float x) { return (x < edge) ? 0.0f : 1.0f; }
static inline float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
static inline float modf_glsl(float x, float y) { return x - y * floorf(x / y); }

/* mat3 * vec3: sum over columns. */
static inline vec3 mat_mul_vec(mat3 m, vec3 v) {
    return mk3(m.c0.x * v.x + m.c1.x * v.y + m.c2.x * v.z,
               m.c0.y * v.x + m.c1.y * v.y + m.c2.y * v.z,
               m.c0.z * v.x + m.c1.z * v.y + m.c2.z * v.z);
}
/* vec3 * mat3: dot with each column. */
static inline vec3 vec_mul_mat(vec3 v, mat3 m) { return mk3(dot3(v, m.c0), dot3(v, m.c1), dot3(v, m.c2)); }
static inline mat3 mat_mul_mat(mat3 a, mat3 b) {
    mat3 r;
    r.c0 = mat_mul_vec(a, b.c0);
    r.c1 = mat_mul_vec(a, b.c1);
    r.c2 = mat_mul_vec(a, b.c2);
    return r;
}

/* refract(I, N, eta) per the GLSL specification. */
static inline vec3 refract3(vec3 I, vec3 N, float eta) {
    float d = dot3(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return mk3(0.0f, 0.0f, 0.0f);
    return sub3(scl3(I, eta), scl3(N, eta * d + sqrtf(k)));
}

/* ------------------------------------------------------------------ */
/* Per-dispatch state                                                  */
/* ------------------------------------------------------------------ */
typedef struct {
    const pt_ubo* u;
    const pt_push* pc;
    const pt_sdf_plugin* plug;
    int nplug;
    vec3 cameraPos; /* SC:127 */
    /* trace bookkeeping (not part of the shader's arithmetic) */
    int last_hit;      /* object index of the last successful hit in Intersection */
    int light_pick;
    int shadow_state;
    uint64_t* cnt;     /* work counters of this thread (PTO_C_*) or NULL */
    const pt_scene_ext* x; /* full-form extensions (all zero: the reference's method) */
    int medium;        /* extension dielectrics: bit 0 inside one, bit 1 once the path carries l.x alone */
} ctx_t;

static const pt_scene_ext kNoExt; /* all zero: the reference's method */

static inline float OBJ(const ctx_t* c, int i) { return (i >= 0 && i < PT_MAX_OBJECTS_SIZE) ? c->u->objects[i] : 0.0f; }
static inline float SDFS(const ctx_t* c, int i) { return (i >= 0 && i < PT_MAX_SDFS_SIZE) ? c->u->sdfs[i] : 0.0f; }
static inline float MATS(const ctx_t* c, int i) { return (i >= 0 && i < PT_MAX_MATERIALS_SIZE) ? c->u->materials[i] : 0.0f; }
static inline float LIGHTS(const ctx_t* c, int i) { return (i >= 0 && i < PT_MAX_LIGHTS_SIZE) ? c->u->lights[i] : 0.0f; }
static inline float LIGHTIDS(const ctx_t* c, int i) { return (i >= 0 && i < PT_MAX_LIGHTIDS_SIZE) ? c->u->lightIDs[i] : 0.0f; }
static inline float CIE(const ctx_t* c, int i) { return (i >= 0 && i < PT_CIE_TABLE_SIZE) ? c->u->CIEXYZ1931[i] : 0.0f; }

typedef struct { vec3 origin, dir; } Ray;
typedef struct { vec3 pos; float radius; int materialID, lightID; } sphere_t;
typedef struct { vec3 pos; int materialID, lightID; } plane_t;
typedef struct { vec3 pos, rotation, size; int materialID, lightID; } box_t;
typedef struct { vec3 pos; float radius, sliceSize; int is1stSlice; vec3 rotation; int materialID, lightID; } slice_t;
typedef struct { vec3 pos, rotation; float radius, focalLength, thickness; int isConverging; int materialID, lightID; } lens_t;
typedef struct { vec3 pos, rotation, scale; float a, b, c, d, brad; int materialID, lightID; } cyclide_t;
typedef struct { vec3 reflection; } material_t;
typedef struct { float x, y; } light_t;

/* SC:129-140 */
static vec3 WaveToXYZ(const ctx_t* c, float wave) {
    vec3 XYZ = mk3(0.0f, 0.0f, 0.0f);
    if ((wave >= 360.0f) && (wave <= 800.0f)) {
        int index3 = 3 * (int)(floorf(wave) - 360.0f);
        vec3 t1 = mk3(CIE(c, index3), CIE(c, index3 + 1), CIE(c, index3 + 2));
        vec3 t2 = mk3(CIE(c, index3 + 3), CIE(c, index3 + 4), CIE(c, index3 + 5));
        float a = wave - floorf(wave);
        XYZ = mk3(mixf(t1.x, t2.x, a), mixf(t1.y, t2.y, a), mixf(t1.z, t2.z, a));
    }
    return XYZ;
}

/* Extension PT_EXT_ANALYTIC_CMF: the multi-lobe Gaussian fit of the CIE 1931
 * matching functions (Wyman, Sloan and Shirley 2013) evaluated at the
 * wavelength; each lobe has a different width on each side of its peak. */
static inline float cmf_lobe(float x, float mu, float s1, float s2) {
    float t = (x - mu) / ((x < mu) ? s1 : s2);
    return ptm_expf(-0.5f * t * t);
}
static vec3 cmf_analytic(float wave) {
    float x = (1.056f * cmf_lobe(wave, 599.8f, 37.9f, 31.0f) + 0.362f * cmf_lobe(wave, 442.0f, 16.0f, 26.7f)) -
              0.065f * cmf_lobe(wave, 501.1f, 20.4f, 26.2f);
    float y = 0.821f * cmf_lobe(wave, 568.8f, 46.9f, 40.5f) + 0.286f * cmf_lobe(wave, 530.9f, 16.3f, 31.1f);
    float z = 1.217f * cmf_lobe(wave, 437.0f, 11.8f, 36.0f) + 0.681f * cmf_lobe(wave, 459.0f, 26.0f, 13.8f);
    return mk3(x, y, z);
}
static vec3 WaveToXYZx(const ctx_t* c, float wave) {
    return (c->x->flags & PT_EXT_ANALYTIC_CMF) ? cmf_analytic(wave) : WaveToXYZ(c, wave);
}

/* SC:143-152 */
static mat3 RotationMatrix(vec3 angle) {
    angle = scl3(angle, 0.0174532925199f);
    vec3 s = mk3(ptm_sinf(angle.x), ptm_sinf(angle.y), ptm_sinf(angle.z));
    vec3 co = mk3(ptm_cosf(angle.x), ptm_cosf(angle.y), ptm_cosf(angle.z));
    mat3 mX = {{1.0f, 0.0f, 0.0f}, {0.0f, co.x, -s.x}, {0.0f, s.x, co.x}};
    mat3 mY = {{co.y, 0.0f, s.y}, {0.0f, 1.0f, 0.0f}, {-s.y, 0.0f, co.y}};
    mat3 mZ = {{co.z, -s.z, 0.0f}, {s.z, co.z, 0.0f}, {0.0f, 0.0f, 1.0f}};
    return mat_mul_mat(mat_mul_mat(mX, mY), mZ);
}

/* SC:154-235 */
static sphere_t UnpackSphere(const ctx_t* c, int index) {
    sphere_t o;
    index *= 6;
    o.pos = mk3(OBJ(c, index), OBJ(c, index + 1), OBJ(c, index + 2));
    o.radius = OBJ(c, index + 3);
    o.materialID = (int)OBJ(c, index + 4) - 1;
    o.lightID = (int)OBJ(c, index + 5) - 1;
    return o;
}
static plane_t UnpackPlane(const ctx_t* c, int index, int offset) {
    plane_t o;
    index *= 5;
    o.pos = mk3(OBJ(c, index + offset), OBJ(c, index + 1 + offset), OBJ(c, index + 2 + offset));
    o.materialID = (int)OBJ(c, index + 3 + offset) - 1;
    o.lightID = (int)OBJ(c, index + 4 + offset) - 1;
    return o;
}
static box_t UnpackBox(const ctx_t* c, int index, int offset) {
    box_t o;
    index *= 11;
    o.pos = mk3(OBJ(c, index + offset), OBJ(c, index + 1 + offset), OBJ(c, index + 2 + offset));
    o.rotation = mk3(OBJ(c, index + 3 + offset), OBJ(c, index + 4 + offset), OBJ(c, index + 5 + offset));
    o.size = mk3(OBJ(c, index + 6 + offset), OBJ(c, index + 7 + offset), OBJ(c, index + 8 + offset));
    o.materialID = (int)OBJ(c, index + 9 + offset) - 1;
    o.lightID = (int)OBJ(c, index + 10 + offset) - 1;
    return o;
}
static lens_t UnpackLens(const ctx_t* c, int index, int offset) {
    lens_t o;
    index *= 12;
    o.pos = mk3(OBJ(c, index + offset), OBJ(c, index + 1 + offset), OBJ(c, index + 2 + offset));
    o.rotation = mk3(OBJ(c, index + 3 + offset), OBJ(c, index + 4 + offset), OBJ(c, index + 5 + offset));
    o.radius = OBJ(c, index + 6 + offset);
    o.focalLength = OBJ(c, index + 7 + offset);
    o.thickness = OBJ(c, index + 8 + offset);
    o.isConverging = OBJ(c, index + 9 + offset) != 0.0f;
    o.materialID = (int)OBJ(c, index + 10 + offset) - 1;
    o.lightID = (int)OBJ(c, index + 11 + offset) - 1;
    return o;
}
static cyclide_t UnpackCyclide(const ctx_t* c, int index, int offset) {
    cyclide_t o;
    index *= 16;
    o.pos = mk3(OBJ(c, index + offset), OBJ(c, index + offset + 1), OBJ(c, index + offset + 2));
    o.rotation = mk3(OBJ(c, index + 3 + offset), OBJ(c, index + 4 + offset), OBJ(c, index + 5 + offset));
    o.scale = mk3(OBJ(c, index + 6 + offset), OBJ(c, index + 7 + offset), OBJ(c, index + 8 + offset));
    o.a = OBJ(c, index + 9 + offset);
    o.b = OBJ(c, index + 10 + offset);
    o.c = OBJ(c, index + 11 + offset);
    o.d = OBJ(c, index + 12 + offset);
    o.brad = OBJ(c, index + 13 + offset);
    o.materialID = (int)OBJ(c, index + 14 + offset) - 1;
    o.lightID = (int)OBJ(c, index + 15 + offset) - 1;
    return o;
}
static material_t UnpackMaterial(const ctx_t* c, int index) {
    material_t m;
    index *= 3;
    m.reflection = mk3(MATS(c, index), MATS(c, index + 1), MATS(c, index + 2));
    return m;
}
static light_t UnpackLight(const ctx_t* c, int index) {
    light_t l;
    if (index == -1) {
        l.x = 5500.0f;
        l.y = 0.0f;
        return l;
    }
    index *= 2;
    l.x = LIGHTS(c, index);
    l.y = LIGHTS(c, index + 1);
    return l;
}
/* SC:237-254 */
static material_t GetMaterialMix(const ctx_t* c, float materialID) {
    material_t m1 = UnpackMaterial(c, (int)floorf(materialID));
    material_t m2 = UnpackMaterial(c, (int)ceilf(materialID));
    float x = materialID - floorf(materialID);
    material_t m;
    m.reflection = mk3(mixf(m1.reflection.x, m2.reflection.x, x), mixf(m1.reflection.y, m2.reflection.y, x),
                       mixf(m1.reflection.z, m2.reflection.z, x));
    return m;
}
static light_t GetLightMix(const ctx_t* c, float lightID) { return UnpackLight(c, (int)lightID); }

/* SC:263-276 */
static int BoundingSphere(Ray ray, vec3 pos, float radius2) {
    vec3 lo = sub3(ray.origin, pos);
    float b = dot3(ray.dir, lo);
    float cc = dot3(lo, lo) - radius2;
    if ((b * b) < cc) return 0;
    if ((b >= 0.0f) && (cc >= 0.0f)) return 0;
    return 1;
}

/* SC:278-287 (SortMinMax SC:256-261) */
static vec2 RayIntersectAABB(vec3 origin, vec3 invdir, vec3 pos, vec3 size) {
    vec3 lo = sub3(origin, pos);
    vec3 tMin = mul3(fma3(size, mk3(-0.5f, -0.5f, -0.5f), neg3(lo)), invdir);
    vec3 tMax = mul3(fma3(size, mk3(0.5f, 0.5f, 0.5f), neg3(lo)), invdir);
    vec3 a = min3(tMin, tMax), b = max3(tMin, tMax);
    float t1 = fmaxf(fmaxf(a.x, a.y), a.z);
    float t2 = fminf(fminf(b.x, b.y), b.z);
    return mk2(t1, t2);
}

typedef struct {
    float hitdist;
    vec3 normal;
    float materialID;
    float lightID;
} hit_t;

/* SC:289-317 */
static int SphereIntersection(Ray ray, sphere_t o, hit_t* h) {
    vec3 lo = sub3(ray.origin, o.pos);
    float b = 2.0f * dot3(ray.dir, lo);
    float cc = dot3(lo, lo) - (o.radius * o.radius);
    float disc = b * b - 4.0f * cc;
    if (disc < 0.0f) return 0;
    float sqrtD = sqrtf(disc);
    float t1 = (-b - sqrtD) * 0.5f;
    float t2 = (-b + sqrtD) * 0.5f;
    float t = (t1 > 0.0f) ? t1 : t2;
    int isOutside = (t1 > 0.0f) ? 1 : -1;
    if (t < 1e-4f) return 0;
    if (t < h->hitdist) {
        h->hitdist = t;
        h->normal = normalize3(scl3(fma3(ray.dir, mk3(t, t, t), lo), (float)isOutside));
        h->materialID = (float)o.materialID;
        h->lightID = (float)o.lightID;
        return 1;
    }
    return 0;
}

/* SC:319-335 */
static int PlaneIntersection(Ray ray, plane_t o, hit_t* h) {
    vec3 lo = sub3(ray.origin, o.pos);
    float t = -lo.y / ray.dir.y;
    if (t < 1e-4f) return 0;
    if (t < h->hitdist) {
        h->hitdist = t;
        /* faceforward(N, I, Nref) = dot(Nref, I) < 0 ? N : -N with N = Nref = (0,1,0) */
        float d = 0.0f * ray.dir.x + 1.0f * ray.dir.y + 0.0f * ray.dir.z;
        h->normal = (d < 0.0f) ? mk3(0.0f, 1.0f, 0.0f) : mk3(-0.0f, -1.0f, -0.0f);
        h->materialID = (float)o.materialID;
        h->lightID = (float)o.lightID;
        return 1;
    }
    return 0;
}

/* SC:337-364 */
static int BoxIntersection(Ray ray, box_t o, hit_t* h) {
    mat3 m = RotationMatrix(o.rotation);
    vec3 lo = vec_mul_mat(sub3(ray.origin, o.pos), m);
    vec3 dir = vec_mul_mat(ray.dir, m);
    vec3 invdir = mk3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    vec3 tMin = mul3(fma3(o.size, mk3(-0.5f, -0.5f, -0.5f), neg3(lo)), invdir);
    vec3 tMax = mul3(fma3(o.size, mk3(0.5f, 0.5f, 0.5f), neg3(lo)), invdir);
    vec3 a = min3(tMin, tMax), b = max3(tMin, tMax);
    float t1 = fmaxf(fmaxf(a.x, a.y), a.z);
    float t2 = fminf(fminf(b.x, b.y), b.z);
    float t = (t1 < 0.0f) ? t2 : t1;
    if ((t1 > t2) || (t < 1e-4f)) return 0;
    if (t < h->hitdist) {
        h->hitdist = t;
        vec3 p = abs3(div3(add3(lo, scl3(dir, t)), o.size));
        float mx = fmaxf(fmaxf(p.x, p.y), p.z);
        vec3 st = mk3(stepf_glsl(mx, p.x), stepf_glsl(mx, p.y), stepf_glsl(mx, p.z));
        vec3 sg = mk3(-signf_glsl(dir.x), -signf_glsl(dir.y), -signf_glsl(dir.z));
        h->normal = mat_mul_vec(m, mul3(st, sg));
        h->materialID = (float)o.materialID;
        h->lightID = (float)o.lightID;
        return 1;
    }
    return 0;
}

/* SC:366-417 */
static int SphereSliceIntersection(Ray ray, slice_t o, float localSlicePos, int isSideInvert, hit_t* h, int* isOutside) {
    mat3 m = RotationMatrix(o.rotation);
    float sliceOffset = o.radius - o.sliceSize;
    vec3 org = vec_mul_mat(sub3(ray.origin, o.pos), m);
    if (o.is1stSlice) {
        org.x += localSlicePos - o.sliceSize - sliceOffset;
    } else {
        org.x -= localSlicePos - o.sliceSize - sliceOffset;
    }
    vec3 dir = vec_mul_mat(ray.dir, m);
    float b = 2.0f * dot3(dir, org);
    float cc = dot3(org, org) - (o.radius * o.radius);
    float disc = b * b - 4.0f * cc;
    float t = 1e6f;
    int isOut = 1;
    if (disc < 0.0f) return 0;
    float sqrtD = sqrtf(disc);
    float t1 = (-b - sqrtD) * 0.5f;
    float t2 = (-b + sqrtD) * 0.5f;
    if (o.is1stSlice) {
        t1 = (fmaf(dir.x, t1, org.x) > -sliceOffset) ? 1e6f : t1;
        t2 = (fmaf(dir.x, t2, org.x) > -sliceOffset) ? 1e6f : t2;
    } else {
        t1 = (fmaf(dir.x, t1, org.x) < sliceOffset) ? 1e6f : t1;
        t2 = (fmaf(dir.x, t2, org.x) < sliceOffset) ? 1e6f : t2;
    }
    t = (t1 > 0.0f) ? t1 : t;
    if (t2 < t) {
        t = t2;
        isOut = -1;
    }
    if (t < 1e-4f) return 0;
    if (t < h->hitdist) {
        h->hitdist = t;
        h->normal = mat_mul_vec(m, normalize3(scl3(fma3(dir, mk3(t, t, t), org), (float)isOut)));
        *isOutside = (!isSideInvert) ? isOut : -isOut;
        h->materialID = (float)o.materialID;
        h->lightID = (float)o.lightID;
        return 1;
    }
    return 0;
}

/* SC:419-448 */
static int LensIntersection(Ray ray, lens_t o, hit_t* h, int* isOutside) {
    float lensThicknessHalf = 2.0f * o.focalLength - sqrtf(4.0f * o.focalLength * o.focalLength - o.radius * o.radius);
    float lensSlicePos = 0.5f * (o.isConverging ? o.thickness : -o.thickness);
    if (o.isConverging) lensSlicePos += lensThicknessHalf;
    int isIntersect = 0;
    for (int i = 0; i < 2; i++) {
        slice_t s;
        s.pos = o.pos;
        s.radius = 2.0f * o.focalLength;
        s.sliceSize = lensThicknessHalf;
        s.is1stSlice = (i == 0);
        s.rotation = o.rotation;
        s.materialID = o.materialID;
        s.lightID = o.lightID;
        if (SphereSliceIntersection(ray, s, lensSlicePos, !o.isConverging, h, isOutside)) isIntersect = 1;
    }
    return isIntersect;
}

/* SC:450-472 */
static inline float EvalQuadratic(float a, float b, float c, float x) { return x * (x * a + b) + c; }
static inline float EvalCubic(float a, float b, float c, float d, float x) { return x * (x * (x * a + b) + c) + d; }
static inline float EvalQuartic(float a, float b, float c, float d, float e, float x) {
    return x * (x * (x * (x * a + b) + c) + d) + e;
}

/* SC:474-503; returns the number of leading real roots flagged (1 or 3). */
static int SolveCubic(float b, float c, float d, vec3* roots) {
    float bdiv3 = b * ONEBYTHREE;
    float Q = c * ONEBYTHREE - bdiv3 * bdiv3;
    float R = 0.5f * bdiv3 * c - bdiv3 * bdiv3 * bdiv3 - 0.5f * d;
    float D = Q * Q * Q + R * R;
    if (D > 0.0f) {
        float u = R + sqrtf(D);
        float v = R - sqrtf(D);
        float S = signf_glsl(u) * ptm_powf(fabsf(u), ONEBYTHREE);
        float T = signf_glsl(v) * ptm_powf(fabsf(v), ONEBYTHREE);
        roots->x = S + T - bdiv3;
        for (int i = 0; i < 2; i++) {
            roots->x -= EvalCubic(1.0f, b, c, d, roots->x) / EvalQuadratic(3.0f, 2.0f * b, c, roots->x);
        }
        return 1;
    }
    float sqrtnegQ = sqrtf(-Q);
    float thetadiv3 = ptm_acosf(R / (sqrtnegQ * sqrtnegQ * sqrtnegQ)) * ONEBYTHREE;
    float TWOPIBYTHREE = fmaf(2.0f, PI_F, ONEBYTHREE);
    float k = 2.0f * sqrtnegQ;
    roots->x = k * ptm_cosf(thetadiv3) - bdiv3;
    roots->y = k * ptm_cosf(thetadiv3 + TWOPIBYTHREE) - bdiv3;
    roots->z = k * ptm_cosf(fmaf(2.0f, TWOPIBYTHREE, thetadiv3)) - bdiv3;
    for (int i = 0; i < 2; i++) {
        roots->x -= EvalCubic(1.0f, b, c, d, roots->x) / EvalQuadratic(3.0f, 2.0f * b, c, roots->x);
        roots->y -= EvalCubic(1.0f, b, c, d, roots->y) / EvalQuadratic(3.0f, 2.0f * b, c, roots->y);
        roots->z -= EvalCubic(1.0f, b, c, d, roots->z) / EvalQuadratic(3.0f, 2.0f * b, c, roots->z);
    }
    return 3;
}

/* SC:505-541; real[i] flags which of roots[0..3] are set. */
static void SolveQuartic(float a, float b, float c, float d, float e, float roots[4], int real[4]) {
    float inva = 1.0f / a;
    float inva2 = inva * 0.5f;
    float inva2a2 = inva2 * inva2;
    float bb = b * b;
    float p = -1.5f * bb * inva2a2 + c * inva;
    float q = bb * b * inva2a2 * inva2 - b * c * inva * inva2 + d * inva;
    float r = -0.1875f * bb * bb * inva2a2 * inva2a2 + 0.5f * c * bb * inva2a2 * inva2 - b * d * inva2a2 + e * inva;
    vec3 s = mk3(0.0f, 0.0f, 0.0f);
    SolveCubic(0.5f * -p, -r, 0.5f * p * r - 0.125f * q * q, &s);
    real[0] = real[1] = real[2] = real[3] = 0;
    float s2subp = 2.0f * s.x - p;
    if (s2subp < 0.0f) return;
    float invs2subp = -2.0f * s.x - p;
    float sqrts2subp = sqrtf(s2subp);
    float q2divsqrt = 2.0f * q / sqrts2subp;
    float invaddq2div = invs2subp + q2divsqrt;
    float invsubq2div = invs2subp - q2divsqrt;
    float bdiv4a = 0.25f * inva * b;
    if (invaddq2div >= 0.0f) {
        float sq = sqrtf(invaddq2div);
        roots[0] = 0.5f * (-sqrts2subp + 1.0f * sq) - bdiv4a;
        roots[1] = 0.5f * (-sqrts2subp + -1.0f * sq) - bdiv4a;
        for (int i = 0; i < 2; i++) {
            roots[i] -= EvalQuartic(a, b, c, d, e, roots[i]) / EvalCubic(4.0f * a, 3.0f * b, 2.0f * c, d, roots[i]);
        }
        real[0] = real[1] = 1;
    }
    if (invsubq2div >= 0.0f) {
        float sq = sqrtf(invsubq2div);
        roots[2] = 0.5f * (sqrts2subp + 1.0f * sq) - bdiv4a;
        roots[3] = 0.5f * (sqrts2subp + -1.0f * sq) - bdiv4a;
        for (int i = 2; i < 4; i++) {
            roots[i] -= EvalQuartic(a, b, c, d, e, roots[i]) / EvalCubic(4.0f * a, 3.0f * b, 2.0f * c, d, roots[i]);
        }
        real[2] = real[3] = 1;
    }
}

/* Swizzles used by the cyclide. */
static inline vec3 xzy(vec3 v) { return mk3(v.x, v.z, v.y); }
static inline vec3 yzx(vec3 v) { return mk3(v.y, v.z, v.x); }
static inline vec3 zxy(vec3 v) { return mk3(v.z, v.x, v.y); }

/* SC:633-679 */
static int DupinCyclide(Ray ray, cyclide_t ob, hit_t* h) {
    mat3 m = RotationMatrix(ob.rotation);
    vec3 o = xzy(div3(vec_mul_mat(sub3(ray.origin, ob.pos), m), ob.scale));
    vec3 d = xzy(div3(vec_mul_mat(ray.dir, m), ob.scale));
    float A = ob.a, B = ob.b, C = ob.c, Dd = ob.d;
    vec3 dd = mul3(d, d), oo = mul3(o, o), od = mul3(o, d);
    vec3 dyzx = yzx(d), dzxy = zxy(d), oyzx = yzx(o), ozxy = zxy(o);
    float a4 = dot3(dd, dd) + 2.0f * dot3(dd, mul3(dyzx, dyzx));
    float a3 = 4.0f * (dot3(o, mul3(dd, d)) + dot3(od, mul3(dyzx, dyzx)) + dot3(od, mul3(dzxy, dzxy)));
    float a2 = 6.0f * dot3(oo, dd) + 8.0f * dot3(od, mul3(oyzx, dyzx)) +
               2.0f * (dot3(oo, mul3(dyzx, dyzx)) + dot3(oo, mul3(dzxy, dzxy))) +
               2.0f * (B * B - Dd * Dd) * dot3(d, d) - 4.0f * (A * A * d.x * d.x + B * B * d.y * d.y);
    float a1 = 4.0f * (dot3(mul3(oo, o), d) + dot3(oo, mul3(oyzx, dyzx)) + dot3(oo, mul3(ozxy, dzxy)) +
                       2.0f * A * C * Dd * d.x + (B * B - Dd * Dd) * dot3(o, d) -
                       2.0f * (A * A * o.x * d.x + B * B * o.y * d.y));
    float a0 = dot3(oo, oo) + 2.0f * dot3(oo, mul3(oyzx, oyzx)) + B * B * B * B + Dd * Dd * Dd * Dd -
               2.0f * B * B * Dd * Dd - 4.0f * C * C * Dd * Dd + 8.0f * A * C * Dd * o.x +
               2.0f * (B * B - Dd * Dd) * dot3(o, o) - 4.0f * (A * A * o.x * o.x + B * B * o.y * o.y);
    float roots[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    int real[4];
    SolveQuartic(a4, a3, a2, a1, a0, roots, real);
    float t = 1e6f;
    for (int i = 0; i < 4; i++) {
        if (real[i]) {
            if ((roots[i] < t) && (roots[i] > 0.0f)) t = roots[i];
        }
    }
    if (t < h->hitdist) {
        h->hitdist = t;
        float x = o.x + d.x * t;
        float y = o.y + d.y * t;
        float z = o.z + d.z * t;
        float term1 = x * x + y * y + z * z + B * B - Dd * Dd;
        vec3 n;
        n.x = 4.0f * (x * term1 - 2.0f * A * (A * x - C * Dd));
        n.y = 4.0f * z * term1;
        n.z = 4.0f * y * (term1 - 2.0f * B * B);
        h->normal = normalize3(n);
        h->materialID = (float)ob.materialID;
        h->lightID = (float)ob.lightID;
        return 1;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* SDF plug-ins (sdfs/<name>.glsl) and the spliced SDF()/SDFMATERIAL()  */
/* ------------------------------------------------------------------ */
/* SC:686-702 */
static inline float smin1(float x, float y) {
    float k = 0.02f;
    k *= 6.0f;
    float h = fmaxf(k - fabsf(x - y), 0.0f) / k;
    float m = h * h * h * 0.5f;
    float s = m * k * ONEBYTHREE;
    return fminf(x, y) - s;
}
static inline vec2 smin2(vec2 x, vec2 y) {
    float k = 0.02f;
    k *= 6.0f;
    float h = fmaxf(k - fabsf(x.x - y.x), 0.0f) / k;
    float m = h * h * h * 0.5f;
    float s = m * k * ONEBYTHREE;
    return (x.x < y.x) ? mk2(x.x - s, x.y + (y.y - x.y) * m) : mk2(y.x - s, x.y + (y.y - x.y) * (1.0f - m));
}

/* sdfs/blob.glsl:1-8 */
static float blob_sdf(vec3 p) {
    float s1 = length3(p) - 1.0f;
    float s2 = length3(mk3(p.x, p.y - 1.0f, p.z)) - 0.7f;
    float s3 = length3(mk3(p.x - 0.25f, p.y - 1.25f, p.z - 0.5f)) - 0.25f;
    float s4 = length3(mk3(p.x + 0.25f, p.y - 1.25f, p.z - 0.5f)) - 0.25f;
    return smin1(smin1(smin1(s1, s2), s3), s4);
}
/* sdfs/blob.glsl:10-17 (lobe material IDs parameterised) */
static float blob_material(vec3 p, const float* m) {
    vec2 s1 = mk2(length3(p) - 1.0f, m[0]);
    vec2 s2 = mk2(length3(mk3(p.x, p.y - 1.0f, p.z)) - 0.7f, m[1]);
    vec2 s3 = mk2(length3(mk3(p.x - 0.25f, p.y - 1.25f, p.z - 0.5f)) - 0.25f, m[2]);
    vec2 s4 = mk2(length3(mk3(p.x + 0.25f, p.y - 1.25f, p.z - 0.5f)) - 0.25f, m[2]);
    return smin2(smin2(smin2(s1, s2), s3), s4).y;
}

static _Thread_local uint64_t* tl_cnt; /* work counters of the calling thread (for the plug-ins) */

/* sdfs/mandelbulb.glsl:3-52 */
static float mandelbulb_sdf(vec3 p) {
    vec3 z = p;
    float r = length3(z);
    float dr = 1.0f;
    for (int i = 0; i < 4; i++) {
        if (tl_cnt) tl_cnt[PTO_C_MANDELBULB_ITERS]++;
        dr = 8.0f * ptm_powf(r, 7.0f) * dr + 1.0f;
        float invr = 1.0f / r;
        float invl = 1.0f / sqrtf(z.x * z.x + z.z * z.z);
        r *= r;
        r *= r;
        r *= r;
        float cost = z.z * invl;
        float cosp = z.y * invr;
        float sint = z.x * invl;
        float sinp = invr / invl;
        float cost2 = cost * cost;
        float cosp2 = cosp * cosp;
        float cost8 = fmaf(fmaf(fmaf(fmaf(128.0f, cost2, -256.0f), cost2, 160.0f), cost2, -32.0f), cost2, 1.0f);
        float cosp8 = fmaf(fmaf(fmaf(fmaf(128.0f, cosp2, -256.0f), cosp2, 160.0f), cosp2, -32.0f), cosp2, 1.0f);
        float sint8 = fmaf(fmaf(fmaf(128.0f, cost2, -192.0f), cost2, 80.0f), cost2, -8.0f) * sint * cost;
        float sinp8 = fmaf(fmaf(fmaf(128.0f, cosp2, -192.0f), cosp2, 80.0f), cosp2, -8.0f) * sinp * cosp;
        z = scl3(mk3(sint8 * sinp8, cosp8, cost8 * sinp8), r);
        z = add3(z, p);
        r = length3(z);
        if (r > 16.0f) break;
    }
    return 0.5f * ptm_logf(r) * r / dr;
}
/* sdfs/mandelbulb.glsl:54-58 (mix endpoints parameterised) */
static float mandelbulb_material(vec3 p, const float* m) {
    float factor = dot3(p, p);
    return mixf(m[0], m[1], factor / (0.8f + factor));
}

/* sdfs/menger.glsl:2-23 */
static float menger_sdf(vec3 p) {
    vec3 q = sub3(abs3(p), mk3(1.0f, 1.0f, 1.0f));
    float d = length3(max3(q, mk3(0.0f, 0.0f, 0.0f))) + fminf(fmaxf(q.x, fmaxf(q.y, q.z)), 0.0f);
    float s = 1.0f;
    for (int m = 0; m < 5; m++) {
        vec3 ps = scl3(p, s);
        vec3 a = mk3(modf_glsl(ps.x, 2.0f) - 1.0f, modf_glsl(ps.y, 2.0f) - 1.0f, modf_glsl(ps.z, 2.0f) - 1.0f);
        s *= 3.0f;
        vec3 r = mk3(fabsf(1.0f - 3.0f * fabsf(a.x)), fabsf(1.0f - 3.0f * fabsf(a.y)), fabsf(1.0f - 3.0f * fabsf(a.z)));
        float da = fmaxf(r.x, r.y);
        float db = fmaxf(r.y, r.z);
        float dc = fmaxf(r.z, r.x);
        float c = (fminf(da, fminf(db, dc)) - 1.0f) / s;
        d = fmaxf(d, c);
    }
    return d;
}

/* sdfs/terrain.glsl:1-8 */
static float terrain_height(float x) {
    return ptm_sinf(0.0625f * x) + ptm_sinf(0.125f * (x + 10.0f)) + 0.25f * ptm_sinf(0.25f * x) + 0.125f * ptm_sinf(0.5f * x) +
           0.25f * ptm_sinf(x) + 0.25f * ptm_sinf(2.0f * x + 1.0f) + 0.125f * ptm_sinf(4.0f * x + 2.0f) +
           0.0625f * ptm_sinf(8.0f * x + 1.0f) + 0.03125f * ptm_sinf(16.0f * x + 5.0f) + 0.015625f * ptm_sinf(32.0f * x) +
           0.0078125f * ptm_sinf(64.0f * x);
}
static float terrain_sdf(vec3 p) { return p.y - (terrain_height(p.x) + terrain_height(p.z)); }

/* SDF slots holding other GLSL text (PT_SDF_CUSTOM): the tests register a C
 * restatement of each such snippet (oracle/user_sdfs.c) per slot. */
typedef float (*pto_user_fn)(float x, float y, float z);
static pto_user_fn g_user_sdf[PT_MAX_LIVE_SDFS];
static pto_user_fn g_user_mat[PT_MAX_LIVE_SDFS];

int pto_set_user_sdf(int slot, pto_user_fn sdf, pto_user_fn material) {
    if (slot < 0 || slot >= PT_MAX_LIVE_SDFS) return 1;
    g_user_sdf[slot] = sdf;
    g_user_mat[slot] = material;
    return 0;
}

static float plugin_sdf(const pt_sdf_plugin* pl, int slot, vec3 p) {
    switch (pl->kind) {
        case PT_SDF_BLOB: return blob_sdf(p);
        case PT_SDF_MANDELBULB: return mandelbulb_sdf(p);
        case PT_SDF_MENGER: return menger_sdf(p);
        case PT_SDF_TERRAIN: return terrain_sdf(p);
        case PT_SDF_CUSTOM:
            return (slot >= 0 && slot < PT_MAX_LIVE_SDFS && g_user_sdf[slot]) ? g_user_sdf[slot](p.x, p.y, p.z) : MAXDIST;
        default: return MAXDIST;
    }
}
static float plugin_material(const pt_sdf_plugin* pl, int slot, vec3 p) {
    if (pl->material_mode == PT_SDFMAT_CONSTANT) return pl->material[0];
    switch (pl->kind) {
        case PT_SDF_BLOB: return blob_material(p, pl->material);
        case PT_SDF_MANDELBULB: return mandelbulb_material(p, pl->material);
        case PT_SDF_CUSTOM:
            return (slot >= 0 && slot < PT_MAX_LIVE_SDFS && g_user_mat[slot]) ? g_user_mat[slot](p.x, p.y, p.z)
                                                                                : pl->material[0];
        default: return pl->material[0];
    }
}

/* The work counter of one plug-in evaluation, by kind. */
static int sdf_counter(int kind) {
    switch (kind) {
        case PT_SDF_BLOB: return PTO_C_SDF_BLOB;
        case PT_SDF_MANDELBULB: return PTO_C_SDF_MANDELBULB;
        case PT_SDF_MENGER: return PTO_C_SDF_MENGER;
        case PT_SDF_TERRAIN: return PTO_C_SDF_TERRAIN;
        default: return PTO_C_SDF_CUSTOM;
    }
}

static inline vec3 sdf_pos(const ctx_t* c, int i) { return mk3(SDFS(c, 6 * i), SDFS(c, 6 * i + 1), SDFS(c, 6 * i + 2)); }

/* SC:706-711 with the code InsertSDF splices in (src/pathtracer.cpp:2004-2054):
 * for each SDF i in scene order, if bit i of set1 is set: sdf = min(sdf, SDFi(p - pos_i)). */
static float SDF(const ctx_t* c, vec3 p, uint32_t set1) {
    float sdf = MAXDIST;
    int n = c->nplug < PT_MAX_LIVE_SDFS ? c->nplug : PT_MAX_LIVE_SDFS;
    for (int i = 0; i < n; i++) {
        uint32_t code = 1u << i;
        if ((set1 & code) == code && c->plug[i].kind != PT_SDF_NONE) {
            COUNT(c, sdf_counter(c->plug[i].kind));
            sdf = fminf(sdf, plugin_sdf(&c->plug[i], i, sub3(p, sdf_pos(c, i))));
        }
    }
    return sdf;
}
/* SC:713-719 with the spliced lines: material = minMaterial(sdf, SDFi, material, SDFiMATERIAL);
 * sdf = min(sdf, SDFi) — minMaterial(x,y,m1,m2) = x < y ? m1 : m2 (SC:681-683). */
static float SDFMATERIAL(const ctx_t* c, vec3 p, uint32_t set1) {
    float sdf = MAXDIST;
    float mat = 0.0f;
    int n = c->nplug < PT_MAX_LIVE_SDFS ? c->nplug : PT_MAX_LIVE_SDFS;
    for (int i = 0; i < n; i++) {
        uint32_t code = 1u << i;
        if ((set1 & code) == code && c->plug[i].kind != PT_SDF_NONE) {
            vec3 q = sub3(p, sdf_pos(c, i));
            COUNT(c, sdf_counter(c->plug[i].kind));
            float di = plugin_sdf(&c->plug[i], i, q);
            if (!(sdf < di)) COUNT(c, PTO_C_SDF_MATERIAL);
            mat = (sdf < di) ? mat : plugin_material(&c->plug[i], i, q);
            sdf = fminf(sdf, di);
        }
    }
    return mat;
}

/* SC:721-730 */
static vec3 CalculateNumericalSDFNormals(const ctx_t* c, vec3 p, uint32_t set1) {
    float e = 1e-4f;
    vec3 n = mk3(SDF(c, mk3(p.x + e, p.y + 0.0f, p.z + 0.0f), set1) - SDF(c, mk3(p.x - e, p.y - 0.0f, p.z - 0.0f), set1),
                 SDF(c, mk3(p.x + 0.0f, p.y + e, p.z + 0.0f), set1) - SDF(c, mk3(p.x - 0.0f, p.y - e, p.z - 0.0f), set1),
                 SDF(c, mk3(p.x + 0.0f, p.y + 0.0f, p.z + e), set1) - SDF(c, mk3(p.x - 0.0f, p.y - 0.0f, p.z - e), set1));
    return normalize3(n);
}

/* SC:732-777 */
static int SearchSDF(const ctx_t* c, vec3 p, vec3 invdir, vec2* tMinMax, uint32_t* set1) {
    int found = 0;
    *set1 = 0;
    for (int i = 0; (float)i < c->u->numObjects[5]; i++) {
        vec3 pos = sdf_pos(c, i);
        vec3 size = mk3(SDFS(c, 6 * i + 3), SDFS(c, 6 * i + 4), SDFS(c, 6 * i + 5));
        COUNT(c, PTO_C_AABB);
        vec2 bm = RayIntersectAABB(p, invdir, pos, size);
        uint32_t bit = (i < 32) ? (1u << i) : 0u;
        if ((bm.x > bm.y) || (bm.y < 0.0f)) continue;
        if (bm.x < tMinMax->x) {
            found = 1;
            if (bm.y < tMinMax->x) {
                *tMinMax = bm;
                *set1 = bit;
            } else {
                if (bm.y < tMinMax->y) {
                    tMinMax->x = bm.x;
                    *set1 += bit;
                } else {
                    *tMinMax = bm;
                    *set1 += bit;
                }
            }
        } else {
            if (bm.x < tMinMax->y) {
                found = 1;
                if (bm.y > tMinMax->y) {
                    tMinMax->y = bm.y;
                    *set1 += bit;
                } else {
                    *set1 += bit;
                }
            }
        }
    }
    return found;
}

/* SC:779-860 */
static int SphereTracing(const ctx_t* c, Ray ray, hit_t* h) {
    float t = 1e-3f;
    float insT = 0.0f;
    const float omegaMax = 1.70f;
    const float omegaSpeed = 0.20f;
    float omega = omegaMax;
    float omegaSpeedFactor = 0.0f;
    float previousRadius = 0.0f;
    vec3 p = ray.origin;
    vec3 invdir = mk3(1.0f / ray.dir.x, 1.0f / ray.dir.y, 1.0f / ray.dir.z);
    int points = 0;
    vec2 tMinMax = mk2(MAXDIST, MAXDIST);
    uint32_t set1 = 0;
    if (SearchSDF(c, p, invdir, &tMinMax, &set1)) {
        t = fmaxf(tMinMax.x, t);
        p = fma3(ray.dir, mk3(t, t, t), ray.origin);
    } else {
        return 0;
    }
    float k = signf_glsl(SDF(c, ray.origin, set1));
    /* Extension PT_EXT_MARCH: the scene's step count, hit epsilon and
     * distance cap instead of 512 steps, 1e-4 and none. */
    const int xm = (c->x->flags & PT_EXT_MARCH) != 0;
    const int maxSteps = xm ? c->x->march_max_steps : 512;
    const float eps = xm ? c->x->march_epsilon : 1e-4f;
    for (int i = 0; i < maxSteps; i++) {
        if (xm && t > c->x->march_max_distance) return 0;
        COUNT(c, PTO_C_MARCH_STEPS);
        float radius = SDF(c, p, set1);
        if (insT > (fabsf(previousRadius) + fabsf(radius))) {
            t -= insT;
            omega = 1.0f;
            insT = previousRadius * omega * k;
            t += insT;
            p = fma3(ray.dir, mk3(t, t, t), ray.origin);
            continue;
        }
        if (fabsf(radius) < eps) break;
        if (t > tMinMax.y) {
            points += 1;
        } else {
            points = 0;
        }
        if (points >= 2) {
            t = tMinMax.y + 1e-3f;
            tMinMax = mk2(MAXDIST, MAXDIST);
            if (SearchSDF(c, fma3(ray.dir, mk3(t, t, t), ray.origin), invdir, &tMinMax, &set1)) {
                tMinMax.x += t;
                tMinMax.y += t;
                t = fmaxf(tMinMax.x, t);
                p = fma3(ray.dir, mk3(t, t, t), ray.origin);
                continue;
            } else {
                return 0;
            }
        }
        insT = radius * omega * k;
        t += insT;
        p = fma3(ray.dir, mk3(t, t, t), ray.origin);
        omegaSpeedFactor = fminf(radius / previousRadius, 0.99f);
        omega += omegaSpeed * (fminf(1.0f / (1.0f - omegaSpeedFactor), omegaMax) - omega);
        previousRadius = radius;
    }
    if (t < h->hitdist) {
        h->hitdist = t - 1e-3f;
        p = fma3(ray.dir, mk3(t, t, t), ray.origin);
        h->normal = CalculateNumericalSDFNormals(c, p, set1);
        h->materialID = SDFMATERIAL(c, p, set1);
        h->lightID = -1.0f;
        return 1;
    }
    return 0;
}

/* SC:543-588: the quartic surface x^2(x^2 + 2y^2 - 6y + 2z^2) +
 * y^2(y^2 + 2y + 2z^2) + z^2(10z^2 - 12) + 1 = 0 at the origin, in the
 * ray's xzy frame.  The reference defines it but its call sites are
 * commented out (SC:926-931, :1207-1216), so no scene reaches it. */
static int Thritorius(Ray ray, hit_t* h) {
    if (!BoundingSphere(ray, mk3(0.0f, 0.0f, 0.0f), 4.05f)) return 0;
    vec3 o = xzy(ray.origin);
    vec3 d = xzy(ray.dir);
    vec3 ddd = mul3(mul3(d, d), d);
    vec3 d10 = mk3(d.x, d.y, 10.0f * d.z);
    vec3 o10 = mk3(o.x, o.y, 10.0f * o.z);
    float a4 = dot3(d10, ddd) + 2.0f * dot3(mul3(d, d), mul3(yzx(d), yzx(d)));
    vec3 dd2 = mk3(d.y * d.y + d.z * d.z, d.x * d.x + d.z * d.z, d.x * d.x + d.y * d.y);
    float a3 = 4.0f * (dot3(o10, ddd) + dot3(mul3(o, d), dd2)) + 2.0f * d.y * d.y * d.y - 6.0f * d.x * d.x * d.y;
    vec3 oxxy = mk3(o.x, o.x, o.y), dxxy = mk3(d.x, d.x, d.y), oyzz = mk3(o.y, o.z, o.z), dyzz = mk3(d.y, d.z, d.z);
    float a2 = 6.0f * dot3(o10, mul3(mul3(o, d), d)) +
               2.0f * ((o.x * o.x * (d.y * d.y) + o.y * o.y * (d.x * d.x)) +
                       (o.x * o.x * (d.z * d.z) + o.z * o.z * (d.x * d.x)) +
                       (o.y * o.y * (d.z * d.z) + o.z * o.z * (d.y * d.y))) +
               8.0f * dot3(mul3(oxxy, dxxy), mul3(oyzz, dyzz)) + 6.0f * o.y * d.y * d.y - 6.0f * o.y * d.x * d.x -
               12.0f * o.x * d.x * d.y - 12.0f * d.z * d.z;
    float a1 = 4.0f * (dot3(mul3(mul3(o10, o), o), d) + (o.x * o.x * (o.y * d.y) + o.x * o.x * (o.z * d.z)) +
                       (o.y * o.y * (o.x * d.x) + o.y * o.y * (o.z * d.z)) +
                       (o.z * o.z * (o.x * d.x) + o.z * o.z * (o.y * d.y))) +
               6.0f * o.y * o.y * d.y - 6.0f * o.x * o.x * d.y - 12.0f * o.x * o.y * d.x - 24.0f * o.z * d.z;
    float a0 = dot3(o10, mul3(mul3(o, o), o)) + 2.0f * dot3(mul3(oxxy, oxxy), mul3(oyzz, oyzz)) +
               2.0f * o.y * o.y * o.y - 6.0f * o.x * o.x * o.y - 12.0f * o.z * o.z + 1.0f;
    float roots[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    int real[4];
    SolveQuartic(a4, a3, a2, a1, a0, roots, real);
    float t = 1e6f;
    for (int i = 0; i < 4; i++) {
        if (real[i]) {
            if ((roots[i] < t) && (roots[i] > 0.0f)) t = roots[i];
        }
    }
    if (t < h->hitdist) {
        h->hitdist = t;
        float x = o.x + d.x * t;
        float y = o.y + d.y * t;
        float z = o.z + d.z * t;
        vec3 n;
        n.x = 4.0f * x * x * x + 4.0f * x * y * y - 12.0f * x * y + 4.0f * x * z * z;
        n.y = 40.0f * z * z * z + 4.0f * x * x * z + 4.0f * y * y * z - 24.0f * z;
        n.z = 4.0f * y * y * y + 4.0f * x * x * y - 6.0f * x * x + 6.0f * y * y + 4.0f * y * z * z;
        if ((o.x * o.x * (o.x * o.x + 2.0f * o.y * o.y - 6.0f * o.y + 2.0f * o.z * o.z) +
             o.y * o.y * (o.y * o.y + 2.0f * o.y + 2.0f * o.z * o.z) + o.z * o.z * (10.0f * o.z * o.z - 12.0f) +
             1.0f) < 0.0f)
            n = scl3(n, -1.0f);
        h->normal = normalize3(n);
        h->materialID = 1.0f;
        h->lightID = -1.0f;
        return 1;
    }
    return 0;
}

/* SC:590-631: the superquadric x^4 + y^4 + z^4 = 1 at the origin (disabled
 * in the reference like Thritorius). */
static int SmoothCuboid(Ray ray, hit_t* h) {
    if (!BoundingSphere(ray, mk3(0.0f, 0.0f, 0.0f), 1.80f)) return 0;
    vec3 o = ray.origin;
    vec3 d = ray.dir;
    float a4 = dot3(mul3(d, d), mul3(d, d));
    float a3 = 4.0f * dot3(o, mul3(mul3(d, d), d));
    float a2 = 6.0f * dot3(mul3(o, o), mul3(d, d));
    float a1 = 4.0f * dot3(mul3(mul3(o, o), o), d);
    float a0 = dot3(mul3(o, o), mul3(o, o)) - 1.0f;
    float roots[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    int real[4];
    SolveQuartic(a4, a3, a2, a1, a0, roots, real);
    float t = 1e6f;
    for (int i = 0; i < 4; i++) {
        if (real[i]) {
            if ((roots[i] < t) && (roots[i] > 0.0f)) t = roots[i];
        }
    }
    if (t < h->hitdist) {
        h->hitdist = t;
        vec3 n = fma3(d, mk3(t, t, t), o);
        n = mul3(mul3(n, n), n);
        if (dot3(mul3(o, o), mul3(o, o)) < 1.0f) n = scl3(n, -1.0f);
        h->normal = normalize3(n);
        h->materialID = 3.0f;
        h->lightID = -1.0f;
        return 1;
    }
    return 0;
}

static inline int NUM(const ctx_t* c, int k) { return (int)c->u->numObjects[k]; }

static float lens_bounding_radius(lens_t o) {
    float br;
    if (o.isConverging) {
        br = (o.radius * o.radius) + (0.25f * o.thickness * o.thickness);
    } else {
        br = 0.5f * o.thickness + 2.0f * o.focalLength - sqrtf(4.0f * o.focalLength * o.focalLength - o.radius * o.radius);
        br = br * br + o.radius * o.radius;
    }
    return br;
}

/* SC:862-934 (Intersection) and SC:1121-1223 (LightSourceVisibilityCheck) share
 * this loop; *objectID receives the index of the last object whose test hit
 * (-1 for an SDF hit or no hit), as LightSourceVisibilityCheck computes it. */
static void IntersectAll(const ctx_t* c, Ray ray, hit_t* h, int* objectID) {
    int offset = 0, objectOffset = 0;
    int id = -1;
    for (int i = 0; (float)i < c->u->numObjects[0]; i++) {
        sphere_t o = UnpackSphere(c, i);
        COUNT(c, PTO_C_SPHERE);
        if (SphereIntersection(ray, o, h)) id = i;
    }
    offset += 6 * NUM(c, 0);
    objectOffset += NUM(c, 0);
    for (int i = 0; (float)i < c->u->numObjects[1]; i++) {
        plane_t o = UnpackPlane(c, i, offset);
        COUNT(c, PTO_C_PLANE);
        if (PlaneIntersection(ray, o, h)) id = i + objectOffset;
    }
    offset += 5 * NUM(c, 1);
    objectOffset += NUM(c, 1);
    for (int i = 0; (float)i < c->u->numObjects[2]; i++) {
        box_t o = UnpackBox(c, i, offset);
        COUNT(c, PTO_C_BOUNDING_SPHERE);
        if (!BoundingSphere(ray, o.pos, 0.25f * dot3(o.size, o.size))) continue;
        COUNT(c, PTO_C_BOX);
        if (BoxIntersection(ray, o, h)) id = i + objectOffset;
    }
    offset += 11 * NUM(c, 2);
    objectOffset += NUM(c, 2);
    for (int i = 0; (float)i < c->u->numObjects[3]; i++) {
        lens_t o = UnpackLens(c, i, offset);
        int isOutside = 1;
        COUNT(c, PTO_C_BOUNDING_SPHERE);
        if (!BoundingSphere(ray, o.pos, lens_bounding_radius(o))) continue;
        if (c->cnt) c->cnt[PTO_C_LENS_SLICE] += 2;
        if (LensIntersection(ray, o, h, &isOutside)) id = i + objectOffset;
    }
    offset += 12 * NUM(c, 3);
    objectOffset += NUM(c, 3);
    for (int i = 0; (float)i < c->u->numObjects[4]; i++) {
        cyclide_t o = UnpackCyclide(c, i, offset);
        COUNT(c, PTO_C_BOUNDING_SPHERE);
        if (!BoundingSphere(ray, o.pos, o.brad)) continue;
        COUNT(c, PTO_C_CYCLIDE);
        if (DupinCyclide(ray, o, h)) id = i + objectOffset;
    }
    if (SphereTracing(c, ray, h)) id = -2; /* SDF */
    *objectID = id;
}

/* SC:937-958 */
uint32_t pto_pcg32(uint32_t seed) {
    uint32_t state = seed * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
static inline float RandomFloatPCG32(uint32_t* seed) {
    *seed = pto_pcg32(*seed);
    return (float)(*seed) / 4294967296.0f; /* float(seed) / float(0xFFFFFFFFu) */
}
float pto_random_float(uint32_t* seed) { return RandomFloatPCG32(seed); }

/* SC:976-1028 */
static vec2 SampleUniformUnitDisk(uint32_t* seed) {
    float rx = RandomFloatPCG32(seed);
    float ry = RandomFloatPCG32(seed);
    float phi = 2.0f * PI_F * ry;
    float d = sqrtf(rx);
    return mk2(d * ptm_cosf(phi), d * ptm_sinf(phi));
}
static vec3 SampleUniformUnitSphere(uint32_t* seed) {
    float rx = RandomFloatPCG32(seed);
    float ry = RandomFloatPCG32(seed);
    float phi = 2.0f * PI_F * ry;
    float sinTheta = 2.0f * rx - 1.0f;
    float cosTheta = sqrtf(fmaf(-sinTheta, sinTheta, 1.0f));
    return mk3(ptm_cosf(phi) * cosTheta, ptm_sinf(phi) * cosTheta, sinTheta);
}
/* SC:999-1003 */
static vec3 SampleCosineDirectionHemisphere(vec3 normal, uint32_t* seed) {
    return normalize3(add3(normal, SampleUniformUnitSphere(seed)));
}
/* SC:1005-1010 */
static inline float CosineDirectionPDF(float cosTheta) { return cosTheta / PI_F; }
/* SC:1025-1028 */
static inline float CosineUnitConePDF(float cosTheta, float cosThetaMax) {
    return cosTheta / (PI_F * (1.0f - cosThetaMax * cosThetaMax));
}
/* SC:960-963 */
static inline float SampleHeroWavelength(float l_min, float l_max, uint32_t* seed) {
    return mixf(l_min, l_max, RandomFloatPCG32(seed));
}
static vec3 SampleCosineUnitCone(uint32_t* seed, float cosThetaMax) {
    float rx = RandomFloatPCG32(seed);
    float ry = RandomFloatPCG32(seed);
    float cosAlphaMax = 2.0f * cosThetaMax * cosThetaMax - 1.0f;
    float phi = 2.0f * PI_F * ry;
    float cosTheta = (1.0f - cosAlphaMax) * rx + cosAlphaMax;
    float sinTheta = sqrtf(fmaf(-cosTheta, cosTheta, 1.0f));
    return normalize3(mk3(ptm_cosf(phi) * sinTheta, ptm_sinf(phi) * sinTheta, cosTheta + 1.0f));
}

/* SC:971-974: l_h - 390 + 0.25 * (1, 2, 3, 4) * 330 = offsets 82.5, 165, 247.5, 330 (exact) */
static vec4 SampleWavelengths(float l_h) {
    float base = l_h - 390.0f;
    return mk4(390.0f + modf_glsl(base + 82.5f, 330.0f), 390.0f + modf_glsl(base + 165.0f, 330.0f),
               390.0f + modf_glsl(base + 247.5f, 330.0f), 390.0f + modf_glsl(base + 330.0f, 330.0f));
}

/* SC:1030-1055 */
static vec4 SpectralPowerDistribution(vec4 l, float l_peak, float d, int invert) {
    float den = 2.0f * d * d;
    vec4 x = mk4((l.x - l_peak) / den, (l.y - l_peak) / den, (l.z - l_peak) / den, (l.w - l_peak) / den);
    vec4 r = mk4(ptm_expf(-x.x * x.x), ptm_expf(-x.y * x.y), ptm_expf(-x.z * x.z), ptm_expf(-x.w * x.w));
    float a = (float)invert;
    return mk4(mixf(r.x, 1.0f - r.x, a), mixf(r.y, 1.0f - r.y, a), mixf(r.z, 1.0f - r.z, a), mixf(r.w, 1.0f - r.w, a));
}
static inline float bb1(float l, float T) {
    return (1.1910429724e-16f * ptm_powf(l, -5.0f)) / (ptm_expf(0.014387768775f / (l * T)) - 1.0f);
}
static inline float BlackBodyRadiationPeak(float T) { return 4.0956746759e-6f * ptm_powf(T, 5.0f); }
static vec4 Emit(vec4 l, light_t lt) {
    float temperature = fmaxf(lt.x, 0.0f);
    vec4 lm = scl4(l, 1e-9f);
    float peak = BlackBodyRadiationPeak(temperature);
    vec4 e = mk4(bb1(lm.x, temperature) / peak, bb1(lm.y, temperature) / peak, bb1(lm.z, temperature) / peak,
                 bb1(lm.w, temperature) / peak);
    return scl4(e, fmaxf(lt.y, 0.0f));
}
void pto_blackbody(const float* l_m, float T, float* out4) {
    for (int i = 0; i < 4; i++) out4[i] = bb1(l_m[i], T);
}
float pto_blackbody_peak(float T) { return BlackBodyRadiationPeak(T); }

/* SC:1064-1073 */
static float RefractiveIndexBK7Glass(float l) {
    l *= 1e-3f;
    float l2 = l * l;
    float n2 = 1.0f;
    n2 += (1.03961212f * l2) / (l2 - 6.00069867e-3f);
    n2 += (0.231792344f * l2) / (l2 - 2.00179144e-2f);
    n2 += (1.01046945f * l2) / (l2 - 1.03560653e2f);
    return sqrtf(n2);
}
float pto_bk7_index(float l) { return RefractiveIndexBK7Glass(l); }

/* SC:1075-1080 */
static vec4 EvaluateBRDF(vec4 l, material_t mat) {
    vec4 s = SpectralPowerDistribution(l, mat.reflection.x, mat.reflection.y, (int)mat.reflection.z);
    return div4s(s, PI_F);
}

/* EvaluateBRDF, or the extension Lambertian of the hit's material. */
static vec4 ExtLambert(const pt_material_ext* m, vec4 l);
static vec4 EvaluateBRDFx(const ctx_t* c, vec4 l, material_t mat, const pt_material_ext* xm) {
    (void)c;
    return xm ? ExtLambert(xm, l) : EvaluateBRDF(l, mat);
}

/* SC:1093-1119 */
static vec3 ToWorld(vec3 v, vec3 n) {
    vec3 b1 = mk3(0.0f, -1.0f, 0.0f);
    vec3 b2 = mk3(-1.0f, 0.0f, 0.0f);
    if (n.z >= -0.9999999f) {
        float a = 1.0f / (1.0f + n.z);
        float b = -n.x * n.y * a;
        b1 = mk3(1.0f - (n.x * n.x * a), b, -n.x);
        b2 = mk3(b, 1.0f - (n.y * n.y * a), -n.y);
    }
    return add3(add3(scl3(b1, v.x), scl3(b2, v.y)), scl3(n, v.z));
}

/* SC:1225-1285 */
static int SampleRandomLightSource(ctx_t* c, uint32_t* seed, float* boundingRadius, vec3* pos, float* lightID) {
    int randomLight = (int)floorf(RandomFloatPCG32(seed) * c->u->numObjects[6]);
    c->light_pick = randomLight;
    int randomLightID = (int)LIGHTIDS(c, randomLight);
    int offset = 0;
    if (randomLightID < NUM(c, 0)) {
        sphere_t o = UnpackSphere(c, randomLightID);
        *boundingRadius = o.radius;
        *pos = o.pos;
        *lightID = (float)o.lightID;
        return (int)LIGHTIDS(c, randomLight);
    }
    randomLightID -= NUM(c, 0);
    offset += 6 * NUM(c, 0);
    if (randomLightID < NUM(c, 1)) {
        plane_t o = UnpackPlane(c, randomLightID, offset);
        *boundingRadius = 1e5f;
        *pos = o.pos;
        *lightID = (float)o.lightID;
        return (int)LIGHTIDS(c, randomLight);
    }
    randomLightID -= NUM(c, 1);
    offset += 5 * NUM(c, 1);
    if (randomLightID < NUM(c, 2)) {
        box_t o = UnpackBox(c, randomLightID, offset);
        *boundingRadius = 0.5f * length3(o.size);
        *pos = o.pos;
        *lightID = (float)o.lightID;
        return (int)LIGHTIDS(c, randomLight);
    }
    randomLightID -= NUM(c, 2);
    offset += 11 * NUM(c, 2);
    if (randomLightID < NUM(c, 2)) { /* SC:1264 compares with numObjects[2] */
        lens_t o = UnpackLens(c, randomLightID, offset);
        *boundingRadius = sqrtf((o.radius * o.radius) + (0.25f * o.thickness * o.thickness));
        *pos = o.pos;
        *lightID = (float)o.lightID;
        return (int)LIGHTIDS(c, randomLight);
    }
    randomLightID -= NUM(c, 3);
    offset += 12 * NUM(c, 3);
    if (randomLightID < NUM(c, 3)) { /* SC:1275 compares with numObjects[3] */
        cyclide_t o = UnpackCyclide(c, randomLightID, offset);
        *boundingRadius = sqrtf(o.brad);
        *pos = o.pos;
        *lightID = (float)o.lightID;
        return (int)LIGHTIDS(c, randomLight);
    }
    return 0;
}

/* SC:1121-1223 */
static int LightSourceVisibilityCheck(const ctx_t* c, Ray ray, int lightObjectID) {
    COUNT(c, PTO_C_SHADOW_RAYS);
    hit_t h;
    h.hitdist = MAXDIST;
    h.normal = mk3(0.0f, 0.0f, 0.0f);
    h.materialID = 0.0f;
    h.lightID = -1.0f;
    int objectID = -1;
    IntersectAll(c, ray, &h, &objectID);
    if (objectID == -2) objectID = -1;
    return objectID == lightObjectID;
}

static inline float MISPowerHeuristicsBeta2(float pdf1, float pdf2) { return pdf1 * pdf1 / (pdf1 * pdf1 + pdf2 * pdf2); }

/* SC:1298-1343 */
static vec4 SampleLightSource(ctx_t* c, vec4 l, vec4 rayradiance, vec3 outOrigin, vec3 normal, material_t mat,
                              const pt_material_ext* xm, uint32_t* seed, float BRDFpdf, float* MISBRDFWeight) {
    float boundingRadius = 0.0f;
    vec3 lightPos = mk3(0.0f, 0.0f, 0.0f);
    float lightIDOut = -1.0f;
    int lightObjectID = 0;
    float lightpdf = 0.0f;
    c->shadow_state = 0;
    c->light_pick = 0;
    if (c->u->numObjects[6] > 0.0f) {
        lightObjectID = SampleRandomLightSource(c, seed, &boundingRadius, &lightPos, &lightIDOut);
        vec3 toL = sub3(lightPos, outOrigin);
        float invLightDistance = 1.0f / length3(toL);
        vec3 lightDir = scl3(sub3(lightPos, outOrigin), invLightDistance);
        float sinthetaMax = fminf(boundingRadius * invLightDistance, 1.0f);
        float costhetaMax = sqrtf(1.0f - sinthetaMax * sinthetaMax);
        Ray outRay;
        outRay.origin = outOrigin;
        outRay.dir = ToWorld(SampleCosineUnitCone(seed, costhetaMax), lightDir);
        lightpdf = 1.0f / c->u->numObjects[6];
        lightpdf *= CosineUnitConePDF(dot3(outRay.dir, lightDir), costhetaMax);
        *MISBRDFWeight = MISPowerHeuristicsBeta2(BRDFpdf, lightpdf);
        float costheta = dot3(outRay.dir, normal);
        float deathProbability = 1.25f * fmaxf(*MISBRDFWeight - 0.2f, 0.0f);
        if (costheta >= 0.0f) {
            if (RandomFloatPCG32(seed) > deathProbability) {
                int vis = LightSourceVisibilityCheck(c, outRay, lightObjectID);
                c->shadow_state = vis ? 3 : 2;
                if (vis) {
                    COUNT(c, PTO_C_EMIT);
                    COUNT(c, PTO_C_BRDF);
                    light_t lt = GetLightMix(c, lightIDOut);
                    vec4 brdf = EvaluateBRDFx(c, l, mat, xm);
                    vec4 f = div4s(scl4(brdf, costheta), lightpdf);
                    rayradiance = mul4(rayradiance, f);
                    return scl4(mul4(Emit(l, lt), rayradiance), 1.0f - *MISBRDFWeight);
                }
            } else {
                *MISBRDFWeight = 1.0f;
                c->shadow_state = 1;
            }
        }
        return s4(0.0f);
    }
    *MISBRDFWeight = MISPowerHeuristicsBeta2(BRDFpdf, lightpdf);
    return s4(0.0f);
}

/* ---- Extension surface models (PT_EXT_MATERIALS) ---- */
static const pt_material_ext* ExtMaterial(const ctx_t* c, float materialID) {
    if (!(c->x->flags & PT_EXT_MATERIALS)) return NULL;
    int mi = (int)floorf(materialID);
    if (mi < 0 || mi >= c->x->nmat || mi >= PT_MAX_EXT_MATERIALS) return NULL;
    const pt_material_ext* m = &c->x->mat[mi];
    return (m->type == PT_BSDF_REFERENCE) ? NULL : m;
}
/* Cauchy n = A + B / l^2, or Sellmeier n^2 = 1 + sum B l^2 / (l^2 - C), l in um. */
static float ExtIOR(const pt_material_ext* m, float l) {
    float u = l * 1e-3f;
    float u2 = u * u;
    if (m->type == PT_BSDF_CAUCHY) return m->p[0] + m->p[1] / u2;
    float n2 = 1.0f;
    n2 += (m->p[0] * u2) / (u2 - m->p[3]);
    n2 += (m->p[1] * u2) / (u2 - m->p[4]);
    n2 += (m->p[2] * u2) / (u2 - m->p[5]);
    return sqrtf(n2);
}
/* Unpolarised Fresnel reflectance for eta = n1/n2 at incidence cosine cosi;
 * 1 under total internal reflection; *cost: the transmitted cosine. */
static float FresnelDielectric(float eta, float cosi, float* cost) {
    float sin2t = (eta * eta) * (1.0f - cosi * cosi);
    if (sin2t >= 1.0f) {
        *cost = 0.0f;
        return 1.0f;
    }
    float ct = sqrtf(1.0f - sin2t);
    float rs = (eta * cosi - ct) / (eta * cosi + ct);
    float rp = (cosi - eta * ct) / (cosi + eta * ct);
    *cost = ct;
    return 0.5f * (rs * rs + rp * rp);
}
/* Lambertian extension reflectance at four wavelengths, / PI. */
static vec4 ExtLambert(const pt_material_ext* m, vec4 l) {
    if (m->type == PT_BSDF_FLAT) return div4s(s4(m->p[0]), PI_F);
    vec4 x = mk4((l.x - m->p[2]) / m->p[3], (l.y - m->p[2]) / m->p[3], (l.z - m->p[2]) / m->p[3],
                 (l.w - m->p[2]) / m->p[3]);
    vec4 v = mk4(m->p[0] + m->p[1] * ptm_expf(-(x.x * x.x)), m->p[0] + m->p[1] * ptm_expf(-(x.y * x.y)),
                 m->p[0] + m->p[1] * ptm_expf(-(x.z * x.z)), m->p[0] + m->p[1] * ptm_expf(-(x.w * x.w)));
    return div4s(v, PI_F);
}
/* A specular bounce (mirror, dielectric): new direction from the hit point,
 * throughput, MIS weight 1 for the next emitter hit.  A dielectric chooses
 * reflection or transmission by the Fresnel reflectance at l.x; reflection
 * keeps every wavelength weighted by its reflectance over the chosen one;
 * from the first transmission on the path carries l.x alone at 4x (each
 * wavelength bends differently).  The new ray starts 2e-4 along its
 * direction (from the surface point itself the sphere test's near root can
 * round to a tiny positive distance below the 1e-4 threshold and the ray
 * would miss the sphere's far side).
 * Russian roulette follows in the caller.  Returns the event bits. */
static uint32_t ExtSpecular(ctx_t* c, const pt_material_ext* m, vec4 l, vec4* rayradiance, Ray* ray, float hitdist,
                            vec3 normal, uint32_t* seed, float* MISBRDFWeight) {
    ray->origin = fma3(ray->dir, mk3(hitdist, hitdist, hitdist), ray->origin);
    vec3 n = normal;
    float cdot = dot3(ray->dir, n);
    if (cdot > 0.0f) {
        n = neg3(n);
        cdot = -cdot;
    }
    *MISBRDFWeight = 1.0f;
    float cosi = -cdot;
    if (m->type == PT_BSDF_MIRROR) {
        ray->dir = add3(ray->dir, scl3(n, 2.0f * cosi));
        ray->origin = fma3(ray->dir, mk3(2e-4f, 2e-4f, 2e-4f), ray->origin);
        *rayradiance = scl4(*rayradiance, m->p[0]);
        return PT_EV_SPECULAR;
    }
    int inside = (c->medium & 1) != 0;
    float nh = ExtIOR(m, l.x);
    float eta = inside ? nh : 1.0f / nh;
    float cost = 0.0f;
    float F = FresnelDielectric(eta, cosi, &cost);
    if (RandomFloatPCG32(seed) < F) {
        ray->dir = add3(ray->dir, scl3(n, 2.0f * cosi));
        float ct;
        float ny = ExtIOR(m, l.y), nz = ExtIOR(m, l.z), nw = ExtIOR(m, l.w);
        float Fy = FresnelDielectric(inside ? ny : 1.0f / ny, cosi, &ct);
        float Fz = FresnelDielectric(inside ? nz : 1.0f / nz, cosi, &ct);
        float Fw = FresnelDielectric(inside ? nw : 1.0f / nw, cosi, &ct);
        vec4 r = *rayradiance;
        *rayradiance = mk4(r.x, r.y * (Fy / F), r.z * (Fz / F), r.w * (Fw / F));
        ray->origin = fma3(ray->dir, mk3(2e-4f, 2e-4f, 2e-4f), ray->origin);
        return PT_EV_SPECULAR;
    }
    ray->dir = normalize3(add3(scl3(ray->dir, eta), scl3(n, eta * cosi - cost)));
    if (!(c->medium & 2)) { /* the first transmission: l.x alone from here on */
        *rayradiance = mk4(rayradiance->x * 4.0f, 0.0f, 0.0f, 0.0f);
        c->medium |= 2;
    }
    c->medium ^= 1;
    ray->origin = fma3(ray->dir, mk3(2e-4f, 2e-4f, 2e-4f), ray->origin);
    return PT_EV_REFRACT;
}

/* SC:1345-1391; *event receives the trace word of this bounce. */
static vec4 TraceRay(ctx_t* c, vec4 l, vec4* rayradiance, Ray* inRay, uint32_t* seed, float* MISBRDFWeight,
                     int* isTerminate, uint32_t* event) {
    vec4 radiance = s4(0.0f);
    hit_t h;
    h.hitdist = MAXDIST;
    h.normal = mk3(0.0f, 0.0f, 0.0f);
    h.materialID = 0.0f;
    h.lightID = -1.0f;
    int objectID = -1;
    COUNT(c, PTO_C_PATH_RAYS);
    IntersectAll(c, *inRay, &h, &objectID);
    float hitdist = h.hitdist;
    material_t mat = GetMaterialMix(c, h.materialID);
    light_t lt = GetLightMix(c, h.lightID);
    uint32_t ev = PT_EV_VALID;
    if (hitdist < MAXDIST) {
        ev |= (objectID == -2) ? PT_EV_HIT_SDF : (uint32_t)(objectID & 0xFFF);
        if (lt.y > 0.0f) {
            COUNT(c, PTO_C_EMIT);
            radiance = scl4(mul4(Emit(l, lt), *rayradiance), *MISBRDFWeight);
            *isTerminate = 1;
            *event = ev | PT_EV_EMITTER;
            return radiance;
        }
        COUNT(c, PTO_C_SURFACE_HITS);
        const pt_material_ext* xm = ExtMaterial(c, h.materialID);
        if (xm && xm->type >= PT_BSDF_MIRROR) {
            ev |= ExtSpecular(c, xm, l, rayradiance, inRay, hitdist, h.normal, seed, MISBRDFWeight);
            vec4 rr = *rayradiance;
            float rp = fminf(fmaxf(fmaxf(rr.x, fmaxf(rr.y, fmaxf(rr.z, rr.w))), 0.0f), 0.99f);
            if (RandomFloatPCG32(seed) > rp) {
                *isTerminate = 1;
                *event = ev | PT_EV_RR_KILL;
                return radiance;
            }
            *rayradiance = scl4(*rayradiance, 1.0f / rp);
            *event = ev;
            return radiance;
        }
        COUNT(c, PTO_C_BRDF);
        Ray outRay;
        outRay.origin = fma3(inRay->dir, mk3(hitdist, hitdist, hitdist), inRay->origin);
        outRay.dir = SampleCosineDirectionHemisphere(h.normal, seed);
        float BRDFpdf = CosineDirectionPDF(dot3(outRay.dir, h.normal));
        radiance = SampleLightSource(c, l, *rayradiance, outRay.origin, h.normal, mat, xm, seed, BRDFpdf,
                                     MISBRDFWeight);
        ev |= ((uint32_t)(c->light_pick & 0x7F) << PT_EV_LIGHT_SHIFT) | ((uint32_t)c->shadow_state << PT_EV_SHADOW_SHIFT);
        float costheta = dot3(outRay.dir, h.normal);
        vec4 brdf = EvaluateBRDFx(c, l, mat, xm);
        vec4 f = div4s(scl4(brdf, costheta), BRDFpdf);
        *rayradiance = mul4(*rayradiance, f);
        vec4 rr = *rayradiance;
        float rp = fminf(fmaxf(fmaxf(rr.x, fmaxf(rr.y, fmaxf(rr.z, rr.w))), 0.0f), 0.99f);
        if (RandomFloatPCG32(seed) > rp) {
            *isTerminate = 1;
            *event = ev | PT_EV_RR_KILL;
            return radiance;
        }
        *rayradiance = scl4(*rayradiance, 1.0f / rp);
        *inRay = outRay;
    } else {
        ev |= PT_EV_HIT_MISS;
        if (c->x->flags & PT_EXT_SKY) { /* extension: the sky, weight 1 (no light sample reaches it) */
            light_t sky;
            sky.x = c->x->sky_temperature;
            sky.y = c->x->sky_luminosity;
            COUNT(c, PTO_C_EMIT);
            radiance = mul4(Emit(l, sky), *rayradiance);
        }
        *isTerminate = 1;
    }
    *event = ev;
    return radiance;
}

/* SC:1393-1407 */
static vec4 TracePath(ctx_t* c, vec4 l, Ray ray, uint32_t* seed, uint32_t* events, int depth_cap, uint32_t* nev) {
    vec4 radiance = s4(0.0f);
    vec4 rayradiance = s4(1.0f);
    float MISBRDFWeight = 1.0f;
    int isTerminate = 0;
    int n = 0;
    c->medium = 0;
    for (int i = 0; i < c->pc->pathLength; i++) {
        uint32_t ev = 0;
        radiance = add4(radiance, TraceRay(c, l, &rayradiance, &ray, seed, &MISBRDFWeight, &isTerminate, &ev));
        if (events && n < depth_cap) events[n] = ev;
        n++;
        if (isTerminate) break;
    }
    if (nev) *nev = (uint32_t)n;
    return radiance;
}

/* SC:1409-1444 */
static void TracePathLens(const ctx_t* c, float l, Ray* ray, vec3 forwardDir) {
    const pt_push* pc = c->pc;
    lens_t o;
    o.radius = pc->lensRadius;
    o.focalLength = pc->lensFocalLength;
    o.thickness = pc->lensThickness;
    o.isConverging = 1;
    o.pos = add3(c->cameraPos, scl3(forwardDir, pc->lensDistance));
    o.rotation = mk3(0.0f, 90.0f - pc->cameraAngle[1], pc->cameraAngle[0]);
    o.materialID = 0;
    o.lightID = 0;
    for (int i = 0; i < 2; i++) {
        hit_t h;
        h.hitdist = 1e6f;
        h.normal = mk3(0.0f, 0.0f, 0.0f);
        h.materialID = 0.0f;
        h.lightID = -1.0f;
        int isOutside = 1;
        LensIntersection(*ray, o, &h, &isOutside);
        float n1, n2;
        if (isOutside == 1) {
            n1 = 1.0f;
            n2 = RefractiveIndexBK7Glass(l);
        } else {
            n1 = RefractiveIndexBK7Glass(l);
            n2 = 1.0f;
        }
        float n12 = n1 / n2;
        l = l * n12;
        ray->origin = fma3(ray->dir, mk3(h.hitdist, h.hitdist, h.hitdist), ray->origin);
        ray->dir = refract3(ray->dir, h.normal, n12);
    }
}

/* SC:1446-1490 */
static vec3 Scene(ctx_t* c, uint32_t xx, uint32_t xy_y, vec2 uv, int k, uint32_t* events, int depth_cap, uint32_t* nev) {
    const pt_push* pc = c->pc;
    COUNT(c, PTO_C_SAMPLES);
    if (c->cnt) c->cnt[PTO_C_LENS_SLICE] += 4; /* the camera lens: 2 intersections x 2 slices */
    uint32_t seed = pto_generate_seed(xx, xy_y, pc->frame, pc->samplesPerFrame, k, pc->resolution[0]);
    float jx = 2.0f * RandomFloatPCG32(&seed) - 0.5f;
    float jy = 2.0f * RandomFloatPCG32(&seed) - 0.5f;
    uv.x += jx / (float)pc->resolution[0];
    uv.y += jy / (float)pc->resolution[1];
    mat3 m = RotationMatrix(mk3(pc->cameraAngle[0], pc->cameraAngle[1], 0.0f));
    float sc = -pc->cameraSize * 0.5f;
    uv.x *= sc;
    uv.y *= sc;
    Ray ray;
    ray.origin = add3(c->cameraPos, vec_mul_mat(mk3(uv.x, uv.y, 0.0f), m));
    vec2 disk = SampleUniformUnitDisk(&seed);
    float ha = 0.5f * pc->apertureSize;
    vec3 pointOnAperture = add3(c->cameraPos, vec_mul_mat(mk3(ha * disk.x, ha * disk.y, pc->apertureDist), m));
    ray.dir = normalize3(sub3(pointOnAperture, ray.origin));
    vec3 forwardDir = mk3(m.c0.z, m.c1.z, m.c2.z);
    const int xr = (c->x->flags & PT_EXT_WAVELENGTHS) != 0;
    float l_h = xr ? SampleHeroWavelength(c->x->lambda_min, c->x->lambda_max, &seed)
                   : SampleHeroWavelength(360.0f, 800.0f, &seed);
    TracePathLens(c, l_h, &ray, forwardDir);
    vec4 l;
    float range;
    if (xr) { /* extension: the hero and three rotations a quarter of the range apart */
        float lo = c->x->lambda_min, R = c->x->lambda_max - c->x->lambda_min;
        float base = l_h - lo, q = R * 0.25f;
        l = mk4(lo + modf_glsl(base + q, R), lo + modf_glsl(base + q * 2.0f, R), lo + modf_glsl(base + q * 3.0f, R),
                lo + modf_glsl(base + R, R));
        range = R;
    } else {
        l = SampleWavelengths(l_h);
        range = 720.0f - 390.0f;
    }
    vec4 radiance = TracePath(c, l, ray, &seed, events, depth_cap, nev);
    vec3 wx = WaveToXYZx(c, l.x), wy = WaveToXYZx(c, l.y), wz = WaveToXYZx(c, l.z), ww = WaveToXYZx(c, l.w);
    vec3 sum = add3(add3(add3(scl3(wx, radiance.x), scl3(wy, radiance.y)), scl3(wz, radiance.z)), scl3(ww, radiance.w));
    vec3 color = scl3(scl3(sum, range), 0.25f);
    if (color.x != color.x) return mk3(0.0f, 0.0f, 0.0f);
    if (color.y != color.y) return mk3(0.0f, 0.0f, 0.0f);
    if (color.z != color.z) return mk3(0.0f, 0.0f, 0.0f);
    return color;
}

uint32_t pto_generate_seed(uint32_t x, uint32_t y, int frame, int spf, int k, int width) {
    uint32_t seed = (uint32_t)(frame - spf + k);
    seed = pto_pcg32(seed);
    seed += x + (uint32_t)width * y;
    return seed;
}

void pto_wave_to_xyz(const float* cie, float wave, float* out3) {
    pt_ubo* u = (pt_ubo*)calloc(1, sizeof(pt_ubo));
    memcpy(u->CIEXYZ1931, cie, sizeof(u->CIEXYZ1931));
    ctx_t c;
    memset(&c, 0, sizeof(c));
    c.u = u;
    c.x = &kNoExt;
    vec3 r = WaveToXYZ(&c, wave);
    out3[0] = r.x;
    out3[1] = r.y;
    out3[2] = r.z;
    free(u);
}

float pto_sdf_eval(const pt_sdf_plugin* pl, const float* p) { return plugin_sdf(pl, 0, mk3(p[0], p[1], p[2])); }
float pto_sdf_material(const pt_sdf_plugin* pl, const float* p) { return plugin_material(pl, 0, mk3(p[0], p[1], p[2])); }

/* SC:1492-1533 */
int pto_dispatch(const pt_ubo* ubo, const pt_push* pc, const pt_sdf_plugin* plugins, int nplugins, float* accum,
                 int x0, int y0, int x1, int y1, const pto_trace* trace, int nthreads) {
    return pto_dispatch_ext(ubo, NULL, pc, plugins, nplugins, accum, x0, y0, x1, y1, trace, nthreads);
}

int pto_dispatch_ext(const pt_ubo* ubo, const pt_scene_ext* ext, const pt_push* pc, const pt_sdf_plugin* plugins,
                     int nplugins, float* accum, int x0, int y0, int x1, int y1, const pto_trace* trace, int nthreads) {
    if (!ext) ext = &kNoExt;
    if (!ubo || !pc || !accum) return PT_ERR_INVALID;
    const int W = pc->resolution[0], H = pc->resolution[1];
    if (W <= 0 || H <= 0 || pc->samplesPerFrame <= 0) return PT_ERR_INVALID;
    if (x0 < 0 || y0 < 0 || x1 > W || y1 > H || x0 > x1 || y0 > y1) return PT_ERR_INVALID;
    if (nplugins < 0 || (nplugins > 0 && !plugins)) return PT_ERR_INVALID;
    const int spf = pc->samplesPerFrame;
    const int rw = x1 - x0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = y0; y < y1; y++) {
        ctx_t c;
        uint64_t cnt[PTO_C_COUNT];
        memset(&c, 0, sizeof(c));
        memset(cnt, 0, sizeof(cnt));
        c.u = ubo;
        c.pc = pc;
        c.plug = plugins;
        c.nplug = nplugins;
        c.cameraPos = mk3(pc->cameraPosX, pc->cameraPosY, pc->cameraPosZ);
        c.x = ext;
        c.cnt = (trace && trace->counters) ? cnt : NULL;
        tl_cnt = c.cnt;
        for (int x = x0; x < x1; x++) {
            size_t coords = (size_t)x + (size_t)W * (size_t)y;
            float* px = accum + 4 * coords;
            vec3 inColor = mk3(px[0], px[1], px[2]);
            /* Rendering SC:1509-1523 */
            uint32_t xx = (uint32_t)x;
            uint32_t yy = (uint32_t)H - (uint32_t)y;
            vec2 uv = mk2((2.0f * (float)xx - (float)W) / (float)H, (2.0f * (float)yy - (float)H) / (float)H);
            vec3 outColor = mk3(0.0f, 0.0f, 0.0f);
            for (int i = 0; i < spf; i++) {
                size_t pidx = ((size_t)(y - y0) * (size_t)rw + (size_t)(x - x0)) * (size_t)spf + (size_t)i;
                uint32_t* ev = NULL;
                uint32_t* nev = NULL;
                int cap = 0;
                if (trace && trace->events) {
                    ev = trace->events + pidx * (size_t)trace->depth_cap;
                    cap = trace->depth_cap;
                }
                if (trace && trace->nevents) nev = trace->nevents + pidx;
                vec3 col = Scene(&c, xx, yy, uv, i, ev, cap, nev);
                if (trace && trace->colors) {
                    trace->colors[pidx * 3 + 0] = col.x;
                    trace->colors[pidx * 3 + 1] = col.y;
                    trace->colors[pidx * 3 + 2] = col.z;
                }
                outColor = add3(outColor, col);
            }
            float fs = (float)spf;
            outColor = mk3(outColor.x / fs, outColor.y / fs, outColor.z / fs);
            outColor = scl3(outColor, pc->apertureSize * pc->apertureSize * (float)pc->ISO);
            /* Accumulate SC:1492-1507 */
            if ((pc->currentSamples == pc->samplesPerFrame) && (pc->frame > pc->samplesPerFrame)) {
                float weight = ptm_powf(2.0f, -8.0f / (pc->FPS * pc->persistence));
                outColor = add3(scl3(outColor, 1.0f - weight), scl3(inColor, weight));
            } else {
                int unitSamples = pc->currentSamples / pc->samplesPerFrame;
                float us = (float)unitSamples;
                vec3 t = add3(scl3(inColor, (float)(unitSamples - 1)), outColor);
                outColor = mk3(t.x / us, t.y / us, t.z / us);
            }
            px[0] = outColor.x;
            px[1] = outColor.y;
            px[2] = outColor.z;
            px[3] = 1.0f;
        }
        if (c.cnt) {
            for (int k = 0; k < PTO_C_COUNT; k++) {
#pragma omp atomic
                trace->counters[k] += cnt[k];
            }
        }
        tl_cnt = NULL;
    }
    return PT_OK;
}

/* Evaluates one pt_mathf function over arrays (for accuracy tests):
 * fn 0 sin, 1 cos, 2 exp, 3 log, 4 pow(x, y), 5 acos. */
int pto_mathf_eval(int fn, const float* x, const float* y, float* out, int n) {
    for (int i = 0; i < n; i++) {
        switch (fn) {
            case 0: out[i] = ptm_sinf(x[i]); break;
            case 1: out[i] = ptm_cosf(x[i]); break;
            case 2: out[i] = ptm_expf(x[i]); break;
            case 3: out[i] = ptm_logf(x[i]); break;
            case 4: out[i] = ptm_powf(x[i], y[i]); break;
            case 5: out[i] = ptm_acosf(x[i]); break;
            case 6: out[i] = ptm_asinf(x[i]); break;
            case 7: out[i] = ptm_atanf(x[i]); break;
            case 8: out[i] = ptm_atan2f(x[i], y[i]); break;
            case 9: out[i] = ptm_exp2f(x[i]); break;
            case 10: out[i] = ptm_log2f(x[i]); break;
            default: return PT_ERR_INVALID;
        }
    }
    return PT_OK;
}

/* Single shader functions for the known-answer tests against the reference's
 * own shader source (tests/test_oracle_reference.py): each runs the same code
 * the dispatch above runs.  Vectors are float arrays, matrices column-major. */
void pto_fn_sample_disk(uint32_t* seed, float* out2) {
    vec2 v = SampleUniformUnitDisk(seed);
    out2[0] = v.x, out2[1] = v.y;
}
void pto_fn_sample_sphere(uint32_t* seed, float* out3) {
    vec3 v = SampleUniformUnitSphere(seed);
    out3[0] = v.x, out3[1] = v.y, out3[2] = v.z;
}
void pto_fn_sample_hemisphere(const float* n3, uint32_t* seed, float* out3) {
    vec3 v = SampleCosineDirectionHemisphere(mk3(n3[0], n3[1], n3[2]), seed);
    out3[0] = v.x, out3[1] = v.y, out3[2] = v.z;
}
void pto_fn_sample_cone(uint32_t* seed, float cosThetaMax, float* out3) {
    vec3 v = SampleCosineUnitCone(seed, cosThetaMax);
    out3[0] = v.x, out3[1] = v.y, out3[2] = v.z;
}
void pto_fn_sample_wavelengths(float l_h, float* out4) {
    vec4 v = SampleWavelengths(l_h);
    out4[0] = v.x, out4[1] = v.y, out4[2] = v.z, out4[3] = v.w;
}
void pto_fn_spd(const float* l4, float peak, float d, int invert, float* out4) {
    vec4 v = SpectralPowerDistribution(mk4(l4[0], l4[1], l4[2], l4[3]), peak, d, invert);
    out4[0] = v.x, out4[1] = v.y, out4[2] = v.z, out4[3] = v.w;
}
void pto_fn_to_world(const float* v3, const float* n3, float* out3) {
    vec3 v = ToWorld(mk3(v3[0], v3[1], v3[2]), mk3(n3[0], n3[1], n3[2]));
    out3[0] = v.x, out3[1] = v.y, out3[2] = v.z;
}
float pto_fn_mis(float pdf1, float pdf2) { return MISPowerHeuristicsBeta2(pdf1, pdf2); }
float pto_fn_cosine_pdf(float cosTheta) { return CosineDirectionPDF(cosTheta); }
float pto_fn_cone_pdf(float cosTheta, float cosThetaMax) { return CosineUnitConePDF(cosTheta, cosThetaMax); }
float pto_fn_hero_wavelength(float l_min, float l_max, uint32_t* seed) {
    return SampleHeroWavelength(l_min, l_max, seed);
}
float pto_fn_smin(float x, float y) { return smin1(x, y); }
void pto_fn_smin2(const float* x2, const float* y2, float* out2) {
    vec2 v = smin2(mk2(x2[0], x2[1]), mk2(y2[0], y2[1]));
    out2[0] = v.x, out2[1] = v.y;
}
int pto_fn_solve_cubic(float b, float c, float d, float* roots3) {
    vec3 r = mk3(roots3[0], roots3[1], roots3[2]);
    int n = SolveCubic(b, c, d, &r);
    roots3[0] = r.x, roots3[1] = r.y, roots3[2] = r.z;
    return n;
}
void pto_fn_solve_quartic(float a, float b, float c, float d, float e, float* roots4, int* real4) {
    SolveQuartic(a, b, c, d, e, roots4, real4);
}
void pto_fn_rotation(const float* angle3, float* out9) {
    mat3 m = RotationMatrix(mk3(angle3[0], angle3[1], angle3[2]));
    const vec3 cols[3] = {m.c0, m.c1, m.c2};
    for (int j = 0; j < 3; j++) out9[3 * j] = cols[j].x, out9[3 * j + 1] = cols[j].y, out9[3 * j + 2] = cols[j].z;
}

/* The analytic intersections (SC:263-448, SC:633-679) for the same tests.
 * ray6 = origin, dir; hit6 = hitdist (in: the closest so far), normal,
 * materialID, lightID (updated on a hit).  Object arrays follow the
 * shader's struct fields in order, ids as floats. */
static Ray ray_of(const float* r) { Ray ray; ray.origin = mk3(r[0], r[1], r[2]); ray.dir = mk3(r[3], r[4], r[5]); return ray; }
static hit_t hit_of(const float* h) {
    hit_t t;
    t.hitdist = h[0], t.normal = mk3(h[1], h[2], h[3]), t.materialID = h[4], t.lightID = h[5];
    return t;
}
static void put_hit(float* h, hit_t t) {
    h[0] = t.hitdist, h[1] = t.normal.x, h[2] = t.normal.y, h[3] = t.normal.z, h[4] = t.materialID, h[5] = t.lightID;
}
int pto_fn_bounding_sphere(const float* ray6, const float* pos3, float radius2) {
    return BoundingSphere(ray_of(ray6), mk3(pos3[0], pos3[1], pos3[2]), radius2);
}
void pto_fn_aabb(const float* origin3, const float* invdir3, const float* pos3, const float* size3, float* out2) {
    vec2 v = RayIntersectAABB(mk3(origin3[0], origin3[1], origin3[2]), mk3(invdir3[0], invdir3[1], invdir3[2]),
                              mk3(pos3[0], pos3[1], pos3[2]), mk3(size3[0], size3[1], size3[2]));
    out2[0] = v.x, out2[1] = v.y;
}
int pto_fn_sphere(const float* ray6, const float* o, float* hit6) {
    sphere_t s = {mk3(o[0], o[1], o[2]), o[3], (int)o[4], (int)o[5]};
    hit_t h = hit_of(hit6);
    int r = SphereIntersection(ray_of(ray6), s, &h);
    put_hit(hit6, h);
    return r;
}
int pto_fn_plane(const float* ray6, const float* o, float* hit6) {
    plane_t p = {mk3(o[0], o[1], o[2]), (int)o[3], (int)o[4]};
    hit_t h = hit_of(hit6);
    int r = PlaneIntersection(ray_of(ray6), p, &h);
    put_hit(hit6, h);
    return r;
}
int pto_fn_box(const float* ray6, const float* o, float* hit6) {
    box_t b = {mk3(o[0], o[1], o[2]), mk3(o[3], o[4], o[5]), mk3(o[6], o[7], o[8]), (int)o[9], (int)o[10]};
    hit_t h = hit_of(hit6);
    int r = BoxIntersection(ray_of(ray6), b, &h);
    put_hit(hit6, h);
    return r;
}
int pto_fn_lens(const float* ray6, const float* o, float* hit6, int* isOutside) {
    lens_t l = {mk3(o[0], o[1], o[2]), mk3(o[3], o[4], o[5]), o[6], o[7], o[8], (int)o[9], (int)o[10], (int)o[11]};
    hit_t h = hit_of(hit6);
    int r = LensIntersection(ray_of(ray6), l, &h, isOutside);
    put_hit(hit6, h);
    return r;
}
int pto_fn_cyclide(const float* ray6, const float* o, float* hit6) {
    cyclide_t c = {mk3(o[0], o[1], o[2]), mk3(o[3], o[4], o[5]), mk3(o[6], o[7], o[8]), o[9], o[10], o[11], o[12],
                   o[13], (int)o[14], (int)o[15]};
    hit_t h = hit_of(hit6);
    int r = DupinCyclide(ray_of(ray6), c, &h);
    put_hit(hit6, h);
    return r;
}

int pto_fn_thritorius(const float* ray6, const float* o, float* hit6) {
    (void)o;
    hit_t h = hit_of(hit6);
    int r = Thritorius(ray_of(ray6), &h);
    put_hit(hit6, h);
    return r;
}
int pto_fn_smooth_cuboid(const float* ray6, const float* o, float* hit6) {
    (void)o;
    hit_t h = hit_of(hit6);
    int r = SmoothCuboid(ray_of(ray6), &h);
    put_hit(hit6, h);
    return r;
}

/* Intersection (SC:862-934) of one ray with a whole packed scene, SDFs
 * included: out6 = hitdist, normal, materialID, lightID as TraceRay sees them
 * (hitdist MAXDIST for no hit). */
void pto_fn_intersection(const pt_ubo* ubo, const pt_push* pc, const pt_sdf_plugin* plugins, int nplugins,
                         const float* ray6, float* out6) {
    ctx_t c;
    memset(&c, 0, sizeof(c));
    c.u = ubo;
    c.pc = pc;
    c.plug = plugins;
    c.nplug = nplugins;
    c.cameraPos = mk3(pc->cameraPosX, pc->cameraPosY, pc->cameraPosZ);
    c.x = &kNoExt;
    hit_t h;
    h.hitdist = MAXDIST;
    h.normal = mk3(0.0f, 0.0f, 0.0f);
    h.materialID = 0.0f;
    h.lightID = -1.0f;
    int objectID = -1;
    IntersectAll(&c, ray_of(ray6), &h, &objectID);
    put_hit(out6, h);
}
