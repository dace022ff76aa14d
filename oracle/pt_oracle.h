/*
 * pt_oracle.h — CPU restatement of the reference's per-pixel spectral
 * path-tracing kernel (src/shader.comp) for checking libpt_cuda.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this
 * library; only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it, as the oracle the GPU results are compared with.
 *
 * Parity status: the reference has no tests, golden vectors or images, and
 * it cannot run on these machines (Vulkan + Windows), so this restatement is
 * "parity unpinned" against the reference itself.  Its primitives are pinned
 * by known-answer values derived from the reference's formulas (PCG32 hash,
 * seeds, BK7 index, blackbody peak); see tests/test_oracle_kat.py.
 */
#ifndef PT_ORACLE_H
#define PT_ORACLE_H

#include <stdint.h>
#include "../include/pt_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pto_trace {
    int depth_cap;      /* event words stored per path */
    uint32_t* events;   /* [npaths * depth_cap] */
    uint32_t* nevents;  /* [npaths] */
    float* colors;      /* [npaths * 3] */
    uint64_t* counters; /* [PTO_C_COUNT] work counters, summed over the dispatch (or NULL) */
} pto_trace;

/* Work counters: how often each unit of the shader's work runs.  Multiplied
 * by the floating-point operations each unit performs, they give the
 * algorithmic FP32 work of a render (the roofline numerator). */
enum {
    PTO_C_SAMPLES = 0,       /* Scene() calls: camera paths */
    PTO_C_PATH_RAYS,         /* TraceRay: Intersection of a path ray */
    PTO_C_SHADOW_RAYS,       /* LightSourceVisibilityCheck */
    PTO_C_SPHERE,            /* SphereIntersection */
    PTO_C_PLANE,             /* PlaneIntersection */
    PTO_C_BOUNDING_SPHERE,   /* BoundingSphere (boxes, lenses, cyclides) */
    PTO_C_BOX,               /* BoxIntersection */
    PTO_C_LENS_SLICE,        /* SphereSliceIntersection (scene lenses and the camera lens) */
    PTO_C_CYCLIDE,           /* DupinCyclide */
    PTO_C_AABB,              /* RayIntersectAABB (SearchSDF) */
    PTO_C_MARCH_STEPS,       /* SphereTracing loop iterations */
    PTO_C_SDF_BLOB,          /* plug-in evaluations by kind */
    PTO_C_SDF_MANDELBULB,
    PTO_C_MANDELBULB_ITERS,  /* iterations inside the mandelbulb loop */
    PTO_C_SDF_MENGER,
    PTO_C_SDF_TERRAIN,
    PTO_C_SDF_MATERIAL,      /* sdfmaterial evaluations */
    PTO_C_EMIT,              /* Emit (4 wavelengths) */
    PTO_C_BRDF,              /* EvaluateBRDF (4 wavelengths) */
    PTO_C_SURFACE_HITS,      /* non-emissive hits: BRDF sampling + light sampling */
    PTO_C_SDF_CUSTOM,        /* evaluations of other GLSL text (PT_SDF_CUSTOM slots) */
    PTO_C_COUNT
};

/*
 * Runs the shader's main() (src/shader.comp:1525-1533) for every invocation
 * (x, y) in [x0, x1) x [y0, y1), reading and writing `accum` (W*H float4,
 * index x + W*y).  Path index for the trace is
 * ((y - y0) * (x1 - x0) + (x - x0)) * samplesPerFrame + k.
 * nthreads <= 0 uses all OpenMP threads.  Returns 0 or an error code.
 */
int pto_dispatch(const pt_ubo* ubo, const pt_push* pc, const pt_sdf_plugin* plugins, int nplugins,
                 float* accum, int x0, int y0, int x1, int y1, const pto_trace* trace, int nthreads);
/* The same with the scene's full-form extensions (ext NULL: the reference's
 * method; include/pt_cuda.h, pt_scene_ext). */
int pto_dispatch_ext(const pt_ubo* ubo, const pt_scene_ext* ext, const pt_push* pc, const pt_sdf_plugin* plugins,
                     int nplugins, float* accum, int x0, int y0, int x1, int y1, const pto_trace* trace, int nthreads);

/* Primitives exposed for known-answer tests. */
uint32_t pto_pcg32(uint32_t seed);
float pto_random_float(uint32_t* seed);
uint32_t pto_generate_seed(uint32_t x, uint32_t y, int frame, int spf, int k, int width);
float pto_bk7_index(float wavelength_nm);
void pto_blackbody(const float* l_m, float T, float* out4);
float pto_blackbody_peak(float T);
float pto_sdf_eval(const pt_sdf_plugin* plugin, const float* p3);
float pto_sdf_material(const pt_sdf_plugin* plugin, const float* p3);
void pto_wave_to_xyz(const float* cie, float wave, float* out3);
int pto_mathf_eval(int fn, const float* x, const float* y, float* out, int n);
/* Single shader functions (SC line ranges at their definitions in pt_oracle.c). */
void pto_fn_sample_disk(uint32_t* seed, float* out2);
void pto_fn_sample_sphere(uint32_t* seed, float* out3);
void pto_fn_sample_hemisphere(const float* n3, uint32_t* seed, float* out3);
void pto_fn_sample_cone(uint32_t* seed, float cosThetaMax, float* out3);
void pto_fn_sample_wavelengths(float l_h, float* out4);
void pto_fn_spd(const float* l4, float peak, float d, int invert, float* out4);
void pto_fn_to_world(const float* v3, const float* n3, float* out3);
float pto_fn_mis(float pdf1, float pdf2);
float pto_fn_cosine_pdf(float cosTheta);
float pto_fn_cone_pdf(float cosTheta, float cosThetaMax);
float pto_fn_hero_wavelength(float l_min, float l_max, uint32_t* seed);
float pto_fn_smin(float x, float y);
void pto_fn_smin2(const float* x2, const float* y2, float* out2);
int pto_fn_solve_cubic(float b, float c, float d, float* roots3);
void pto_fn_solve_quartic(float a, float b, float c, float d, float e, float* roots4, int* real4);
void pto_fn_rotation(const float* angle3, float* out9);
int pto_fn_bounding_sphere(const float* ray6, const float* pos3, float radius2);
void pto_fn_aabb(const float* origin3, const float* invdir3, const float* pos3, const float* size3, float* out2);
int pto_fn_sphere(const float* ray6, const float* sphere6, float* hit6);
int pto_fn_plane(const float* ray6, const float* plane5, float* hit6);
int pto_fn_box(const float* ray6, const float* box11, float* hit6);
int pto_fn_lens(const float* ray6, const float* lens12, float* hit6, int* isOutside);
int pto_fn_cyclide(const float* ray6, const float* cyclide16, float* hit6);
void pto_fn_intersection(const pt_ubo* ubo, const pt_push* pc, const pt_sdf_plugin* plugins, int nplugins,
                         const float* ray6, float* out6);
/* CPU functions of a PT_SDF_CUSTOM slot (the compiled translation of its GLSL). */
int pto_set_user_sdf(int slot, float (*sdf)(float, float, float), float (*material)(float, float, float));

#ifdef __cplusplus
}
#endif

#endif
