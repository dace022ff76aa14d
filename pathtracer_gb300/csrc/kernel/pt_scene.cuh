// pt_scene.cuh — the scene as the megakernel sees it.
//
// Everything the shader reads with warp-uniform indices (object arrays, SDF
// boxes, plug-in table, per-object rotation matrices) travels with each launch
// as a __grid_constant__ kernel parameter, so it sits in that launch's
// constant bank: uniform loads are broadcast, several contexts or scenes can
// be in flight at once, and there is no module-global state to race on.
// The CIE table is read per wavelength (divergent) and stays in global memory.
//
// Rotation matrices of boxes, lenses and cyclides are derived once per scene
// upload by a setup kernel with the same RotationMatrix arithmetic the shader
// evaluates per test (src/shader.comp:143-152), so they are bit-identical to
// recomputing them inline.
#pragma once

#include "../../../include/pt_cuda.h"
#include "pt_vec.cuh"

// Largest object count the 1024-float object array can hold (planes, 5 floats).
#define PT_MAX_SCENE_OBJECTS (PT_MAX_OBJECTS_SIZE / 5)

struct pt_scene_meta {
    int n[7];           // numObjects as integers (validated integral on upload)
    int offset[5];      // float offset of each primitive class in objects[]
    int nplug;          // plug-ins set by pt_set_sdfs (slots beyond evaluate as absent)
    int total_objects;  // n[0] + ... + n[4]
    int custom_base;    // run-time compiled snippets: slot i is snippet custom_base + i of the
                        // compiled program (0 for a context; a batch numbers all its scenes' slots)
};

struct KScene {
    float numObjects[7];
    float objects[PT_MAX_OBJECTS_SIZE];
    float sdfs[PT_MAX_SDFS_SIZE];
    float materials[PT_MAX_MATERIALS_SIZE];
    float lights[PT_MAX_LIGHTS_SIZE];
    float lightIDs[PT_MAX_LIGHTIDS_SIZE];
    pt_scene_meta meta;
    pt_sdf_plugin plug[PT_MAX_LIVE_SDFS];
    float rot[PT_MAX_SCENE_OBJECTS][9];
    pt_scene_ext ext;  // full-form extensions; all zero: the reference's method
};

// Camera quantities that depend only on the push constants (SC:1456,
// SC:1409-1418): derived once per block (megakernel) or per job (wavefront).
template <typename R> struct CamInfoT {
    M3<R> cam;
    M3<R> lensRot;
    V3<R> lensPos;
};
using CamInfo = CamInfoT<float>;

struct KTrace {
    uint32_t* events;
    uint32_t* nevents;
    float* colors;
    int cap;
};

struct KParams {
    KScene s;
    pt_push pc;
    float4* accum;
    const float* cie;  // 1323 floats in global memory
    KTrace trace;
    double* sums;      // the FP64 renderer's target: x, y, z sums of exposed colours and the sample count per pixel
};

// Guarded reads for indices that come from scene data rather than loop
// counters: out-of-range reads give 0, like robust buffer access.
PT_DI float s_obj(const KScene& S, int i) { return ((unsigned)i < (unsigned)PT_MAX_OBJECTS_SIZE) ? S.objects[i] : 0.0f; }
PT_DI float s_mat(const KScene& S, int i) { return ((unsigned)i < (unsigned)PT_MAX_MATERIALS_SIZE) ? S.materials[i] : 0.0f; }
PT_DI float s_light(const KScene& S, int i) { return ((unsigned)i < (unsigned)PT_MAX_LIGHTS_SIZE) ? S.lights[i] : 0.0f; }
PT_DI float s_lightid(const KScene& S, int i) { return ((unsigned)i < (unsigned)PT_MAX_LIGHTIDS_SIZE) ? S.lightIDs[i] : 0.0f; }

PT_DI m3 s_rotation(const KScene& S, int global_index) {
    const float* r = S.rot[global_index];
    return m3{f3(r[0], r[1], r[2]), f3(r[3], r[4], r[5]), f3(r[6], r[7], r[8])};
}
// The same matrix in precision R (the double renderer widens the table's floats).
template <typename R> PT_DI M3<R> s_rotation_r(const KScene& S, int global_index) {
    const float* r = S.rot[global_index];
    return M3<R>{v3<R>(r[0], r[1], r[2]), v3<R>(r[3], r[4], r[5]), v3<R>(r[6], r[7], r[8])};
}
