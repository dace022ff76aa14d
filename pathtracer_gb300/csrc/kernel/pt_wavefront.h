// pt_wavefront.h — data of the wavefront renderer (pt_wavefront.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pt_scene.cuh"

// Path state, structure of arrays, one entry per pool slot (192 B per slot):
//   s0 org.xyz, mis       s1 dir.xyz, brdfPdf    s2 shDir.xyz, cosL
//   s3 nrm.xyz, lightPdf  s4 brdf                s5 throughput
//   s6 radiance           s7 wavelengths         s8 seed, flags|bounce, sample id, shObj
//   s9 shLightID, trace event word               h0 hitdist, materialID, lightID, objectID
//   h1 hit normal
// and the sphere-tracing state of a ray whose march continues in the next
// iteration: m0 t, insT, omega, prevRadius; m1 tMinMax.xy, k, set1 bits;
// m2 saved flag | points << 10 | loop iterations.
struct WfPool {
    float4 *s0, *s1, *s2, *s3, *s4, *s5, *s6, *s7;
    uint4* s8;
    float4 *s9, *h0, *h1;
    float4 *m0, *m1;
    uint32_t* m2;
};

struct WfCounters {
    uint32_t n_isect[2];  // the two ISECT queues (current, next)
    uint32_t cur;
    uint32_t n_march[2];  // the two MARCH queues (current, next)
    uint32_t march_cursor;
    uint32_t n_shade;
    uint32_t n_free;
    uint32_t next_sample;  // samples started so far
    uint32_t total;        // samples in the dispatch
    uint32_t iterations;
    uint32_t done;         // all samples started and finished
    uint32_t pad[4];
};

struct WfArgs {
    const KScene* scene;  // device copy of the scene
    pt_push pc;
    WfPool pool;
    uint32_t* q_isect[2];
    uint32_t* q_march[2];
    uint32_t* q_shade;
    uint32_t* q_free;
    WfCounters* counters;
    float4* colors;  // [k][pixel] sample XYZ
    float4* accum;
    const float* cie;
    KTrace trace;
    uint32_t pool_size;
    uint32_t total;
    int march_budget;  // sphere-tracing iterations per ray per march launch
};

// Bytes of device scratch for a pool of `pool` slots and `total` samples.
inline size_t ptk_wavefront_scratch_bytes(uint32_t pool, uint32_t total) {
    return (size_t)pool * (14 * 16 + 7 * 4) + (size_t)total * 16 + 256;
}

cudaError_t ptk_wavefront_launch_init(const WfArgs* a, cudaStream_t stream);
// One iteration: isect, march, shade, gen, bookkeeping (grid = blocks per stage kernel).
cudaError_t ptk_wavefront_launch_iteration(const WfArgs* a, bool trace, int grid, cudaStream_t stream);
cudaError_t ptk_wavefront_launch_resolve(const WfArgs* a, cudaStream_t stream);
