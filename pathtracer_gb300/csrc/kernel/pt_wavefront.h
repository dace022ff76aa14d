// pt_wavefront.h — data of the wavefront renderer (pt_wavefront.cu) and the
// host-side engine that drives it (pt_engine.cu).
#pragma once

#if !defined(__CUDACC_RTC__)
#include <cuda_runtime.h>
#include <stdint.h>
#endif

#include "pt_scene.cuh"

// Path state, one entry per pool slot, in 16-byte fields:
//   s0 org.xyz, mis       s1 dir.xyz, brdfPdf    s2 shDir.xyz, cosL
//   s3 nrm.xyz, lightPdf  s4 brdf                s5 throughput
//   s6 radiance           s7 wavelengths         s8 seed, flags|bounce, sample (in its pass), job << 12 | shObj
//   s9 shLightID, trace event word               h0 hitdist, materialID, lightID, objectID
//   h1 hit normal
// and the sphere-tracing state of a ray whose march continues in the next
// iteration: m0 t, insT, omega, prevRadius; m1 tMinMax.xy, saved flag |
// (k + 1) << 26 | points << 10 | loop iterations, set1 bits.
// Fields the stages read or write together are stored in pairs, one slot's
// pair in one 32-byte sector: (s0, s1), (s2, s3), (s4, s9), (s5, s6),
// (s7, s8), (h0, h1), (m0, m1).  Slots come from the queues in no useful
// order, so a lone 16-byte field would use half of each sector it moves
// (and a lone store makes the L2 read the other half from DRAM).
struct WfPool {
    float4 *s01, *s23, *s49, *s56, *s78, *h01, *m01;  // 2 x 16 B per slot each
};

// Entries of a job ring at most (a ring index is stored in 20 bits of the
// path state).
constexpr uint32_t kMaxJobRing = 1u << 20;

// One render pass of one job: samplesPerFrame samples of every pixel.
// The table is a ring of job_cap entries: pass number j (counting every pass
// added since the last reset) lives at jobs[j % job_cap].  Passes [job_lo,
// job_hi) are live; an entry is reused only after its pass was resolved.
struct WfJob {
    const KScene* scene;  // device copy of the job's scene
    const float* cie;     // device CIE table
    float4* accum;        // W*H float4 accumulator (read and written by resolve)
    float4* colors;       // W*H*spf sample XYZ, [k][pixel]
    uint64_t first;       // global index of the pass's first sample
    uint32_t count;       // W*H*spf
    uint32_t finished;    // samples finished (atomic)
    int32_t variant;      // primitive classes of the scene (PT_FEAT_*), for the persistent kernel
    uint32_t local_base;  // pass index of this entry's first sample (a pass split between engines; else 0)
    const KScene* host_scene;  // host copy of *scene (persistent single-pass launches; null: none)
    CamInfo cam;          // camera derived on the device (wf_job_setup)
    pt_push pc;
};

struct WfCounters {
    uint32_t n_march[2];   // MARCH queues (current, next)
    uint32_t cur;
    uint32_t march_cursor;
    uint32_t n_shade[2];   // primary-ray hits to shade (current, next)
    uint32_t n_free;
    uint64_t next_sample;  // global samples started so far
    uint64_t total;        // global samples of every pass in the table (written by the bookkeeping kernel)
    uint32_t iterations;
    uint32_t live;         // slots holding a path (pool - n_free)
    uint32_t job_lo;       // oldest pass that may still hold unfinished samples
    uint32_t job_hi;       // passes added so far
    uint64_t pk_end;       // persistent mode: end of the sample range of the current launch
    uint32_t n_shadow[2];  // shadow-ray results to shade (current, next)
    // Kernels built with PT_DEBUG_CHECKS: the first index check that failed
    // since the last reset (PT_CHECK_* site, 0: none) and the index it saw.
    uint32_t check_site;
    uint32_t check_index;
};

// Sites of the index checks of the checked kernel build (PT_DEBUG_CHECKS).
enum {
    PT_CHECK_NONE = 0,
    PT_CHECK_QUEUE_APPEND = 1,  // an append past a queue's capacity (the pool size)
    PT_CHECK_QUEUE_SLOT = 2,    // a slot read from a queue outside the pool
    PT_CHECK_FREE_INDEX = 3,    // a free-list read outside the list
    PT_CHECK_JOB = 4,           // a pass index outside the job ring
    PT_CHECK_SAMPLE = 5,        // a sample index outside its pass (colour buffer)
    PT_CHECK_QUEUE_COUNT = 6,   // a queue or free-list length above the pool size after an iteration
};

// Everything here is fixed between resets, so a captured chain of iterations
// stays valid while passes are added and retired.
struct WfArgs {
    WfJob* jobs;   // device job table (ring)
    uint32_t job_cap;
    WfPool pool;
    uint32_t* q_march[2];
    uint32_t* q_shade[2];   // primary-ray hits (current, next)
    uint32_t* q_shadow[2];  // shadow-ray results (current, next)
    uint32_t* q_free;
    WfCounters* counters;
    KTrace trace;  // single-job dispatches only
    uint32_t pool_size;
    int march_budget;  // sphere-tracing iterations per ray per march launch
    int refill_min;    // idle lanes a march warp gathers before it refills them at once
    int drain_lanes;   // a drained march warp with fewer rays suspends them (0: never)
    int march_inner;   // SDF evaluations per lane between a march warp's refills and queue appends
    int persist_refill;  // idle lanes a persistent warp gathers before starting new samples together
};

// Host side (not seen by the run-time compiled program, pt_jit.cu).
#if !defined(__CUDACC_RTC__)
// Bytes of the engine's device buffers for a pool of `pool` slots.
inline size_t ptk_wavefront_pool_bytes(uint32_t pool) { return (size_t)pool * (14 * 16 + 7 * 4) + 32 * 256; }

cudaError_t ptk_wavefront_launch_init(const WfArgs* a, cudaStream_t stream);
// Writes pass number `index` (camera derived on the device) and publishes
// job_hi = index + 1, job_lo = lo.
cudaError_t ptk_wavefront_launch_job_add(const WfArgs* a, const WfJob* job, uint32_t index, uint32_t lo,
                                         cudaStream_t stream);
// One iteration: march, shade, gen, bookkeeping (grid = blocks per stage
// kernel, capped per kernel at what is resident); with stage_events, 6
// events bracket the 5 stages (isect, done inside shade and gen, stays empty).
// march_kernel: the march kernel to launch instead of the built-in wf_march:
// a run-time compiled one (pt_jit.cu; scenes with SDF snippets compiled at
// run time) or ptk_wavefront_march_warp_normals().
cudaError_t ptk_wavefront_launch_iteration(const WfArgs* a, bool trace, int grid, cudaStream_t stream,
                                           cudaEvent_t* stage_events = nullptr, const void* march_kernel = nullptr);
// The built-in march kernel that probes normals across the warp, for
// dispatches with a mandelbulb (pass it as march_kernel; the default
// built-in kernel probes each ray's normal on its own lane).
const void* ptk_wavefront_march_warp_normals();
// Kernels launched per staged iteration (march, shade, gen, bookkeeping).
constexpr int kWfKernelsPerIteration = 4;
// Stages timed by the engine's stage-timing mode.
enum { PT_STAGE_ISECT = 0, PT_STAGE_MARCH, PT_STAGE_SHADE, PT_STAGE_GEN, PT_STAGE_BOOK, PT_STAGE_COUNT };
// Persistent mode: one launch of the persistent path kernel over the next
// `budget` samples of the job ring, compiled for primitive classes `variant`
// (PT_FEAT_*: 0, BOX, ANALYTIC or ALL), with every block resident at once
// on `sms` multiprocessors.  one_scene (host copy, or null): every sample of
// the launch belongs to one pass of this scene, which then travels as the
// launch's parameter and is read from the constant bank.
cudaError_t ptk_persist_launch(const WfArgs* a, int variant, int sms, uint64_t budget, const KScene* one_scene,
                               cudaStream_t stream);
// Blocks of the persistent kernel variant that fit on one SM at once.
int ptk_persist_blocks_per_sm(int variant);
constexpr int kPersistThreads = 128;
// Rendering/Accumulate of one job pass from its ordered sample colours.
cudaError_t ptk_wavefront_launch_resolve(const WfArgs* a, uint32_t job, const pt_push* pc, float4* accum,
                                         const float4* colors, cudaStream_t stream);

// The launch functions above as a set, for the engine to switch between the
// default build of the wavefront kernels and the checked one.
struct WfKernelSet {
    cudaError_t (*init)(const WfArgs*, cudaStream_t);
    cudaError_t (*job_add)(const WfArgs*, const WfJob*, uint32_t, uint32_t, cudaStream_t);
    cudaError_t (*iteration)(const WfArgs*, bool, int, cudaStream_t, cudaEvent_t*, const void*);
    const void* (*march_warp_normals)();
    cudaError_t (*persist)(const WfArgs*, int, int, uint64_t, const KScene*, cudaStream_t);
    int (*persist_blocks_per_sm)(int);
    cudaError_t (*resolve)(const WfArgs*, uint32_t, const pt_push*, float4*, const float4*, cudaStream_t);
};
// checked = false: the kernels above; true: the same kernels built with
// PT_DEBUG_CHECKS (pt_wavefront_checked.cu): every queue, pool-slot, ring and
// sample index is checked before use, a failed check is recorded in the
// counters (check_site, check_index) and its access skipped.
const WfKernelSet* ptk_wavefront_kernels(bool checked);
#endif  // !__CUDACC_RTC__
