// pt_engine.h — host driver of the wavefront renderer.
//
// One engine owns a pool of path slots, its ray queues and a ring of render
// passes ("jobs": one scene, one accumulator, samplesPerFrame samples of every
// pixel).  Passes can be added while others are in flight; every sample of
// every pass is an independent work item of the same pool, so passes of
// different scenes, resolutions and sample counts share each launch.  The
// caller drives iterations, resolves each pass once all of its samples have
// finished, and retires resolved passes so their ring entries can be reused.
//
// The kernels' arguments do not change between resets (pass bounds live in
// device counters), so a chain of iterations is captured once as a CUDA graph
// and replayed: one launch per chunk instead of five per iteration.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "kernel/pt_wavefront.h"

#include <cmath>
#include <string>

// Checks a scene's extension block (NULL is the reference's method and
// valid); *why receives the reason for a refusal.
inline bool pt_ext_valid(const pt_scene_ext* x, std::string* why) {
    if (!x) return true;
    const int known = PT_EXT_SKY | PT_EXT_WAVELENGTHS | PT_EXT_ANALYTIC_CMF | PT_EXT_MARCH | PT_EXT_MATERIALS;
    if (x->flags & ~known) return (*why = "unknown extension flags", false);
    if ((x->flags & PT_EXT_SKY) && !(x->sky_temperature >= 0.0f && x->sky_luminosity >= 0.0f))
        return (*why = "sky temperature and luminosity must be >= 0", false);
    if (x->flags & PT_EXT_WAVELENGTHS) {
        if (!(x->lambda_min > 0.0f && x->lambda_max > x->lambda_min && x->lambda_max < 1e5f))
            return (*why = "wavelength range must satisfy 0 < min < max", false);
        if (!(x->flags & PT_EXT_ANALYTIC_CMF) && (x->lambda_min < 360.0f || x->lambda_max > 800.0f))
            return (*why = "the tabulated CIE table covers 360-800 nm: use the analytic CMF beyond it", false);
    }
    if ((x->flags & PT_EXT_MARCH) && !(x->march_max_steps >= 1 && x->march_max_steps <= 1023 &&
                                        x->march_epsilon > 0.0f && x->march_max_distance > 0.0f))
        return (*why = "march limits: 1..1023 steps, epsilon > 0, distance > 0", false);
    if (x->flags & PT_EXT_MATERIALS) {
        if (x->nmat < 0 || x->nmat > PT_MAX_EXT_MATERIALS) return (*why = "nmat out of range", false);
        for (int i = 0; i < x->nmat; i++) {
            const pt_material_ext& m = x->mat[i];
            if (m.type < PT_BSDF_REFERENCE || m.type > PT_BSDF_SELLMEIER)
                return (*why = "material " + std::to_string(i + 1) + ": unknown type", false);
            for (int j = 0; j < 6; j++)
                if (!std::isfinite(m.p[j])) return (*why = "material " + std::to_string(i + 1) + ": non-finite parameter", false);
            if (m.type == PT_BSDF_SMOOTH && m.p[3] == 0.0f)
                return (*why = "material " + std::to_string(i + 1) + ": zero width", false);
            if (m.type == PT_BSDF_CAUCHY && !(m.p[0] > 0.0f))
                return (*why = "material " + std::to_string(i + 1) + ": Cauchy A must be > 0", false);
        }
    }
    return true;
}

// Names of the PT_CHECK_* sites for error messages.
inline const char* pt_check_site_name(uint32_t site) {
    switch (site) {
        case PT_CHECK_QUEUE_APPEND: return "queue append past the pool size";
        case PT_CHECK_QUEUE_SLOT: return "queue entry outside the pool";
        case PT_CHECK_FREE_INDEX: return "free-list read outside the list";
        case PT_CHECK_JOB: return "pass index outside the job ring";
        case PT_CHECK_SAMPLE: return "sample index outside its pass";
        case PT_CHECK_QUEUE_COUNT: return "queue length above the pool size";
        default: return "unknown site";
    }
}

struct WfEngine;
// Drains n (1..8) staged engines on different streams, each relaunched as
// soon as its last chunk of iterations has been read back, so that one
// engine's kernels fill the SMs that the others' kernel tails and host
// round trips leave idle.  Same results and iteration bound (per engine) as
// drain() without a trace.
cudaError_t wf_drain_many(WfEngine* const* engines, int n, uint64_t max_iterations);

struct WfEngine {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t pool = 0;
    uint32_t max_jobs = 0;    // ring entries
    int grid = 0;
    WfArgs args{};
    int sms_count = 0;
    int blocks_per_sm = 4;
    WfJob* jobs = nullptr;    // host mirror of the ring (max_jobs entries)
    uint32_t njobs = 0;       // passes added since the last reset (job_hi)
    uint32_t lo = 0;          // passes below this were resolved and retired
    bool owns_jobs = false;
    uint64_t total = 0;       // samples of all passes added
    void* buffer = nullptr;   // device memory of pool, queues, counters and job table
    bool owns_buffer = false;
    size_t buffer_bytes = 0;
    WfCounters* host_counters = nullptr;  // read-back target (pinned when the engine allocated it)
    bool owns_host_counters = false;
    // Graph replay of `graph_chunk` iterations (engines that allocate only).
    bool use_graph = false;
    int graph_chunk = 8;
    cudaGraphExec_t graph = nullptr;
    // Persistent mode: each iteration is one launch of the persistent path
    // kernel over the next `persist_budget` samples instead of one pass of
    // the staged kernels; the pool is not used.
    bool persistent = false;
    int sms = 0;
    uint64_t persist_budget = 1ull << 23;
    // A pass's remainder at least this large gets a launch of its own (with
    // its scene in the constant bank) instead of sharing one with the next.
    static constexpr uint64_t kPersistOnePassMin = 1ull << 20;
    uint64_t persist_issued = 0;  // samples covered by launches so far
    // Stage timing (off by default): every iteration is launched without the
    // graph, bracketed by events; stage_ms accumulates device milliseconds.
    bool stage_timing = false;
    double stage_ms[PT_STAGE_COUNT] = {0, 0, 0, 0, 0};
    uint64_t stage_launches = 0;
    // The march kernel launched instead of the built-in wf_march: a run-time
    // compiled one (scenes with SDF snippets compiled by pt_jit.cu) or the
    // built-in warp-wide-normals one; null for wf_march.
    const void* march_kernel = nullptr;
    // Kernels this engine has launched (graph replays counted per kernel).
    uint64_t kernel_launches = 0;
    // The wavefront kernels launched: the default build, or the checked one
    // (set_checks; its failed index checks are read back by check_failed).
    const WfKernelSet* kernels = ptk_wavefront_kernels(false);
    bool checks = false;

    // Bytes of device memory for `pool` slots and `max_jobs` ring entries.
    static size_t bytes_for(uint32_t pool, uint32_t max_jobs);
    // Allocates its own memory.
    cudaError_t create(int device, cudaStream_t stream, uint32_t pool, uint32_t max_jobs, int march_budget);
    // Uses caller-provided device memory (bytes_for) and host storage for the
    // counters and the job ring (max_jobs entries); allocates nothing and
    // launches kernels one by one.
    cudaError_t attach(int device, cudaStream_t stream, uint32_t pool, uint32_t max_jobs, int march_budget,
                       void* device_buffer, size_t bytes, WfCounters* host_counters_storage, WfJob* host_jobs);
    void destroy();

    // Empties the pool and the job ring (asynchronous, stream-ordered).
    cudaError_t reset();
    // Sphere-tracing iterations per ray per march launch.
    void set_march_budget(int budget);
    // March refill threshold, drain threshold and stage-kernel blocks per SM.
    void set_tuning(int refill_min, int drain_lanes, int blocks_per_sm, int march_inner);
    // Sets march_kernel (null: the built-in kernel).
    void set_march_kernel(const void* kernel);
    // The checked kernel build on or off (the march kernel set by
    // set_march_kernel must be of the same build).
    void set_checks(bool on);
    // After read_counters or drain: the site (PT_CHECK_*) and index of the
    // first failed index check since the last reset, 0 when none failed or
    // the checks are off.
    uint32_t check_failed(uint32_t* index) const;
    // Staged kernels (false) or the persistent path kernel (true).
    void set_persistent(bool on);
    // Persistent mode: every sample added so far is covered by a launch.
    bool persistent_idle() const { return persist_issued >= total; }
    // Stream the kernels are launched on.
    void set_stream(cudaStream_t s);
    // Appends a pass; `job` is filled by the caller except first/count/finished/cam
    // (job.variant: the scene's primitive classes, PT_FEAT_ALL when unknown).
    // Fails with cudaErrorInvalidValue while the ring is full.
    cudaError_t add_pass(const WfJob& job, uint32_t* index);
    // Appends samples [local_base, local_base + count) of a pass (in the
    // pass's sample order, [k][pixel]); the rest of the pass is rendered
    // elsewhere (another engine) and the pass is resolved once both parts
    // have finished.  The colour buffer is the whole pass's.
    cudaError_t add_pass_part(const WfJob& job, uint32_t local_base, uint32_t count, uint32_t* index);
    // Passes [lo, new_lo) were resolved: their ring entries may be reused.
    void retire(uint32_t new_lo);
    // Launches `n` iterations.
    cudaError_t run(int n, bool trace);
    // Stage timing on or off (clears the totals).
    cudaError_t set_stage_timing(bool on);
    // Reads the counters (synchronises the stream).
    cudaError_t read_counters(WfCounters* out);
    // Reads the finished-sample counts of passes [j0, j1) (at most max_jobs;
    // synchronises the stream).
    cudaError_t read_finished(uint32_t j0, uint32_t j1, uint32_t* out);
    // Rendering/Accumulate of pass `j` into its accumulator (on `on`, or the
    // engine's stream).
    cudaError_t resolve(uint32_t j, cudaStream_t on = nullptr);
    // Host copy of pass j (valid until its ring entry is reused).
    const WfJob& job(uint32_t j) const { return jobs[j % max_jobs]; }
    // Runs until every pass added so far has finished (polling between chunks of
    // iterations), or `max_iterations` have run (returns cudaErrorTimeout then).
    cudaError_t drain(bool trace, uint64_t max_iterations);

   private:
    void drop_graph();
    cudaError_t build_graph();
    cudaEvent_t* stage_ev = nullptr;  // [64][6] events, reused in rounds of 64 iterations
    int stage_ev_used = 0;
    cudaError_t flush_stage_events();
};
