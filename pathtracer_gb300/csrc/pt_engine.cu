// pt_engine.cu — host driver of the wavefront renderer (see pt_engine.h).
#include "pt_engine.h"

#include "kernel/pt_features.h"

#include <cstring>
#include <new>

namespace {

constexpr size_t r256(size_t x) { return (x + 255) / 256 * 256; }


template <typename T>
T* take(uintptr_t& p, size_t count) {
    T* r = reinterpret_cast<T*>(p);
    p += r256(count * sizeof(T));
    return r;
}

// Carves the engine's arrays out of one buffer; returns the bytes used.
size_t layout(uintptr_t base, uint32_t pool, uint32_t max_jobs, WfArgs* a) {
    uintptr_t p = base;
    WfPool& P = a->pool;
    P.s01 = take<float4>(p, 2 * (size_t)pool);
    P.s23 = take<float4>(p, 2 * (size_t)pool);
    P.s49 = take<float4>(p, 2 * (size_t)pool);
    P.s56 = take<float4>(p, 2 * (size_t)pool);
    P.s78 = take<float4>(p, 2 * (size_t)pool);
    P.h01 = take<float4>(p, 2 * (size_t)pool);
    P.m01 = take<float4>(p, 2 * (size_t)pool);
    a->q_march[0] = take<uint32_t>(p, pool);
    a->q_march[1] = take<uint32_t>(p, pool);
    a->q_shade[0] = take<uint32_t>(p, pool);
    a->q_shade[1] = take<uint32_t>(p, pool);
    a->q_shadow[0] = take<uint32_t>(p, pool);
    a->q_shadow[1] = take<uint32_t>(p, pool);
    a->q_free = take<uint32_t>(p, pool);
    a->counters = take<WfCounters>(p, 1);
    a->jobs = take<WfJob>(p, max_jobs);
    return (size_t)(p - base);
}

#define EN_TRY(call)                    \
    do {                                \
        const cudaError_t e_ = (call);  \
        if (e_ != cudaSuccess) return e_; \
    } while (0)

}  // namespace

size_t WfEngine::bytes_for(uint32_t pool, uint32_t max_jobs) {
    WfArgs a;
    std::memset(&a, 0, sizeof a);
    return layout(0, pool, max_jobs, &a);
}

static cudaError_t common_setup(WfEngine& e, int device, cudaStream_t stream, uint32_t pool, uint32_t max_jobs,
                                int march_budget) {
    e.device = device;
    e.stream = stream;
    e.pool = pool;
    e.max_jobs = max_jobs;
    std::memset(&e.args, 0, sizeof e.args);
    layout(reinterpret_cast<uintptr_t>(e.buffer), pool, max_jobs, &e.args);
    e.args.job_cap = max_jobs;
    e.args.pool_size = pool;
    e.args.march_budget = march_budget;
    e.args.refill_min = 2;
    e.args.drain_lanes = 24;
    e.args.march_inner = 6;      // measured best on GB300 (mandelbulb, menger + terrain)
    e.args.persist_refill = 16;  // measured best on GB300 (batch of 64 sphere jobs)
    e.args.trace = KTrace{nullptr, nullptr, nullptr, 0};
    int sms = 0;
    EN_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    e.sms = e.sms_count = sms;
    e.grid = sms * e.blocks_per_sm;  // blocks of 256 threads (64 registers per thread: 4 fit on an SM)
    return e.reset();
}

cudaError_t WfEngine::create(int dev, cudaStream_t s, uint32_t pool_slots, uint32_t max_job_count, int march_budget) {
    if (max_job_count == 0 || max_job_count > kMaxJobRing) return cudaErrorInvalidValue;
    destroy();
    buffer_bytes = bytes_for(pool_slots, max_job_count);
    EN_TRY(cudaMalloc(&buffer, buffer_bytes));
    owns_buffer = true;
    EN_TRY(cudaMallocHost(&host_counters, sizeof(WfCounters)));
    owns_host_counters = true;
    jobs = new (std::nothrow) WfJob[max_job_count];
    if (!jobs) return cudaErrorMemoryAllocation;
    owns_jobs = true;
    use_graph = true;
    return common_setup(*this, dev, s, pool_slots, max_job_count, march_budget);
}

cudaError_t WfEngine::attach(int dev, cudaStream_t s, uint32_t pool_slots, uint32_t max_job_count, int march_budget,
                             void* device_buffer, size_t bytes, WfCounters* host_counters_storage,
                             WfJob* host_jobs) {
    if (bytes < bytes_for(pool_slots, max_job_count) || !device_buffer || !host_counters_storage || !host_jobs ||
        max_job_count == 0 || max_job_count > kMaxJobRing)
        return cudaErrorInvalidValue;
    jobs = host_jobs;
    owns_jobs = false;
    buffer = device_buffer;
    buffer_bytes = bytes;
    owns_buffer = false;
    host_counters = host_counters_storage;
    owns_host_counters = false;
    use_graph = false;
    return common_setup(*this, dev, s, pool_slots, max_job_count, march_budget);
}

void WfEngine::drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
}

void WfEngine::destroy() {
    drop_graph();
    set_stage_timing(false);
    if (owns_buffer && buffer) cudaFree(buffer);
    if (owns_host_counters && host_counters) cudaFreeHost(host_counters);
    if (owns_jobs && jobs) delete[] jobs;
    buffer = nullptr;
    host_counters = nullptr;
    jobs = nullptr;
    owns_buffer = owns_host_counters = owns_jobs = false;
    use_graph = false;
    njobs = lo = 0;
    total = 0;
}

void WfEngine::set_march_budget(int budget) {
    if (budget != args.march_budget) drop_graph();
    args.march_budget = budget;
}

void WfEngine::set_stream(cudaStream_t s) { stream = s; }

void WfEngine::set_tuning(int refill, int drain, int bps, int inner) {
    if (refill != args.refill_min || drain != args.drain_lanes || bps != blocks_per_sm || inner != args.march_inner)
        drop_graph();
    args.refill_min = refill;
    args.drain_lanes = drain;
    args.march_inner = inner;
    blocks_per_sm = bps;
    grid = sms_count * bps;
}

void WfEngine::set_persistent(bool on) { persistent = on; }

void WfEngine::set_checks(bool on) {
    if (on != checks) drop_graph();
    checks = on;
    kernels = ptk_wavefront_kernels(on);
}

uint32_t WfEngine::check_failed(uint32_t* index) const {
    if (!checks || !host_counters || host_counters->check_site == PT_CHECK_NONE) return PT_CHECK_NONE;
    if (index) *index = host_counters->check_index;
    return host_counters->check_site;
}

extern const WfKernelSet ptk_wavefront_kernel_set;
extern const WfKernelSet ptk_wavefront_kernel_set_checked;
const WfKernelSet* ptk_wavefront_kernels(bool checked) {
    return checked ? &ptk_wavefront_kernel_set_checked : &ptk_wavefront_kernel_set;
}

void WfEngine::set_march_kernel(const void* kernel) {
    if (kernel != march_kernel) drop_graph();
    march_kernel = kernel;
}

cudaError_t WfEngine::reset() {
    njobs = lo = 0;
    total = 0;
    persist_issued = 0;
    kernel_launches += 1;
    return kernels->init(&args, stream);
}

cudaError_t WfEngine::add_pass(const WfJob& job, uint32_t* index) {
    return add_pass_part(job, 0, (uint32_t)((uint64_t)job.pc.resolution[0] * (uint64_t)job.pc.resolution[1] *
                                            (uint64_t)job.pc.samplesPerFrame),
                         index);
}

cudaError_t WfEngine::add_pass_part(const WfJob& job, uint32_t local_base, uint32_t count, uint32_t* index) {
    if (njobs - lo >= max_jobs) return cudaErrorInvalidValue;
    const uint64_t whole = (uint64_t)job.pc.resolution[0] * (uint64_t)job.pc.resolution[1] *
                           (uint64_t)job.pc.samplesPerFrame;
    if ((uint64_t)local_base + count > whole) return cudaErrorInvalidValue;
    WfJob j = job;
    j.first = total;
    j.count = count;
    j.local_base = local_base;
    j.finished = 0;
    std::memset(&j.cam, 0, sizeof j.cam);
    const uint32_t idx = njobs;
    // Stream-ordered: kernels launched from now on see job_hi = idx + 1 and
    // derive the sample total from this entry.
    EN_TRY(kernels->job_add(&args, &j, idx, lo, stream));
    kernel_launches += 1;
    jobs[idx % max_jobs] = j;
    njobs = idx + 1;
    total += j.count;
    if (index) *index = idx;
    return cudaSuccess;
}

void WfEngine::retire(uint32_t new_lo) {
    if (new_lo > lo && new_lo <= njobs) lo = new_lo;
}

cudaError_t WfEngine::build_graph() {
    drop_graph();
    cudaStream_t cs = nullptr;
    EN_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    WfArgs a = args;
    a.trace = KTrace{nullptr, nullptr, nullptr, 0};
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        for (int i = 0; i < graph_chunk && e == cudaSuccess; i++)
            e = kernels->iteration(&a, false, grid, cs, nullptr, march_kernel);
        const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&graph, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) graph = nullptr;
    return e;
}

namespace {
constexpr int kStageEvRounds = 64;
}

cudaError_t WfEngine::set_stage_timing(bool on) {
    if (stage_ev) {
        for (int i = 0; i < kStageEvRounds * 6; i++) cudaEventDestroy(stage_ev[i]);
        delete[] stage_ev;
        stage_ev = nullptr;
    }
    stage_ev_used = 0;
    stage_timing = on;
    for (double& v : stage_ms) v = 0.0;
    stage_launches = 0;
    if (!on) return cudaSuccess;
    stage_ev = new (std::nothrow) cudaEvent_t[kStageEvRounds * 6];
    if (!stage_ev) return cudaErrorMemoryAllocation;
    for (int i = 0; i < kStageEvRounds * 6; i++) EN_TRY(cudaEventCreate(&stage_ev[i]));
    return cudaSuccess;
}

// Adds the recorded rounds to stage_ms (synchronises on the last event).
cudaError_t WfEngine::flush_stage_events() {
    if (!stage_ev_used) return cudaSuccess;
    EN_TRY(cudaEventSynchronize(stage_ev[stage_ev_used * 6 - 1]));
    for (int r = 0; r < stage_ev_used; r++) {
        for (int k = 0; k < PT_STAGE_COUNT; k++) {
            float ms = 0.0f;
            EN_TRY(cudaEventElapsedTime(&ms, stage_ev[r * 6 + k], stage_ev[r * 6 + k + 1]));
            stage_ms[k] += ms;
        }
    }
    stage_launches += (uint64_t)stage_ev_used;
    stage_ev_used = 0;
    return cudaSuccess;
}

cudaError_t WfEngine::run(int n, bool trace) {
    if (stage_timing && !persistent) {
        for (int i = 0; i < n; i++) {
            if (stage_ev_used == kStageEvRounds) EN_TRY(flush_stage_events());
            EN_TRY(kernels->iteration(&args, trace, grid, stream, &stage_ev[stage_ev_used * 6], march_kernel));
            kernel_launches += kWfKernelsPerIteration;
            stage_ev_used++;
        }
        return flush_stage_events();
    }
    if (persistent) {
        // One kernel variant covering every pass still in the ring.
        int variant = 0;
        for (uint32_t j = lo; j < njobs; j++) variant = pt_variant_union(variant, jobs[j % max_jobs].variant);
        for (int i = 0; i < n && persist_issued < total; i++) {
            // A launch that stays within one pass (the rest of a large pass,
            // or the next budget of it) takes that pass's scene as its
            // parameter, read from the constant bank like the megakernel's;
            // a launch spanning passes reads each lane's scene by pointer.
            uint64_t budget = total - persist_issued < persist_budget ? total - persist_issued : persist_budget;
            const KScene* one = nullptr;
            int v = variant;
            for (uint32_t j = lo; j < njobs; j++) {
                const WfJob& J = jobs[j % max_jobs];
                if (persist_issued < J.first || persist_issued >= J.first + J.count) continue;
                const uint64_t left = J.first + J.count - persist_issued;
                if (J.host_scene && (left >= budget || left >= kPersistOnePassMin)) {
                    budget = left < budget ? left : budget;
                    one = J.host_scene;
                    v = J.variant;
                }
                break;
            }
            EN_TRY(kernels->persist(&args, v, sms, budget, one, stream));
            kernel_launches += 2;  // setup + persistent kernel
            persist_issued += budget;
        }
        return cudaSuccess;
    }
    if (use_graph && !trace && n >= graph_chunk) {
        if (!graph) EN_TRY(build_graph());
        for (; n >= graph_chunk; n -= graph_chunk) {
            EN_TRY(cudaGraphLaunch(graph, stream));
            kernel_launches += (uint64_t)graph_chunk * kWfKernelsPerIteration;
        }
    }
    for (int i = 0; i < n; i++) {
        EN_TRY(kernels->iteration(&args, trace, grid, stream, nullptr, march_kernel));
        kernel_launches += kWfKernelsPerIteration;
    }
    return cudaSuccess;
}

cudaError_t WfEngine::read_counters(WfCounters* out) {
    EN_TRY(cudaMemcpyAsync(host_counters, args.counters, sizeof(WfCounters), cudaMemcpyDeviceToHost, stream));
    EN_TRY(cudaStreamSynchronize(stream));
    *out = *host_counters;
    return cudaSuccess;
}

cudaError_t WfEngine::read_finished(uint32_t j0, uint32_t j1, uint32_t* out) {
    if (j1 < j0 || j1 - j0 > max_jobs) return cudaErrorInvalidValue;
    // The `finished` fields of a run of ring entries: one strided copy, two
    // where the run wraps.
    uint32_t j = j0;
    while (j < j1) {
        const uint32_t r = j % max_jobs;
        const uint32_t n = (j1 - j < max_jobs - r) ? (j1 - j) : (max_jobs - r);
        EN_TRY(cudaMemcpy2DAsync(out + (j - j0), sizeof(uint32_t), &args.jobs[r].finished, sizeof(WfJob),
                                 sizeof(uint32_t), n, cudaMemcpyDeviceToHost, stream));
        j += n;
    }
    return cudaStreamSynchronize(stream);
}

cudaError_t WfEngine::resolve(uint32_t j, cudaStream_t on) {
    if (j >= njobs || j < lo) return cudaErrorInvalidValue;
    const WfJob& J = job(j);
    kernel_launches += 1;
    return kernels->resolve(&args, j % max_jobs, &J.pc, J.accum, J.colors, on ? on : stream);
}

cudaError_t wf_drain_many(WfEngine* const* e, int n, uint64_t max_iterations) {
    constexpr int kMax = 8;
    if (n < 1 || n > kMax) return cudaErrorInvalidValue;
    for (int i = 0; i < n; i++) {
        if (e[i]->persistent) return cudaErrorInvalidValue;
        for (int k = 0; k < i; k++)
            if (e[k]->stream == e[i]->stream) return cudaErrorInvalidValue;
    }
    int chunk[kMax];
    uint64_t iter[kMax];
    bool done[kMax];
    for (int i = 0; i < n; i++) {
        chunk[i] = 8;
        iter[i] = 8;
        done[i] = false;
        EN_TRY(e[i]->run(chunk[i], false));
    }
    for (int left = n; left > 0;) {
        for (int i = 0; i < n; i++) {
            if (done[i]) continue;
            WfCounters c;
            EN_TRY(e[i]->read_counters(&c));  // waits for this engine's stream only
            // finished, or stopped by a failed index check (the caller reports it)
            if ((c.next_sample == c.total && c.live == 0) || c.check_site != PT_CHECK_NONE) {
                done[i] = true;
                left--;
                continue;
            }
            if (iter[i] > max_iterations) return cudaErrorTimeout;
            if (chunk[i] < 64) chunk[i] *= 2;
            EN_TRY(e[i]->run(chunk[i], false));
            iter[i] += (uint64_t)chunk[i];
        }
    }
    return cudaSuccess;
}

cudaError_t WfEngine::drain(bool trace, uint64_t max_iterations) {
    if (persistent) {
        // Every launch finishes the samples it covers.
        for (uint64_t launches = 0; persist_issued < total; launches++) {
            if (launches >= max_iterations) return cudaErrorTimeout;
            EN_TRY(run(1, false));
        }
        return read_counters(host_counters);
    }
    uint64_t iter = 0;
    int chunk = 8;
    WfCounters c;
    for (;;) {
        EN_TRY(run(chunk, trace));
        iter += (uint64_t)chunk;
        EN_TRY(read_counters(&c));
        if (c.next_sample == c.total && c.live == 0) return cudaSuccess;
        // A failed index check skipped an access and may have lost a path:
        // stop here; the caller reports it (check_failed).
        if (c.check_site != PT_CHECK_NONE) return cudaSuccess;
        if (iter > max_iterations) return cudaErrorTimeout;
        if (chunk < 64) chunk *= 2;
    }
}
