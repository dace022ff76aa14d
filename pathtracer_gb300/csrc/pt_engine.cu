// pt_engine.cu — host driver of the wavefront renderer (see pt_engine.h).
#include "pt_engine.h"

#include <cstring>

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
    P.s0 = take<float4>(p, pool);
    P.s1 = take<float4>(p, pool);
    P.s2 = take<float4>(p, pool);
    P.s3 = take<float4>(p, pool);
    P.s4 = take<float4>(p, pool);
    P.s5 = take<float4>(p, pool);
    P.s6 = take<float4>(p, pool);
    P.s7 = take<float4>(p, pool);
    P.s8 = take<uint4>(p, pool);
    P.s9 = take<float4>(p, pool);
    P.h0 = take<float4>(p, pool);
    P.h1 = take<float4>(p, pool);
    P.m0 = take<float4>(p, pool);
    P.m1 = take<float4>(p, pool);
    P.m2 = take<uint32_t>(p, pool);
    a->q_isect[0] = take<uint32_t>(p, pool);
    a->q_isect[1] = take<uint32_t>(p, pool);
    a->q_march[0] = take<uint32_t>(p, pool);
    a->q_march[1] = take<uint32_t>(p, pool);
    a->q_shade = take<uint32_t>(p, pool);
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
    e.args.pool_size = pool;
    e.args.march_budget = march_budget;
    e.args.trace = KTrace{nullptr, nullptr, nullptr, 0};
    int sms = 0;
    EN_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    e.grid = sms * 4;  // 4 blocks of 256 threads per SM (64 registers per thread)
    return e.reset();
}

cudaError_t WfEngine::create(int dev, cudaStream_t s, uint32_t pool_slots, uint32_t max_job_count, int march_budget) {
    destroy();
    buffer_bytes = bytes_for(pool_slots, max_job_count);
    EN_TRY(cudaMalloc(&buffer, buffer_bytes));
    owns_buffer = true;
    EN_TRY(cudaMallocHost(&host_counters, sizeof(WfCounters)));
    owns_host_counters = true;
    // Pinned: each entry is written once and copied to the device asynchronously.
    EN_TRY(cudaMallocHost(&jobs, sizeof(WfJob) * max_job_count));
    owns_jobs = true;
    return common_setup(*this, dev, s, pool_slots, max_job_count, march_budget);
}

cudaError_t WfEngine::attach(int dev, cudaStream_t s, uint32_t pool_slots, uint32_t max_job_count, int march_budget,
                             void* device_buffer, size_t bytes, WfCounters* host_counters_storage,
                             WfJob* host_jobs) {
    if (bytes < bytes_for(pool_slots, max_job_count) || !device_buffer || !host_counters_storage || !host_jobs)
        return cudaErrorInvalidValue;
    jobs = host_jobs;
    owns_jobs = false;
    buffer = device_buffer;
    buffer_bytes = bytes;
    owns_buffer = false;
    host_counters = host_counters_storage;
    owns_host_counters = false;
    return common_setup(*this, dev, s, pool_slots, max_job_count, march_budget);
}

void WfEngine::destroy() {
    if (owns_buffer && buffer) cudaFree(buffer);
    if (owns_host_counters && host_counters) cudaFreeHost(host_counters);
    if (owns_jobs && jobs) cudaFreeHost(jobs);
    buffer = nullptr;
    host_counters = nullptr;
    jobs = nullptr;
    owns_buffer = owns_host_counters = owns_jobs = false;
    njobs = 0;
    total = 0;
}

cudaError_t WfEngine::reset() {
    njobs = 0;
    total = 0;
    args.njobs = 0;
    return ptk_wavefront_launch_init(&args, stream);
}

cudaError_t WfEngine::add_pass(const WfJob& job, uint32_t* index) {
    if (njobs >= max_jobs) return cudaErrorInvalidValue;
    WfJob j = job;
    j.first = total;
    j.count = (uint32_t)((uint64_t)j.pc.resolution[0] * (uint64_t)j.pc.resolution[1] *
                         (uint64_t)j.pc.samplesPerFrame);
    j.finished = 0;
    std::memset(&j.cam, 0, sizeof j.cam);
    const uint32_t idx = njobs++;
    jobs[idx] = j;
    total += j.count;
    // Stream-ordered: the table entry, then its camera.  Kernels launched from
    // now on see njobs = idx + 1 and derive the sample total from this entry.
    EN_TRY(cudaMemcpyAsync(args.jobs + idx, &jobs[idx], sizeof(WfJob), cudaMemcpyHostToDevice, stream));
    args.njobs = idx + 1;
    EN_TRY(ptk_wavefront_launch_job_setup(&args, idx, idx + 1, stream));
    if (index) *index = idx;
    return cudaSuccess;
}

cudaError_t WfEngine::run(int n, bool trace) {
    for (int i = 0; i < n; i++) EN_TRY(ptk_wavefront_launch_iteration(&args, trace, grid, stream));
    return cudaSuccess;
}

cudaError_t WfEngine::read_counters(WfCounters* out) {
    EN_TRY(cudaMemcpyAsync(host_counters, args.counters, sizeof(WfCounters), cudaMemcpyDeviceToHost, stream));
    EN_TRY(cudaStreamSynchronize(stream));
    *out = *host_counters;
    return cudaSuccess;
}

cudaError_t WfEngine::read_finished(uint32_t j0, uint32_t j1, uint32_t* out) {
    for (uint32_t j = j0; j < j1; j++)
        EN_TRY(cudaMemcpyAsync(out + (j - j0), &args.jobs[j].finished, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                               stream));
    return cudaStreamSynchronize(stream);
}

cudaError_t WfEngine::resolve(uint32_t j) {
    if (j >= njobs) return cudaErrorInvalidValue;
    const WfJob& J = jobs[j];
    return ptk_wavefront_launch_resolve(&args, j, &J.pc, J.accum, J.colors, stream);
}

cudaError_t WfEngine::drain(bool trace, uint64_t max_iterations) {
    uint64_t iter = 0;
    int chunk = 8;
    WfCounters c;
    for (;;) {
        EN_TRY(run(chunk, trace));
        iter += (uint64_t)chunk;
        EN_TRY(read_counters(&c));
        if (c.next_sample == c.total && c.live == 0) return cudaSuccess;
        if (iter > max_iterations) return cudaErrorTimeout;
        if (chunk < 64) chunk *= 2;
    }
}
