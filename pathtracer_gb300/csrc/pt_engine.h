// pt_engine.h — host driver of the wavefront renderer.
//
// One engine owns a pool of path slots, its ray queues and a table of render
// passes ("jobs": one scene, one accumulator, samplesPerFrame samples of every
// pixel).  Passes can be added while others are in flight; every sample of
// every pass is an independent work item of the same pool, so passes of
// different scenes, resolutions and sample counts share each launch.  The
// caller drives iterations and resolves each pass once all of its samples
// have finished.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "kernel/pt_wavefront.h"

struct WfEngine {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t pool = 0;
    uint32_t max_jobs = 0;
    int grid = 0;
    WfArgs args{};
    WfJob* jobs = nullptr;    // host mirror of the job table (max_jobs entries)
    uint32_t njobs = 0;
    bool owns_jobs = false;
    uint64_t total = 0;       // samples of all passes added
    void* buffer = nullptr;   // device memory of pool, queues, counters and job table
    bool owns_buffer = false;
    size_t buffer_bytes = 0;
    WfCounters* host_counters = nullptr;  // read-back target (pinned when the engine allocated it)
    bool owns_host_counters = false;

    // Bytes of device memory for `pool` slots and `max_jobs` passes.
    static size_t bytes_for(uint32_t pool, uint32_t max_jobs);
    // Allocates its own memory.
    cudaError_t create(int device, cudaStream_t stream, uint32_t pool, uint32_t max_jobs, int march_budget);
    // Uses caller-provided device memory (bytes_for) and host storage for the
    // counters and the job table (max_jobs entries); allocates nothing.
    cudaError_t attach(int device, cudaStream_t stream, uint32_t pool, uint32_t max_jobs, int march_budget,
                       void* device_buffer, size_t bytes, WfCounters* host_counters_storage, WfJob* host_jobs);
    void destroy();

    // Empties the pool and the job table (asynchronous, stream-ordered).
    cudaError_t reset();
    // Appends a pass; `job` is filled by the caller except first/count/finished/cam.
    cudaError_t add_pass(const WfJob& job, uint32_t* index);
    // Launches `n` iterations.
    cudaError_t run(int n, bool trace);
    // Reads the counters (synchronises the stream).
    cudaError_t read_counters(WfCounters* out);
    // Reads the finished-sample counts of passes [j0, j1) (synchronises the stream).
    cudaError_t read_finished(uint32_t j0, uint32_t j1, uint32_t* out);
    // Rendering/Accumulate of pass `j` into its accumulator.
    cudaError_t resolve(uint32_t j);
    // Runs until every pass added so far has finished (polling between chunks of
    // iterations), or `max_iterations` have run (returns cudaErrorTimeout then).
    cudaError_t drain(bool trace, uint64_t max_iterations);
};
