// pt_noalloc.cu — pt_dispatch_noalloc: one wavefront dispatch that allocates
// nothing.
//
// Some callers cannot allocate device memory when they render: a plug-in
// inside a host application that owns the GPU's memory budget and forbids
// allocations after start-up, or a real-time loop that cannot afford an
// allocator's latency or fragmentation.  This entry point takes the scene
// and push constants by host pointer and the accumulator as caller-owned
// device memory, and keeps all of its own working memory — the device copy
// of the scene, the CIE table, the path pool, the ray queues, the per-sample
// colours and the counters — in one file-scope __device__ array of fixed size
// (PT_NOALLOC_SCRATCH_BYTES = 32 MiB), which every GPU that loads the
// library holds until the process exits.
//
// In host code the array's name is only a host-side stand-in, so the first
// call on each device looks up its device address with cudaGetSymbolAddress
// (with that device current) and caches it (devices 0..63).  With lazy module
// loading (the CUDA default) that lookup is also what loads this file's
// module, so the first call on a device commits the array's 32 MiB; later
// calls allocate nothing, so make the first call a warm-up.  Every call
// shares the array and overwrites what it needs (the counters are reset,
// the colours and path slots are rewritten), so calls that overlap on the
// GPU race.  A per-device host lock is held for the whole
// call and each call returns only once its work on the stream is complete,
// so calls from several host threads run one after another.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/pt_cuda.h"
#include "kernel/pt_megakernel.h"
#include "kernel/pt_wavefront.h"
#include "pt_engine.h"

namespace {

constexpr size_t r256(size_t x) { return (x + 255) / 256 * 256; }

constexpr uint32_t kPool = PT_NOALLOC_POOL_SLOTS;
constexpr uint32_t kMaxSamples = PT_NOALLOC_MAX_SAMPLES;
// The engine's arrays for kPool slots and one pass (WfEngine::bytes_for).
constexpr size_t kEngineBytes =
    7 * r256((size_t)kPool * 32) + 7 * r256((size_t)kPool * 4) + r256(sizeof(WfCounters)) + r256(sizeof(WfJob));
constexpr size_t kSceneOff = 0;
constexpr size_t kCieOff = kSceneOff + r256(sizeof(KScene));
constexpr size_t kEngineOff = kCieOff + r256(sizeof(float) * PT_CIE_TABLE_SIZE);
constexpr size_t kColorsOff = kEngineOff + kEngineBytes;
constexpr size_t kScratchBytes = kColorsOff + r256((size_t)kMaxSamples * 16);
static_assert(kScratchBytes <= PT_NOALLOC_SCRATCH_BYTES, "PT_NOALLOC_SCRATCH_BYTES is too small");

}  // namespace

// The fixed working memory of pt_dispatch_noalloc (see the file comment).
static __device__ __align__(256) unsigned char pt_noalloc_scratch[PT_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch[kMaxDevices] = {};  // device address of pt_noalloc_scratch per device
std::mutex g_call[kMaxDevices];     // held for a whole call on that device

int scratch_address(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices) return PT_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, pt_noalloc_scratch);
        if (e != cudaSuccess || !p) return PT_ERR_CUDA;
        g_scratch[device] = p;
    }
    *out = static_cast<unsigned char*>(g_scratch[device]);
    return PT_OK;
}

bool valid_count(float v, int max, int* out) {
    if (!(v >= 0.0f) || v > (float)max || std::floor(v) != v) return false;
    *out = (int)v;
    return true;
}

// The launch-parameter image of the scene (as pt_upload_scene builds it),
// without rotation matrices (a kernel writes those into the device copy).
int build_scene(const pt_ubo* ubo, const pt_sdf_plugin* plugins, int nplug, KScene* S) {
    int n[7];
    const int caps[7] = {PT_MAX_OBJECTS_SIZE / 6, PT_MAX_OBJECTS_SIZE / 5, PT_MAX_OBJECTS_SIZE / 11,
                         PT_MAX_OBJECTS_SIZE / 12, PT_MAX_OBJECTS_SIZE / 16, PT_MAX_SDFS_SIZE / 6,
                         PT_MAX_LIGHTIDS_SIZE};
    for (int i = 0; i < 7; i++)
        if (!valid_count(ubo->numObjects[i], caps[i], &n[i])) return PT_ERR_INVALID;
    if (6 * n[0] + 5 * n[1] + 11 * n[2] + 12 * n[3] + 16 * n[4] > PT_MAX_OBJECTS_SIZE) return PT_ERR_INVALID;
    if (n[5] > PT_MAX_LIVE_SDFS || nplug > PT_MAX_LIVE_SDFS) return PT_ERR_UNSUPPORTED;
    for (int i = 0; i < nplug; i++) {
        if (plugins[i].kind == PT_SDF_CUSTOM) return PT_ERR_UNSUPPORTED;  // run-time compiled: pt_dispatch only
        if (plugins[i].kind < PT_SDF_NONE || plugins[i].kind > PT_SDF_TERRAIN) return PT_ERR_INVALID;
    }
    std::memset(S, 0, sizeof(KScene));
    std::memcpy(S->numObjects, ubo->numObjects, sizeof(S->numObjects));
    std::memcpy(S->objects, ubo->objects, sizeof(S->objects));
    std::memcpy(S->sdfs, ubo->sdfs, sizeof(S->sdfs));
    std::memcpy(S->materials, ubo->materials, sizeof(S->materials));
    std::memcpy(S->lights, ubo->lights, sizeof(S->lights));
    std::memcpy(S->lightIDs, ubo->lightIDs, sizeof(S->lightIDs));
    for (int i = 0; i < 7; i++) S->meta.n[i] = n[i];
    S->meta.offset[0] = 0;
    S->meta.offset[1] = 6 * n[0];
    S->meta.offset[2] = S->meta.offset[1] + 5 * n[1];
    S->meta.offset[3] = S->meta.offset[2] + 11 * n[2];
    S->meta.offset[4] = S->meta.offset[3] + 12 * n[3];
    S->meta.total_objects = n[0] + n[1] + n[2] + n[3] + n[4];
    if (nplug > 0) std::memcpy(S->plug, plugins, sizeof(pt_sdf_plugin) * (size_t)nplug);
    S->meta.nplug = nplug;
    return PT_OK;
}

#define PT_NA_TRY(call)                                 \
    do {                                                \
        if ((call) != cudaSuccess) return PT_ERR_CUDA; \
    } while (0)

}  // namespace

extern "C" int pt_dispatch_noalloc(const pt_ubo* ubo, const pt_sdf_plugin* plugins, int nplugins,
                                   const pt_push* push, float* d_accum, void* stream_ptr) {
    if (!ubo || !push || !d_accum || nplugins < 0 || (nplugins > 0 && !plugins)) return PT_ERR_INVALID;
    if (push->resolution[0] <= 0 || push->resolution[1] <= 0 || push->samplesPerFrame <= 0) return PT_ERR_INVALID;
    const uint64_t total64 = (uint64_t)push->resolution[0] * (uint64_t)push->resolution[1] *
                             (uint64_t)push->samplesPerFrame;
    if (total64 > kMaxSamples) return PT_ERR_TOO_LARGE;
    const uint32_t total = (uint32_t)total64;
    cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);

    // The scene image is built on the stack (about 19 KB): no heap use.
    KParams host_params;
    KScene& S = host_params.s;
    const int rc = build_scene(ubo, plugins, nplugins, &S);
    if (rc != PT_OK) return rc;

    int device = 0;
    PT_NA_TRY(cudaGetDevice(&device));
    if (device < 0 || device >= kMaxDevices) return PT_ERR_INVALID;
    std::lock_guard<std::mutex> call_lock(g_call[device]);
    unsigned char* base = nullptr;
    const int rs = scratch_address(device, &base);
    if (rs != PT_OK) return rs;
    KScene* d_scene = reinterpret_cast<KScene*>(base + kSceneOff);
    float* d_cie = reinterpret_cast<float*>(base + kCieOff);

    PT_NA_TRY(cudaMemcpyAsync(d_scene, &S, sizeof(KScene), cudaMemcpyHostToDevice, stream));
    PT_NA_TRY(cudaMemcpyAsync(d_cie, ubo->CIEXYZ1931, sizeof(float) * PT_CIE_TABLE_SIZE, cudaMemcpyHostToDevice,
                              stream));
    if (S.meta.total_objects > 0) PT_NA_TRY(ptk_rotation_setup(&S, &d_scene->rot[0][0], stream));

    if (push->pathLength <= 0) {
        // No bounce is traced: the megakernel needs no scratch beyond the CIE table.
        host_params.pc = *push;
        host_params.accum = reinterpret_cast<float4*>(d_accum);
        host_params.cie = d_cie;
        host_params.trace = KTrace{nullptr, nullptr, nullptr, 0};
        PT_NA_TRY(ptk_launch_megakernel(&host_params, false, stream));
        PT_NA_TRY(cudaStreamSynchronize(stream));
        return PT_OK;
    }

    // The wavefront engine on the fixed array, with host read-back storage on
    // the stack.
    if (WfEngine::bytes_for(kPool, 1) != kEngineBytes) return PT_ERR_INVALID;
    WfEngine engine;
    WfCounters counters;
    WfJob job_table[1];
    PT_NA_TRY(engine.attach(device, stream, total < kPool ? (total < 1024u ? 1024u : total) : kPool, 1, 64,
                            base + kEngineOff, kEngineBytes, &counters, job_table));
    // A mandelbulb marches with the warp-wide normal pass, as pt_dispatch does.
    bool bulb = false;
    for (int i = 0; i < nplugins; i++) bulb = bulb || plugins[i].kind == PT_SDF_MANDELBULB;
    engine.set_march_kernel(bulb ? ptk_wavefront_march_warp_normals() : nullptr);
    WfJob j;
    std::memset(&j, 0, sizeof j);
    j.scene = d_scene;
    j.cie = d_cie;
    j.accum = reinterpret_cast<float4*>(d_accum);
    j.colors = reinterpret_cast<float4*>(base + kColorsOff);
    j.pc = *push;
    uint32_t idx = 0;
    PT_NA_TRY(engine.add_pass(j, &idx));
    const uint64_t march_iters = 512ull / 64ull + 2;
    const uint64_t max_iter =
        ((uint64_t)total / engine.pool + 2) * (2ull * (uint64_t)push->pathLength + 3) * march_iters + 16;
    const cudaError_t e = engine.drain(false, max_iter);
    if (e == cudaErrorTimeout) return PT_ERR_KERNEL;
    PT_NA_TRY(e);
    PT_NA_TRY(engine.resolve(idx));
    PT_NA_TRY(cudaStreamSynchronize(stream));
    return PT_OK;
}
