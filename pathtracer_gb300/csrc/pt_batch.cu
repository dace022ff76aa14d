// pt_batch.cu — batched rendering (include/pt_cuda.h, pt_batch_*).
//
// Many render passes — different scenes, resolutions and sample counts —
// share the device: passes can be added while others are in flight, every
// launch mixes the paths of many passes, and each pass is resolved
// into its target as soon as its last sample finishes (passes of one target
// in the order they were added, so a progressive series accumulates exactly
// as dispatches would).  Scenes and targets stay resident on the device, so a
// job is refined one pass at a time without re-uploading anything.
//
// Two engines share the work (pt_engine.h): passes of scenes with SDFs go to
// the staged wavefront kernels, whose compacted queues keep lanes marching
// together; passes of analytic-only scenes go to the persistent path kernel,
// which keeps every path in registers.  Each engine runs on its own stream,
// so the two kinds of work overlap on the device; resolution runs on the
// batch's stream.
//
// A target is either the reference's float accumulator (Rendering/Accumulate,
// src/shader.comp:1492-1523, bit-identical to pt_dispatch) or an FP64 sum of
// every sample's exposed XYZ, used for high-sample-count reference images:
// FP32 paths, FP64 accumulation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <deque>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/pt_cuda.h"
#include "kernel/pt_features.h"
#include "kernel/pt_megakernel.h"
#include "pt_engine.h"
#include "pt_jit.h"

namespace {

struct BatchScene {
    KScene* d_scene = nullptr;
    std::shared_ptr<KScene> h_scene;  // host copy (rotation matrices and extensions included), for the
                                      // persistent kernel's single-pass launches
    float* d_cie = nullptr;
    bool live = false;
    bool has_sdf = false;
    bool custom = false;        // holds run-time compiled snippets (staged engine only)
    int variant = PT_FEAT_ALL;  // primitive classes present (pt_features.h)
    uint32_t passes_in_flight = 0;
};

struct BatchTarget {
    float4* d_accum = nullptr;  // PT_TARGET_FLOAT
    double* d_sum = nullptr;    // PT_TARGET_FP64: x, y, z, samples per pixel
    int width = 0, height = 0;
    int kind = PT_TARGET_FLOAT;
    bool live = false;
    uint32_t passes_in_flight = 0;
    uint64_t samples = 0;  // resolved samples per pixel
};

struct RmseItem {
    const float4* a;         // image
    const float4* ref;       // float reference, or
    const double* ref_sum;   // FP64 sums (x, y, z, samples) per pixel
    uint32_t n;              // pixels
    uint32_t pad;
};

struct BatchPass {
    int scene = -1, target = -1;
    int engine = 0;     // kStaged or kPersistent
    uint32_t eidx = 0;  // pass number within its engine's ring
    // A large staged pass is split in two: samples [0, count0) on kStaged,
    // [count0, count) on kStaged2 (engine2 = kStaged2, ring entry eidx2).
    int engine2 = -1;
    uint32_t eidx2 = 0;
    uint32_t count0 = 0;
    bool part_finished[2] = {false, false};
    float4* d_colors = nullptr;
    uint32_t count = 0;
    uint32_t spf = 0;
    bool finished = false;  // every sample has its colour
    bool done = false;      // resolved
};

constexpr int kStaged = 0, kPersistent = 1, kStaged2 = 2;
constexpr int kEngines = 3;

}  // namespace

struct pt_batch {
    int device = 0;
    cudaStream_t stream = nullptr;       // resolution, uploads, allocation
    cudaStream_t estream[kEngines] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev = nullptr;            // orders engine work after the batch stream
    cudaMemPool_t mempool = nullptr;     // colour buffers and targets; keeps freed memory mapped
    WfEngine engine[kEngines];           // kStaged, kPersistent, kStaged2
    bool engine_live[kEngines] = {false, false, false};
    std::deque<uint32_t> eorder[kEngines];  // batch pass ids of each engine's ring, from its lo
    // Staged engines a large staged pass is split between (pt_batch_set_wavefront_engines).
    int staged_engines = 2;
    uint32_t pool_slots = 0, max_passes = 0;
    int route = PT_BATCH_ROUTE_AUTO;
    int march_budget = 64;
    int persist_refill = 16;
    bool device_checks = false;  // both engines on the checked kernel build (pt_batch_set_device_checks)
    std::vector<BatchScene> scenes;
    std::vector<BatchTarget> targets;
    std::deque<BatchPass> passes;  // indexed by pass id - pass_base
    uint32_t pass_base = 0;        // pass id of passes[0]
    uint32_t next_pass = 0;
    uint64_t samples_added = 0;
    uint64_t samples_done = 0;
    uint64_t iterations = 0;
    uint64_t kernel_launches = 0;  // the batch's own kernels (the engines count theirs)
    uint32_t* h_finished = nullptr;  // pinned, max_passes entries
    // RMSE reductions: per item, sum of squared differences and sum of squares.
    int rmse_cap = 0;
    struct RmseItem* h_items = nullptr;  // pinned
    struct RmseItem* d_items = nullptr;
    double2* d_partial = nullptr;  // kRmseBlocks per item
    double2* d_rmse = nullptr;
    double2* h_rmse = nullptr;     // pinned
    std::vector<char> blocked;       // per target, scratch of pt_batch_step
    // Run-time compiled SDF snippets of every scene added with sources, numbered
    // across the batch (a scene's slot i is snippet custom_base + i), and the
    // march kernel compiled for all of them (rebuilt before the next step
    // after a scene brought new ones).
    std::vector<JitSlot> custom;
    int custom_next = 0;
    JitModule jit;
    bool jit_dirty = false;
    uint32_t sdf_kinds = 0;  // plug-in kinds of every scene added (bit k: kind k)
    uint32_t jit_kinds = 0;  // the kinds `jit` was compiled for (PT_SDF_KINDS)
    JitModule jit64;  // the FP64 renderer's megakernel for the same snippets (pt_batch_render_fp64), when needed
    // A scene with a mandelbulb was added: the staged engine's built-in march
    // kernel then probes normals across the warp.
    bool bulb = false;
    std::string err;
};

namespace {

int bfail(pt_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    return code;
}

int bcuda(pt_batch* b, cudaError_t e, const char* what) {
    return bfail(b, e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA,
                 std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

#define PT_B_TRY(b, call)                                  \
    do {                                                   \
        const cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) return bcuda(b, e_, #call); \
    } while (0)

bool count_ok(float v, int max, int* out) {
    if (!(v >= 0.0f) || v > (float)max || std::floor(v) != v) return false;
    *out = (int)v;
    return true;
}

BatchPass* pass_at(pt_batch* b, uint32_t j) {
    if (j < b->pass_base || j - b->pass_base >= b->passes.size()) return nullptr;
    return &b->passes[j - b->pass_base];
}

// The staged engine's march kernel: the batch's run-time compiled one, else
// the built-in one with the warp-wide normal pass when a mandelbulb is in
// the batch, else the default built-in one (null).
const void* staged_march_kernel(const pt_batch* b) {
    if (b->jit.lib) return reinterpret_cast<const void*>(b->jit.kernel[0]);
    return b->bulb ? ptk_wavefront_kernels(b->device_checks)->march_warp_normals() : nullptr;
}

// Creates engine e on first use: a staged engine with the batch's pool,
// the persistent engine with the smallest pool (it keeps paths in registers).
cudaError_t ensure_engine(pt_batch* b, int e) {
    if (b->engine_live[e]) return cudaSuccess;
    if (!b->estream[e]) {
        const cudaError_t r = cudaStreamCreateWithFlags(&b->estream[e], cudaStreamNonBlocking);
        if (r != cudaSuccess) return r;
    }
    const uint32_t pool = e == kPersistent ? 1024u : b->pool_slots;
    const cudaError_t r = b->engine[e].create(b->device, b->estream[e], pool, b->max_passes, b->march_budget);
    if (r != cudaSuccess) {
        b->engine[e].destroy();
        return r;
    }
    b->engine[e].set_persistent(e == kPersistent);
    b->engine[e].args.persist_refill = b->persist_refill;
    b->engine[e].set_checks(b->device_checks);
    if (e != kPersistent) b->engine[e].set_march_kernel(staged_march_kernel(b));
    b->engine_live[e] = true;
    return cudaSuccess;
}

// Sets the march kernel of every live staged engine.
void set_staged_march_kernel(pt_batch* b, const void* kernel) {
    for (int e : {kStaged, kStaged2})
        if (b->engine_live[e]) b->engine[e].set_march_kernel(kernel);
}

// FP64 target: adds the pass's exposed sample colours (Rendering's exposure
// factor apertureSize^2 * ISO, src/shader.comp:1517) to the per-pixel sums.
__global__ void resolve_fp64_kernel(const float4* __restrict__ colors, uint32_t npix, int spf, double exposure,
                                    double* __restrict__ sum) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    double x = 0.0, y = 0.0, z = 0.0;
    for (int k = 0; k < spf; k++) {
        const float4 c = colors[(size_t)k * npix + pix];
        x += c.x;
        y += c.y;
        z += c.z;
    }
    double* s = sum + 4 * (size_t)pix;
    s[0] += x * exposure;
    s[1] += y * exposure;
    s[2] += z * exposure;
    s[3] += (double)spf;
}

__global__ void fp64_to_float_kernel(const double* __restrict__ sum, uint32_t npix, float4* __restrict__ out) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    const double* s = sum + 4 * (size_t)pix;
    const double inv = s[3] > 0.0 ? 1.0 / s[3] : 0.0;
    out[pix] = make_float4((float)(s[0] * inv), (float)(s[1] * inv), (float)(s[2] * inv), 1.0f);
}

// Per item (blockIdx.y): sums of squared differences and squared reference
// values over the XYZ channels of an image against a reference given as
// floats or as FP64 sums (divided by their sample count).  Each block writes
// its partial sums; rmse_final adds them in a fixed order, so the result is
// the same bits on every run.
constexpr int kRmseBlocks = 64, kRmseThreads = 256;

__global__ void __launch_bounds__(kRmseThreads) rmse_partial(const RmseItem* __restrict__ items,
                                                             double2* __restrict__ partial) {
    const RmseItem it = items[blockIdx.y];
    double d2 = 0.0, r2 = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < it.n; i += gridDim.x * blockDim.x) {
        const float4 x = it.a[i];
        double rx, ry, rz;
        if (it.ref_sum) {
            const double* s = it.ref_sum + 4 * (size_t)i;
            const double inv = s[3] > 0.0 ? 1.0 / s[3] : 0.0;
            rx = s[0] * inv;
            ry = s[1] * inv;
            rz = s[2] * inv;
        } else {
            const float4 r = it.ref[i];
            rx = r.x;
            ry = r.y;
            rz = r.z;
        }
        const double dx = (double)x.x - rx, dy = (double)x.y - ry, dz = (double)x.z - rz;
        d2 += dx * dx + dy * dy + dz * dz;
        r2 += rx * rx + ry * ry + rz * rz;
    }
    for (int o = 16; o > 0; o >>= 1) {
        d2 += __shfl_down_sync(0xffffffffu, d2, o);
        r2 += __shfl_down_sync(0xffffffffu, r2, o);
    }
    __shared__ double2 warp_sums[kRmseThreads / 32];
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = make_double2(d2, r2);
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 t = warp_sums[0];
        for (int w = 1; w < kRmseThreads / 32; w++) {
            t.x += warp_sums[w].x;
            t.y += warp_sums[w].y;
        }
        partial[blockIdx.y * kRmseBlocks + blockIdx.x] = t;
    }
}

// One warp per item: the block partials in a fixed order.
__global__ void rmse_final(const double2* __restrict__ partial, double2* __restrict__ out) {
    const int lane = (int)threadIdx.x;
    double d2 = 0.0, r2 = 0.0;
    for (int k = lane; k < kRmseBlocks; k += 32) {
        d2 += partial[blockIdx.x * kRmseBlocks + k].x;
        r2 += partial[blockIdx.x * kRmseBlocks + k].y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        d2 += __shfl_down_sync(0xffffffffu, d2, o);
        r2 += __shfl_down_sync(0xffffffffu, r2, o);
    }
    if (lane == 0) out[blockIdx.x] = make_double2(d2, r2);
}

int check_target(pt_batch* b, int target_id, const char* what) {
    if (target_id < 0 || target_id >= (int)b->targets.size() || !b->targets[(size_t)target_id].live)
        return bfail(b, PT_ERR_INVALID, std::string(what) + ": unknown or released target");
    return PT_OK;
}

void free_rmse(pt_batch* b) {
    if (b->h_items) cudaFreeHost(b->h_items);
    if (b->d_items) cudaFree(b->d_items);
    if (b->d_partial) cudaFree(b->d_partial);
    if (b->d_rmse) cudaFree(b->d_rmse);
    if (b->h_rmse) cudaFreeHost(b->h_rmse);
    b->h_items = b->d_items = nullptr;
    b->d_partial = b->d_rmse = b->h_rmse = nullptr;
    b->rmse_cap = 0;
}

cudaError_t reserve_rmse(pt_batch* b, int n) {
    if (n <= b->rmse_cap) return cudaSuccess;
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return e;
    free_rmse(b);
    int cap = 64;
    while (cap < n) cap *= 2;
    e = cudaMallocHost(&b->h_items, sizeof(RmseItem) * (size_t)cap);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_items, sizeof(RmseItem) * (size_t)cap);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_partial, sizeof(double2) * kRmseBlocks * (size_t)cap);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_rmse, sizeof(double2) * (size_t)cap);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_rmse, sizeof(double2) * (size_t)cap);
    if (e != cudaSuccess) {
        free_rmse(b);
        return e;
    }
    b->rmse_cap = cap;
    return cudaSuccess;
}

// Relative RMSE of items [0, n) of b->h_items: one launch, one copy back.
int run_rmse(pt_batch* b, int n, double* out) {
    if (n == 0) return PT_OK;
    PT_B_TRY(b, cudaMemcpyAsync(b->d_items, b->h_items, sizeof(RmseItem) * (size_t)n, cudaMemcpyHostToDevice,
                                b->stream));
    rmse_partial<<<dim3(kRmseBlocks, (unsigned)n), kRmseThreads, 0, b->stream>>>(b->d_items, b->d_partial);
    b->kernel_launches += 2;
    PT_B_TRY(b, cudaGetLastError());
    rmse_final<<<(unsigned)n, 32, 0, b->stream>>>(b->d_partial, b->d_rmse);
    PT_B_TRY(b, cudaGetLastError());
    PT_B_TRY(b, cudaMemcpyAsync(b->h_rmse, b->d_rmse, sizeof(double2) * (size_t)n, cudaMemcpyDeviceToHost,
                                b->stream));
    PT_B_TRY(b, cudaStreamSynchronize(b->stream));
    for (int i = 0; i < n; i++)
        out[i] = (b->h_rmse[i].y > 0.0) ? std::sqrt(b->h_rmse[i].x / b->h_rmse[i].y) : 0.0;
    return PT_OK;
}

}  // namespace

extern "C" {

int pt_batch_create(pt_batch** out, int device, uint32_t pool_slots, uint32_t max_passes) {
    if (!out || pool_slots < 1024 || max_passes < 1 || max_passes > (1u << 20)) return PT_ERR_INVALID;
    *out = nullptr;
    pt_batch* b = new (std::nothrow) pt_batch();
    if (!b) return PT_ERR_OOM;
    b->device = device;
    b->pool_slots = pool_slots;
    b->max_passes = max_passes;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming);
    if (e == cudaSuccess) {
        // A pool of its own: freed colour buffers stay mapped for the next
        // passes instead of going back to the driver at every synchronisation.
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        e = cudaMemPoolCreate(&b->mempool, &props);
        if (e == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            e = cudaMemPoolSetAttribute(b->mempool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_finished, sizeof(uint32_t) * max_passes);
    if (e != cudaSuccess) {
        pt_batch_destroy(b);
        return e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA;
    }
    *out = b;
    return PT_OK;
}

int pt_batch_destroy(pt_batch* b) {
    if (!b) return PT_ERR_INVALID;
    cudaSetDevice(b->device);
    for (int e = 0; e < kEngines; e++)
        if (b->estream[e]) cudaStreamSynchronize(b->estream[e]);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto& s : b->scenes) {
        if (s.d_scene) cudaFree(s.d_scene);
        if (s.d_cie) cudaFree(s.d_cie);
    }
    for (auto& t : b->targets) {
        if (t.d_accum) cudaFreeAsync(t.d_accum, b->stream);
        if (t.d_sum) cudaFreeAsync(t.d_sum, b->stream);
    }
    for (auto& p : b->passes)
        if (p.d_colors) cudaFreeAsync(p.d_colors, b->stream);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (int e = 0; e < kEngines; e++) {
        b->engine[e].destroy();
        if (b->estream[e]) cudaStreamDestroy(b->estream[e]);
    }
    if (b->ev) cudaEventDestroy(b->ev);
    if (b->mempool) cudaMemPoolDestroy(b->mempool);
    if (b->h_finished) cudaFreeHost(b->h_finished);
    free_rmse(b);
    pt_jit_unload(b->jit);
    pt_jit_unload(b->jit64);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return PT_OK;
}

const char* pt_batch_last_error(pt_batch* b) { return b ? b->err.c_str() : "null batch"; }

void* pt_batch_stream(pt_batch* b) { return b ? (void*)b->stream : nullptr; }

int pt_batch_set_march_budget(pt_batch* b, int steps) {
    if (!b) return PT_ERR_INVALID;
    if (steps < 1 || steps > 512) return bfail(b, PT_ERR_INVALID, "pt_batch_set_march_budget: 1..512 steps");
    b->march_budget = steps;
    for (int e = 0; e < kEngines; e++) b->engine[e].set_march_budget(steps);
    return PT_OK;
}

int pt_batch_set_persist_refill(pt_batch* b, int lanes) {
    if (!b) return PT_ERR_INVALID;
    if (lanes < 1 || lanes > 32) return bfail(b, PT_ERR_INVALID, "pt_batch_set_persist_refill: 1..32 lanes");
    b->persist_refill = lanes;
    for (int e = 0; e < kEngines; e++) b->engine[e].args.persist_refill = lanes;
    return PT_OK;
}

int pt_batch_set_wavefront_engines(pt_batch* b, int engines) {
    if (!b) return PT_ERR_INVALID;
    if (engines != 1 && engines != 2) return bfail(b, PT_ERR_INVALID, "pt_batch_set_wavefront_engines: 1 or 2 engines");
    b->staged_engines = engines;
    return PT_OK;
}

int pt_batch_set_route(pt_batch* b, int route) {
    if (!b) return PT_ERR_INVALID;
    if (route != PT_BATCH_ROUTE_AUTO && route != PT_BATCH_ROUTE_STAGED && route != PT_BATCH_ROUTE_PERSISTENT)
        return bfail(b, PT_ERR_INVALID, "pt_batch_set_route: unknown route");
    b->route = route;
    return PT_OK;
}

}  // extern "C"

namespace {

// The scene's device copy; plug-ins of kind PT_SDF_CUSTOM are snippets
// custom_base + slot of the batch's compiled march kernel.
int add_scene(pt_batch* b, const pt_ubo* ubo, const pt_sdf_plugin* plugins, int nplugins, int custom_base,
              int* scene_id) {
    int n[7];
    const int caps[7] = {PT_MAX_OBJECTS_SIZE / 6, PT_MAX_OBJECTS_SIZE / 5, PT_MAX_OBJECTS_SIZE / 11,
                         PT_MAX_OBJECTS_SIZE / 12, PT_MAX_OBJECTS_SIZE / 16, PT_MAX_SDFS_SIZE / 6,
                         PT_MAX_LIGHTIDS_SIZE};
    for (int i = 0; i < 7; i++)
        if (!count_ok(ubo->numObjects[i], caps[i], &n[i]))
            return bfail(b, PT_ERR_INVALID,
                         "pt_batch_add_scene: numObjects[" + std::to_string(i) + "] is not a valid count");
    if (6 * n[0] + 5 * n[1] + 11 * n[2] + 12 * n[3] + 16 * n[4] > PT_MAX_OBJECTS_SIZE)
        return bfail(b, PT_ERR_INVALID, "pt_batch_add_scene: objects overflow the 1024-float object array");
    if (n[5] > PT_MAX_LIVE_SDFS || nplugins > PT_MAX_LIVE_SDFS)
        return bfail(b, PT_ERR_UNSUPPORTED, "pt_batch_add_scene: at most 32 SDFs can be evaluated (32-bit set mask)");
    bool custom = false, bulb = false;
    uint32_t kinds = 0;
    for (int i = 0; i < nplugins; i++) {
        if (plugins[i].kind < PT_SDF_NONE || plugins[i].kind > PT_SDF_CUSTOM)
            return bfail(b, PT_ERR_INVALID, "pt_batch_add_scene: unknown plug-in kind");
        custom = custom || plugins[i].kind == PT_SDF_CUSTOM;
        bulb = bulb || plugins[i].kind == PT_SDF_MANDELBULB;
        kinds |= 1u << plugins[i].kind;
    }
    PT_B_TRY(b, cudaSetDevice(b->device));
    KScene* S = new (std::nothrow) KScene;
    if (!S) return bfail(b, PT_ERR_OOM, "pt_batch_add_scene: out of host memory");
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
    if (nplugins > 0) std::memcpy(S->plug, plugins, sizeof(pt_sdf_plugin) * (size_t)nplugins);
    S->meta.nplug = nplugins;
    S->meta.custom_base = custom_base;
    BatchScene bs;
    cudaError_t e = cudaMalloc(&bs.d_scene, sizeof(KScene));
    if (e == cudaSuccess) e = cudaMalloc(&bs.d_cie, sizeof(float) * PT_CIE_TABLE_SIZE);
    if (e == cudaSuccess) e = cudaMemcpyAsync(bs.d_scene, S, sizeof(KScene), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(bs.d_cie, ubo->CIEXYZ1931, sizeof(float) * PT_CIE_TABLE_SIZE, cudaMemcpyHostToDevice,
                            b->stream);
    // Rotation matrices straight into the device copy (same kernel as pt_upload_scene).
    if (e == cudaSuccess && S->meta.total_objects > 0) {
        e = ptk_rotation_setup(S, &bs.d_scene->rot[0][0], b->stream);
        b->kernel_launches += 1;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);  // the copies read S and ubo
    // keep S as the host copy, with the rotation matrices the device derived
    if (e == cudaSuccess && S->meta.total_objects > 0)
        e = cudaMemcpy(&S->rot[0][0], &bs.d_scene->rot[0][0], sizeof(S->rot), cudaMemcpyDeviceToHost);
    bs.h_scene.reset(S);
    if (e != cudaSuccess) {
        if (bs.d_scene) cudaFree(bs.d_scene);
        if (bs.d_cie) cudaFree(bs.d_cie);
        return bcuda(b, e, "pt_batch_add_scene");
    }
    bs.live = true;
    bs.has_sdf = n[5] > 0;
    bs.custom = custom;
    bs.variant = pt_feature_variant(n);
    b->bulb = b->bulb || bulb;
    // the compiled march kernel holds the code of the kinds seen so far: a
    // scene with another kind needs it compiled again
    b->sdf_kinds |= kinds;
    if (b->jit.lib && (kinds & ~b->jit_kinds)) b->jit_dirty = true;
    *scene_id = (int)b->scenes.size();
    b->scenes.push_back(bs);
    return PT_OK;
}

}  // namespace

extern "C" {

int pt_batch_add_target(pt_batch* b, int width, int height, int kind, int* target_id) {
    if (!b) return PT_ERR_INVALID;
    if (!target_id || width <= 0 || height <= 0 || (long long)width * height > (1ll << 30) ||
        (kind != PT_TARGET_FLOAT && kind != PT_TARGET_FP64))
        return bfail(b, PT_ERR_INVALID, "pt_batch_add_target: bad arguments");
    PT_B_TRY(b, cudaSetDevice(b->device));
    BatchTarget t;
    const size_t npix = (size_t)width * (size_t)height;
    t.width = width;
    t.height = height;
    t.kind = kind;
    if (kind == PT_TARGET_FLOAT) {
        PT_B_TRY(b, cudaMallocFromPoolAsync(&t.d_accum, npix * sizeof(float4), b->mempool, b->stream));
        PT_B_TRY(b, cudaMemsetAsync(t.d_accum, 0, npix * sizeof(float4), b->stream));
    } else {
        PT_B_TRY(b, cudaMallocFromPoolAsync(&t.d_sum, npix * 4 * sizeof(double), b->mempool, b->stream));
        PT_B_TRY(b, cudaMemsetAsync(t.d_sum, 0, npix * 4 * sizeof(double), b->stream));
    }
    t.live = true;
    *target_id = (int)b->targets.size();
    b->targets.push_back(t);
    b->blocked.push_back(0);
    return PT_OK;
}

void* pt_batch_target_device_ptr(pt_batch* b, int target_id) {
    if (!b || target_id < 0 || target_id >= (int)b->targets.size()) return nullptr;
    const BatchTarget& t = b->targets[(size_t)target_id];
    return t.kind == PT_TARGET_FLOAT ? (void*)t.d_accum : (void*)t.d_sum;
}

int pt_batch_add_scene(pt_batch* b, const pt_ubo* ubo, const pt_sdf_plugin* plugins, int nplugins, int* scene_id) {
    if (!b) return PT_ERR_INVALID;
    if (!ubo || !scene_id || nplugins < 0 || (nplugins > 0 && !plugins))
        return bfail(b, PT_ERR_INVALID, "pt_batch_add_scene: bad arguments");
    for (int i = 0; i < nplugins; i++)
        if (plugins[i].kind == PT_SDF_CUSTOM)
            return bfail(b, PT_ERR_UNSUPPORTED,
                         "pt_batch_add_scene: run-time compiled SDFs need their text (pt_batch_add_scene_sources)");
    return add_scene(b, ubo, plugins, nplugins, 0, scene_id);
}

int pt_batch_add_scene_sources(pt_batch* b, const pt_ubo* ubo, const char* const* sources, int n, int* scene_id) {
    if (!b) return PT_ERR_INVALID;
    if (!ubo || !scene_id || n < 0 || (n > 0 && !sources))
        return bfail(b, PT_ERR_INVALID, "pt_batch_add_scene_sources: bad arguments");
    if (n > PT_MAX_LIVE_SDFS)
        return bfail(b, PT_ERR_UNSUPPORTED, "pt_batch_add_scene_sources: at most 32 SDFs can be evaluated");
    pt_sdf_plugin plug[PT_MAX_LIVE_SDFS];
    std::vector<JitSlot> added;
    const int base = b->custom_next;
    for (int i = 0; i < n; i++) {
        if (!sources[i]) return bfail(b, PT_ERR_INVALID, "pt_batch_add_scene_sources: null source");
        if (pt_parse_sdf_source(sources[i], &plug[i]) == PT_OK) continue;
        JitSlot j;
        std::string why;
        const int rc = pt_jit_translate_slot(sources[i], base + i, j, why);
        if (rc != PT_OK) return bfail(b, rc, "pt_batch_add_scene_sources: SDF " + std::to_string(i) + ": " + why);
        plug[i] = pt_sdf_plugin{PT_SDF_CUSTOM, PT_SDFMAT_DEFAULT, {0.0f, 0.0f, 0.0f}};
        added.push_back(j);
    }
    const int rc = add_scene(b, ubo, plug, n, added.empty() ? 0 : base, scene_id);
    if (rc != PT_OK) return rc;
    if (!added.empty()) {
        b->custom.insert(b->custom.end(), added.begin(), added.end());
        b->custom_next = base + n;
        b->jit_dirty = true;
    }
    return PT_OK;
}

int pt_batch_add_pass(pt_batch* b, int scene_id, int target_id, const pt_push* push, int* pass_id) {
    if (!b) return PT_ERR_INVALID;
    if (!push || !pass_id) return bfail(b, PT_ERR_INVALID, "pt_batch_add_pass: bad arguments");
    if (scene_id < 0 || scene_id >= (int)b->scenes.size() || !b->scenes[(size_t)scene_id].live)
        return bfail(b, PT_ERR_INVALID, "pt_batch_add_pass: unknown or released scene");
    if (check_target(b, target_id, "pt_batch_add_pass") != PT_OK) return PT_ERR_INVALID;
    BatchTarget& t = b->targets[(size_t)target_id];
    if (push->resolution[0] != t.width || push->resolution[1] != t.height)
        return bfail(b, PT_ERR_INVALID, "pt_batch_add_pass: resolution differs from the target's");
    if (push->samplesPerFrame <= 0 || push->pathLength <= 0)
        return bfail(b, PT_ERR_INVALID, "pt_batch_add_pass: samplesPerFrame and pathLength must be positive");
    const uint64_t count = (uint64_t)t.width * (uint64_t)t.height * (uint64_t)push->samplesPerFrame;
    if (count >= (1ull << 32)) return bfail(b, PT_ERR_INVALID, "pt_batch_add_pass: more than 2^32 samples in a pass");
    const BatchScene& sc = b->scenes[(size_t)scene_id];
    const int e = b->route == PT_BATCH_ROUTE_STAGED       ? kStaged
                  : b->route == PT_BATCH_ROUTE_PERSISTENT ? kPersistent
                  : (sc.has_sdf ? kStaged : kPersistent);
    if (e == kPersistent && sc.custom && sc.has_sdf)
        return bfail(b, PT_ERR_UNSUPPORTED,
                     "pt_batch_add_pass: scenes with run-time compiled SDFs render on the staged engine");
    PT_B_TRY(b, cudaSetDevice(b->device));
    PT_B_TRY(b, ensure_engine(b, e));
    WfEngine& E = b->engine[e];
    if (E.njobs - E.lo >= E.max_jobs)
        return bfail(b, PT_ERR_BUSY, "pt_batch_add_pass: every pass slot is in flight; step the batch first");
    // A staged pass of at least two pools' worth of samples per engine is
    // split in two halves (in sample order) between two staged engines on
    // two streams: one engine's kernels fill the SMs the other's leave idle.
    const bool split = e == kStaged && b->staged_engines == 2 && count >= 4ull * b->pool_slots;
    if (split) {
        PT_B_TRY(b, ensure_engine(b, kStaged2));
        const WfEngine& E2 = b->engine[kStaged2];
        if (E2.njobs - E2.lo >= E2.max_jobs)
            return bfail(b, PT_ERR_BUSY, "pt_batch_add_pass: every pass slot is in flight; step the batch first");
    }
    BatchPass p;
    p.scene = scene_id;
    p.target = target_id;
    p.engine = e;
    p.count = (uint32_t)count;
    p.count0 = split ? (uint32_t)(count / 2) : (uint32_t)count;
    p.spf = (uint32_t)push->samplesPerFrame;
    // Allocated on the batch stream; engine streams wait for it in pt_batch_step.
    PT_B_TRY(b, cudaMallocFromPoolAsync(&p.d_colors, count * sizeof(float4), b->mempool, b->stream));
    WfJob j;
    std::memset(&j, 0, sizeof j);
    j.scene = sc.d_scene;
    j.cie = sc.d_cie;
    j.accum = t.d_accum;  // null for FP64 targets, which resolve here instead
    j.colors = p.d_colors;
    j.pc = *push;
    j.variant = sc.variant;
    j.host_scene = e == kPersistent ? sc.h_scene.get() : nullptr;
    const cudaError_t r = E.add_pass_part(j, 0, p.count0, &p.eidx);
    if (r != cudaSuccess) {
        cudaFreeAsync(p.d_colors, b->stream);
        return bcuda(b, r, "pt_batch_add_pass");
    }
    if (split) {
        p.engine2 = kStaged2;
        // The first half is in the ring already: should this launch fail (a
        // lost context), the colour buffer is kept rather than freed under it.
        const cudaError_t r2 = b->engine[kStaged2].add_pass_part(j, p.count0, p.count - p.count0, &p.eidx2);
        if (r2 != cudaSuccess) return bcuda(b, r2, "pt_batch_add_pass");
    }
    const uint32_t id = b->next_pass++;
    if (b->passes.empty()) b->pass_base = id;
    b->passes.push_back(p);
    b->eorder[e].push_back(id);
    if (split) b->eorder[kStaged2].push_back(id);
    t.passes_in_flight++;
    b->scenes[(size_t)scene_id].passes_in_flight++;
    b->samples_added += count;
    *pass_id = (int)id;
    return PT_OK;
}

// Runs `iterations` iterations of each engine that has passes in flight,
// then resolves every pass whose samples have all finished (and whose
// earlier passes into the same target are resolved) and reports their ids:
// at most `capacity`, the rest are reported by later calls.
}  // extern "C"

namespace {

// Compiles the march kernel for every snippet the batch holds, if scenes
// brought new ones since the last compile, and hands it to the staged engine.
int prepare_jit(pt_batch* b) {
    if (!b->jit_dirty) return PT_OK;
    const uint32_t kinds = b->sdf_kinds;
    const std::string program = std::string(b->device_checks ? "#define PT_DEBUG_CHECKS 1\n" : "") +
                                "#define PT_SDF_KINDS " + std::to_string(kinds) + "u\n" +
                                pt_jit_program(b->custom, kJitMarch);
    std::vector<char> cubin;
    std::string lowered[kJitMaxKernels], log;
    JitModule m;
    int rc = pt_jit_compile(b->device, program, kJitMarch, cubin, lowered, log);
    if (rc != PT_OK) return bfail(b, rc, "compiling the batch's SDF snippets: " + log);
    rc = pt_jit_load(cubin, kJitMarch, lowered, m, log);
    if (rc != PT_OK) return bfail(b, rc, log);
    m.key = program;
    for (int se : {kStaged, kStaged2}) {
        if (!b->estream[se]) continue;
        const cudaError_t e = cudaStreamSynchronize(b->estream[se]);  // the old module's launches
        if (e != cudaSuccess) {
            pt_jit_unload(m);
            return bcuda(b, e, "pt_batch_step");
        }
    }
    set_staged_march_kernel(b, reinterpret_cast<const void*>(m.kernel[0]));
    pt_jit_unload(b->jit);
    b->jit = m;
    b->jit_kinds = kinds;
    b->jit_dirty = false;
    return PT_OK;
}

// The FP64 renderer's megakernel for every snippet the batch holds, compiled
// again when scenes brought new ones since the last compile.
int prepare_jit64(pt_batch* b) {
    const std::string program = pt_jit_program(b->custom, kJitFp64);
    if (b->jit64.lib && b->jit64.key == program) return PT_OK;
    std::vector<char> cubin;
    std::string lowered[kJitMaxKernels], log;
    JitModule m;
    int rc = pt_jit_compile(b->device, program, kJitFp64, cubin, lowered, log);
    if (rc != PT_OK) return bfail(b, rc, "compiling the batch's SDF snippets in double: " + log);
    rc = pt_jit_load(cubin, kJitFp64, lowered, m, log);
    if (rc != PT_OK) return bfail(b, rc, log);
    m.key = program;
    PT_B_TRY(b, cudaStreamSynchronize(b->stream));  // the old module's launches
    pt_jit_unload(b->jit64);
    b->jit64 = m;
    return PT_OK;
}

}  // namespace

extern "C" {

int pt_batch_step(pt_batch* b, int iterations, int* completed, int capacity, int* ncompleted) {
    if (!b) return PT_ERR_INVALID;
    if (iterations < 0 || capacity < 0 || (capacity > 0 && !completed) || !ncompleted)
        return bfail(b, PT_ERR_INVALID, "pt_batch_step: bad arguments");
    *ncompleted = 0;
    PT_B_TRY(b, cudaSetDevice(b->device));
    const int jr = prepare_jit(b);
    if (jr != PT_OK) return jr;
    for (int se : {kStaged, kStaged2})
        if (b->engine_live[se] && b->engine[se].march_kernel != staged_march_kernel(b)) {
            // a mandelbulb scene arrived: no launch of the old kernel may be in flight
            PT_B_TRY(b, cudaStreamSynchronize(b->estream[se]));
            b->engine[se].set_march_kernel(staged_march_kernel(b));
        }
    bool busy[kEngines];
    bool any = false;
    for (int e = 0; e < kEngines; e++) {
        busy[e] = b->engine_live[e] && b->engine[e].njobs > b->engine[e].lo;
        any = any || busy[e];
    }
    if (iterations > 0 && any) {
        // Colour buffers and job entries were set up on the batch stream.
        PT_B_TRY(b, cudaEventRecord(b->ev, b->stream));
        for (int e = 0; e < kEngines; e++) {
            if (!busy[e]) continue;
            PT_B_TRY(b, cudaStreamWaitEvent(b->estream[e], b->ev, 0));
            PT_B_TRY(b, b->engine[e].run(iterations, false));
        }
        b->iterations += (uint64_t)iterations;
    }
    for (int e = 0; e < kEngines; e++) {
        if (!busy[e]) continue;
        WfEngine& E = b->engine[e];
        if (E.checks) {
            PT_B_TRY(b, E.read_counters(E.host_counters));
            uint32_t bad_index = 0;
            if (const uint32_t site = E.check_failed(&bad_index))
                return bfail(b, PT_ERR_KERNEL, std::string("pt_batch_step: device index check failed: ") +
                                                   pt_check_site_name(site) + " (index " +
                                                   std::to_string(bad_index) + ")");
        }
        PT_B_TRY(b, E.read_finished(E.lo, E.njobs, b->h_finished));
        for (uint32_t j = E.lo; j < E.njobs; j++) {
            BatchPass& p = *pass_at(b, b->eorder[e][j - E.lo]);
            const int part = e == p.engine ? 0 : 1;
            if (b->h_finished[j - E.lo] >= (part == 0 ? p.count0 : p.count - p.count0)) p.part_finished[part] = true;
            p.finished = p.part_finished[0] && (p.engine2 < 0 || p.part_finished[1]);
        }
    }
    std::fill(b->blocked.begin(), b->blocked.end(), 0);
    int nc = 0;
    for (size_t i = 0; i < b->passes.size(); i++) {
        BatchPass& p = b->passes[i];
        if (p.done) continue;
        char& blk = b->blocked[(size_t)p.target];
        if (blk || !p.finished || nc >= capacity) {
            blk = 1;
            continue;
        }
        BatchTarget& t = b->targets[(size_t)p.target];
        WfEngine& E = b->engine[p.engine];
        if (t.kind == PT_TARGET_FLOAT) {
            PT_B_TRY(b, E.resolve(p.eidx, b->stream));
        } else {
            const WfJob& J = E.job(p.eidx);
            const uint32_t npix = (uint32_t)t.width * (uint32_t)t.height;
            const double exposure = (double)J.pc.apertureSize * (double)J.pc.apertureSize * (double)J.pc.ISO;
            b->kernel_launches += 1;
            resolve_fp64_kernel<<<(npix + 255) / 256, 256, 0, b->stream>>>(p.d_colors, npix, J.pc.samplesPerFrame,
                                                                          exposure, t.d_sum);
            PT_B_TRY(b, cudaGetLastError());
        }
        PT_B_TRY(b, cudaFreeAsync(p.d_colors, b->stream));
        p.d_colors = nullptr;
        p.done = true;
        t.passes_in_flight--;
        t.samples += p.spf;
        b->scenes[(size_t)p.scene].passes_in_flight--;
        b->samples_done += p.count;
        completed[nc++] = (int)(b->pass_base + i);
    }
    // Retire each engine's resolved prefix (its ring entries are reused) and
    // drop the batch's resolved prefix.
    for (int e = 0; e < kEngines; e++) {
        if (!b->engine_live[e]) continue;
        uint32_t lo = b->engine[e].lo;
        while (!b->eorder[e].empty() && pass_at(b, b->eorder[e].front())->done) {
            b->eorder[e].pop_front();
            lo++;
        }
        b->engine[e].retire(lo);
    }
    while (!b->passes.empty() && b->passes.front().done) {
        b->passes.pop_front();
        b->pass_base++;
    }
    *ncompleted = nc;
    return PT_OK;
}

int pt_batch_pending(pt_batch* b) {
    if (!b) return -1;
    int n = 0;
    for (const BatchPass& p : b->passes)
        if (!p.done) n++;
    return n;
}

int pt_batch_set_device_checks(pt_batch* b, int on) {
    if (!b) return PT_ERR_INVALID;
    if (pt_batch_pending(b) > 0) return bfail(b, PT_ERR_BUSY, "pt_batch_set_device_checks: passes are in flight");
    PT_B_TRY(b, cudaSetDevice(b->device));
    b->device_checks = on != 0;
    for (int e = 0; e < kEngines; e++) {
        if (!b->engine_live[e]) continue;
        PT_B_TRY(b, cudaStreamSynchronize(b->engine[e].stream));
        b->engine[e].set_checks(b->device_checks);
    }
    if (!b->custom.empty()) b->jit_dirty = true;  // the march kernel of the other build
    if (!b->jit_dirty) set_staged_march_kernel(b, staged_march_kernel(b));
    return PT_OK;
}

int pt_batch_render_fp64(pt_batch* b, int scene_id, int target_id, const pt_push* push) {
    if (!b) return PT_ERR_INVALID;
    if (!push) return bfail(b, PT_ERR_INVALID, "pt_batch_render_fp64: null push constants");
    if (scene_id < 0 || scene_id >= (int)b->scenes.size() || !b->scenes[(size_t)scene_id].live)
        return bfail(b, PT_ERR_INVALID, "pt_batch_render_fp64: unknown or released scene");
    if (check_target(b, target_id, "pt_batch_render_fp64") != PT_OK) return PT_ERR_INVALID;
    BatchTarget& t = b->targets[(size_t)target_id];
    if (t.kind != PT_TARGET_FP64) return bfail(b, PT_ERR_INVALID, "pt_batch_render_fp64: the target is not FP64");
    if (push->resolution[0] != t.width || push->resolution[1] != t.height)
        return bfail(b, PT_ERR_INVALID, "pt_batch_render_fp64: resolution differs from the target's");
    if (push->samplesPerFrame <= 0) return bfail(b, PT_ERR_INVALID, "pt_batch_render_fp64: samplesPerFrame <= 0");
    const BatchScene& sc = b->scenes[(size_t)scene_id];
    PT_B_TRY(b, cudaSetDevice(b->device));
    if (sc.custom) {
        const int jr = prepare_jit64(b);
        if (jr != PT_OK) return jr;
    }
    // The kernel takes the scene by value (its launch's constant bank): read
    // the resident copy back, rotation matrices and extensions included.
    KParams* P = new (std::nothrow) KParams;
    if (!P) return bfail(b, PT_ERR_OOM, "pt_batch_render_fp64: out of host memory");
    std::memset(P, 0, sizeof *P);
    cudaError_t e = cudaMemcpyAsync(&P->s, sc.d_scene, sizeof(KScene), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess) {
        P->pc = *push;
        P->cie = sc.d_cie;
        P->sums = t.d_sum;
        e = sc.custom ? pt_jit_launch(b->jit64, P, false, b->stream) : ptk_launch_fp64(P, false, b->stream);
        b->kernel_launches += 1;
    }
    delete P;
    if (e != cudaSuccess) return bcuda(b, e, "pt_batch_render_fp64");
    t.samples += (uint64_t)push->samplesPerFrame;
    return PT_OK;
}

int pt_batch_run(pt_batch* b, uint64_t max_iterations) {
    if (!b) return PT_ERR_INVALID;
    uint64_t iters = 0;
    int chunk = 8;
    int ids[256];
    while (pt_batch_pending(b) > 0) {
        if (iters >= max_iterations) return bfail(b, PT_ERR_KERNEL, "pt_batch_run: passes did not finish");
        int nc = 0;
        const int rc = pt_batch_step(b, chunk, ids, 256, &nc);
        if (rc != PT_OK) return rc;
        iters += (uint64_t)chunk;
        if (chunk < 64) chunk *= 2;
    }
    PT_B_TRY(b, cudaStreamSynchronize(b->stream));
    return PT_OK;
}

int pt_batch_stats(pt_batch* b, pt_batch_info* out) {
    if (!b || !out) return PT_ERR_INVALID;
    std::memset(out, 0, sizeof *out);
    out->samples_done = b->samples_done;
    out->samples_added = b->samples_added;
    out->iterations = b->iterations;
    out->passes_added = b->next_pass;
    out->passes_pending = (uint32_t)pt_batch_pending(b);
    out->pool_slots = b->pool_slots;
    out->pass_slots = b->max_passes;
    out->passes_staged = b->engine_live[kStaged] ? b->engine[kStaged].njobs : 0;
    out->passes_persistent = b->engine_live[kPersistent] ? b->engine[kPersistent].njobs : 0;
    out->kernel_launches = b->kernel_launches;
    for (int e = 0; e < kEngines; e++)
        if (b->engine_live[e]) out->kernel_launches += b->engine[e].kernel_launches;
    return PT_OK;
}

int pt_batch_target_samples(pt_batch* b, int target_id, uint64_t* samples) {
    if (!b || !samples) return PT_ERR_INVALID;
    if (check_target(b, target_id, "pt_batch_target_samples") != PT_OK) return PT_ERR_INVALID;
    *samples = b->targets[(size_t)target_id].samples;
    return PT_OK;
}

int pt_batch_read_target(pt_batch* b, int target_id, float* host, size_t bytes) {
    if (!b) return PT_ERR_INVALID;
    if (check_target(b, target_id, "pt_batch_read_target") != PT_OK) return PT_ERR_INVALID;
    const BatchTarget& t = b->targets[(size_t)target_id];
    const size_t npix = (size_t)t.width * (size_t)t.height;
    const size_t need = npix * sizeof(float4);
    if (!host || bytes < need) return bfail(b, PT_ERR_INVALID, "pt_batch_read_target: buffer too small");
    PT_B_TRY(b, cudaSetDevice(b->device));
    if (t.kind == PT_TARGET_FLOAT) {
        PT_B_TRY(b, cudaMemcpyAsync(host, t.d_accum, need, cudaMemcpyDeviceToHost, b->stream));
    } else {
        float4* tmp = nullptr;
        PT_B_TRY(b, cudaMallocFromPoolAsync(&tmp, need, b->mempool, b->stream));
        b->kernel_launches += 1;
        fp64_to_float_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, b->stream>>>(t.d_sum, (uint32_t)npix, tmp);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(host, tmp, need, cudaMemcpyDeviceToHost, b->stream);
        cudaFreeAsync(tmp, b->stream);
        PT_B_TRY(b, e);
    }
    PT_B_TRY(b, cudaStreamSynchronize(b->stream));
    return PT_OK;
}

int pt_batch_rmse_many(pt_batch* b, const int* target_ids, const int* reference_ids, int n, double* rel_rmse) {
    if (!b) return PT_ERR_INVALID;
    if (n < 0 || (n > 0 && (!target_ids || !reference_ids || !rel_rmse)))
        return bfail(b, PT_ERR_INVALID, "pt_batch_rmse_many: bad arguments");
    for (int i = 0; i < n; i++) {
        if (check_target(b, target_ids[i], "pt_batch_rmse") != PT_OK) return PT_ERR_INVALID;
        if (check_target(b, reference_ids[i], "pt_batch_rmse") != PT_OK) return PT_ERR_INVALID;
        const BatchTarget& t = b->targets[(size_t)target_ids[i]];
        const BatchTarget& r = b->targets[(size_t)reference_ids[i]];
        if (t.kind != PT_TARGET_FLOAT || t.width != r.width || t.height != r.height)
            return bfail(b, PT_ERR_INVALID, "pt_batch_rmse: target must be a float image of the reference's size");
    }
    PT_B_TRY(b, cudaSetDevice(b->device));
    PT_B_TRY(b, reserve_rmse(b, n));
    for (int i = 0; i < n; i++) {
        const BatchTarget& t = b->targets[(size_t)target_ids[i]];
        const BatchTarget& r = b->targets[(size_t)reference_ids[i]];
        b->h_items[i] = RmseItem{t.d_accum, r.d_accum, r.d_sum, (uint32_t)t.width * (uint32_t)t.height, 0};
    }
    return run_rmse(b, n, rel_rmse);
}

int pt_batch_rmse(pt_batch* b, int target_id, int reference_id, double* rel_rmse) {
    return pt_batch_rmse_many(b, &target_id, &reference_id, 1, rel_rmse);
}

int pt_batch_rmse_image(pt_batch* b, const void* d_image, int width, int height, int reference_id,
                        double* rel_rmse) {
    if (!b) return PT_ERR_INVALID;
    if (!d_image || !rel_rmse) return bfail(b, PT_ERR_INVALID, "pt_batch_rmse_image: bad arguments");
    if (check_target(b, reference_id, "pt_batch_rmse_image") != PT_OK) return PT_ERR_INVALID;
    const BatchTarget& r = b->targets[(size_t)reference_id];
    if (width != r.width || height != r.height)
        return bfail(b, PT_ERR_INVALID, "pt_batch_rmse_image: size differs from the reference's");
    PT_B_TRY(b, cudaSetDevice(b->device));
    PT_B_TRY(b, reserve_rmse(b, 1));
    b->h_items[0] = RmseItem{static_cast<const float4*>(d_image), r.d_accum, r.d_sum,
                             (uint32_t)width * (uint32_t)height, 0};
    return run_rmse(b, 1, rel_rmse);
}

int pt_batch_release_target(pt_batch* b, int target_id) {
    if (!b) return PT_ERR_INVALID;
    if (check_target(b, target_id, "pt_batch_release_target") != PT_OK) return PT_ERR_INVALID;
    BatchTarget& t = b->targets[(size_t)target_id];
    if (t.passes_in_flight) return bfail(b, PT_ERR_BUSY, "pt_batch_release_target: passes still render into it");
    if (t.d_accum) PT_B_TRY(b, cudaFreeAsync(t.d_accum, b->stream));
    if (t.d_sum) PT_B_TRY(b, cudaFreeAsync(t.d_sum, b->stream));
    t.d_accum = nullptr;
    t.d_sum = nullptr;
    t.live = false;
    return PT_OK;
}

int pt_batch_set_scene_ext(pt_batch* b, int scene_id, const pt_scene_ext* ext) {
    if (!b) return PT_ERR_INVALID;
    if (scene_id < 0 || scene_id >= (int)b->scenes.size() || !b->scenes[(size_t)scene_id].live)
        return bfail(b, PT_ERR_INVALID, "pt_batch_set_scene_ext: unknown or released scene");
    BatchScene& s = b->scenes[(size_t)scene_id];
    if (s.passes_in_flight) return bfail(b, PT_ERR_BUSY, "pt_batch_set_scene_ext: passes still read the scene");
    std::string why;
    if (!pt_ext_valid(ext, &why)) return bfail(b, PT_ERR_INVALID, "pt_batch_set_scene_ext: " + why);
    pt_scene_ext x;
    if (ext) {
        x = *ext;
    } else {
        std::memset(&x, 0, sizeof x);
    }
    PT_B_TRY(b, cudaSetDevice(b->device));
    for (int e = 0; e < kEngines; e++)
        if (b->engine_live[e]) PT_B_TRY(b, cudaStreamSynchronize(b->engine[e].stream));
    PT_B_TRY(b, cudaMemcpyAsync(&s.d_scene->ext, &x, sizeof x, cudaMemcpyHostToDevice, b->stream));
    PT_B_TRY(b, cudaStreamSynchronize(b->stream));  // the copy reads the stack
    if (s.h_scene) s.h_scene->ext = x;
    return PT_OK;
}

int pt_batch_release_scene(pt_batch* b, int scene_id) {
    if (!b) return PT_ERR_INVALID;
    if (scene_id < 0 || scene_id >= (int)b->scenes.size() || !b->scenes[(size_t)scene_id].live)
        return bfail(b, PT_ERR_INVALID, "pt_batch_release_scene: unknown or released scene");
    BatchScene& s = b->scenes[(size_t)scene_id];
    if (s.passes_in_flight) return bfail(b, PT_ERR_BUSY, "pt_batch_release_scene: passes still read it");
    PT_B_TRY(b, cudaStreamSynchronize(b->stream));
    cudaFree(s.d_scene);
    cudaFree(s.d_cie);
    s.d_scene = nullptr;
    s.d_cie = nullptr;
    s.h_scene.reset();
    s.live = false;
    return PT_OK;
}

}  // extern "C"
