// pt_api.cu — the C ABI of libpt_cuda (include/pt_cuda.h).
//
// A context stands in for the reference's Vulkan device, compute pipeline,
// uniform buffer, texel buffer and fence (src/pathtracer.cpp:1227-2423,
// 3586-3608, 3843-3880).  It owns its device memory and one stream; nothing
// here is process-global, so contexts may coexist on one device.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pt_cuda.h"
#include "kernel/pt_megakernel.h"
#include "kernel/pt_wavefront.h"
#include "kernel/pt_features.h"
#include "pt_engine.h"
#include "pt_jit.h"

struct pt_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    KParams* params = nullptr;  // host image of the launch parameters
    bool has_scene = false;
    float* d_cie = nullptr;
    float* d_rot = nullptr;
    float4* d_accum = nullptr;
    int width = 0, height = 0;
    pt_sdf_plugin plug[PT_MAX_LIVE_SDFS];
    int nplug = 0;
    KTrace trace{nullptr, nullptr, nullptr, 0};
    int engine = PT_ENGINE_WAVEFRONT;
    uint32_t pool_cap = 1u << 22;  // wavefront path slots: more rays to refill march lanes from (measured best)
    int march_budget = 64;
    bool stage_timing = false;
    int refill_min = 2;    // measured best on GB300 (mandelbulb 1024x1024)
    int drain_lanes = 24;
    int march_inner = 6;
    int blocks_per_sm = 4;
    KScene* d_scene = nullptr;     // device copy for the wavefront kernels
    WfEngine* wf = nullptr;        // wavefront driver (created on first use, grows with the dispatch)
    // More engines, on streams of their own, take equal shares of a large
    // dispatch's samples (pt_set_wavefront_engines); `fork` orders them after
    // the context's stream, `join` the resolve after them.
    static constexpr int kMaxEngines = 4;
    int wf_engines = 2;
    WfEngine* wf_more[kMaxEngines - 1] = {};
    cudaStream_t stream_more[kMaxEngines - 1] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kMaxEngines - 1] = {};
    float4* d_colors = nullptr;    // per-sample colours of the current dispatch
    uint8_t* d_rgb = nullptr;      // pt_read_rgb8 staging (W*H*3 bytes)
    size_t rgb_bytes = 0;
    size_t colors_bytes = 0;
    uint32_t last_iterations = 0;
    uint64_t last_launches = 0;    // kernels the last pt_dispatch launched
    uint64_t drain_limit = 0;      // iteration cap of the wavefront drain (0: the bound computed per dispatch)
    bool fp_contract = false;      // run-time compiled kernels with FMA contraction (pt_set_fp_contract)
    bool device_checks = false;    // the wavefront engine's checked kernel build (pt_set_device_checks)
    // GLSL snippets other than the shipped four (PT_SDF_CUSTOM slots), as
    // translated by pt_glsl_translate, and the module compiled for them.
    std::vector<JitSlot> custom;
    // Modules compiled for this context, per kind, oldest first (at most
    // kJitCache each, so switching between scenes does not recompile), and
    // the one the current snippets use.
    std::vector<JitModule> jit[kJitKinds];
    int jit_cur[kJitKinds] = {-1, -1, -1};
    std::string err;
};

namespace {

int fail(pt_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_fail(pt_ctx* ctx, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(ctx, e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA, m);
}

#define PT_CUDA_TRY(ctx, call)                                   \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

bool integral_count(float v, int max, int* out) {
    if (!(v >= 0.0f) || v > (float)max || std::floor(v) != v) return false;
    *out = (int)v;
    return true;
}

void refresh_plugins(pt_ctx* ctx) {
    std::memset(ctx->params->s.plug, 0, sizeof(ctx->params->s.plug));
    std::memcpy(ctx->params->s.plug, ctx->plug, sizeof(pt_sdf_plugin) * (size_t)ctx->nplug);
    ctx->params->s.meta.nplug = ctx->nplug;
}

// Keeps the device copy of the scene (read by the wavefront kernels) in step
// with the launch-parameter copy (read by the megakernel).
cudaError_t sync_device_scene(pt_ctx* ctx) {
    if (!ctx->has_scene) return cudaSuccess;
    return cudaMemcpyAsync(ctx->d_scene, &ctx->params->s, sizeof(KScene), cudaMemcpyHostToDevice, ctx->stream);
}

}  // namespace

static int dispatch_wavefront(pt_ctx* ctx, const pt_push* push);
static int dispatch_jit(pt_ctx* ctx, bool trace);
static int ensure_jit(pt_ctx* ctx, JitKind kind);
cudaError_t ptk_export_rgb8(const void* d_accum, int width, int height, int tonemap, void* d_rgb, cudaStream_t stream);

extern "C" {

int pt_create(pt_ctx** out, int device) {
    if (!out) return PT_ERR_INVALID;
    *out = nullptr;
    pt_ctx* ctx = new (std::nothrow) pt_ctx();
    if (!ctx) return PT_ERR_OOM;
    ctx->params = new (std::nothrow) KParams();
    if (!ctx->params) {
        delete ctx;
        return PT_ERR_OOM;
    }
    std::memset(ctx->params, 0, sizeof(KParams));
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_cie, sizeof(float) * PT_CIE_TABLE_SIZE);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_rot, sizeof(float) * 9 * PT_MAX_SCENE_OBJECTS);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_scene, sizeof(KScene));
    if (e != cudaSuccess) {
        pt_destroy(ctx);
        return e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    *out = ctx;
    return PT_OK;
}

int pt_destroy(pt_ctx* ctx) {
    if (!ctx) return PT_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->d_accum) cudaFree(ctx->d_accum);
    if (ctx->d_cie) cudaFree(ctx->d_cie);
    if (ctx->d_rot) cudaFree(ctx->d_rot);
    if (ctx->d_scene) cudaFree(ctx->d_scene);
    for (cudaStream_t s : ctx->stream_more)
        if (s) cudaStreamSynchronize(s);
    if (ctx->wf) {
        ctx->wf->destroy();
        delete ctx->wf;
    }
    for (WfEngine* e : ctx->wf_more)
        if (e) {
            e->destroy();
            delete e;
        }
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    for (cudaEvent_t ev : ctx->join)
        if (ev) cudaEventDestroy(ev);
    for (cudaStream_t s : ctx->stream_more)
        if (s) cudaStreamDestroy(s);
    if (ctx->d_colors) cudaFree(ctx->d_colors);
    if (ctx->d_rgb) cudaFree(ctx->d_rgb);
    for (auto& cache : ctx->jit)
        for (JitModule& m : cache) pt_jit_unload(m);
    if (ctx->done) cudaEventDestroy(ctx->done);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx->params;
    delete ctx;
    return PT_OK;
}

int pt_set_sdf_plugins(pt_ctx* ctx, const pt_sdf_plugin* plugins, int n) {
    if (!ctx) return PT_ERR_INVALID;
    if (n < 0 || (n > 0 && !plugins)) return fail(ctx, PT_ERR_INVALID, "pt_set_sdf_plugins: bad plug-in array");
    if (n > PT_MAX_LIVE_SDFS)
        return fail(ctx, PT_ERR_UNSUPPORTED, "pt_set_sdf_plugins: at most 32 SDFs can be evaluated (32-bit set mask)");
    for (int i = 0; i < n; i++) {
        if (plugins[i].kind < PT_SDF_NONE || plugins[i].kind > PT_SDF_TERRAIN)
            return fail(ctx, PT_ERR_INVALID,
                        "pt_set_sdf_plugins: unknown plug-in kind (GLSL text goes through pt_set_sdfs)");
    }
    ctx->custom.clear();
    if (n > 0) std::memcpy(ctx->plug, plugins, sizeof(pt_sdf_plugin) * (size_t)n);
    ctx->nplug = n;
    refresh_plugins(ctx);
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    PT_CUDA_TRY(ctx, sync_device_scene(ctx));
    return PT_OK;
}

int pt_set_sdfs(pt_ctx* ctx, const char* const* sources, int n) {
    if (!ctx) return PT_ERR_INVALID;
    if (n < 0 || (n > 0 && !sources)) return fail(ctx, PT_ERR_INVALID, "pt_set_sdfs: bad source array");
    if (n > PT_MAX_LIVE_SDFS)
        return fail(ctx, PT_ERR_UNSUPPORTED, "pt_set_sdfs: at most 32 SDFs can be evaluated (32-bit set mask)");
    pt_sdf_plugin tmp[PT_MAX_LIVE_SDFS];
    std::vector<JitSlot> custom;
    for (int i = 0; i < n; i++) {
        if (!sources[i]) return fail(ctx, PT_ERR_INVALID, "pt_set_sdfs: null source");
        if (pt_parse_sdf_source(sources[i], &tmp[i]) == PT_OK) continue;
        // Other GLSL: compiled at run time with the megakernel.
        JitSlot j;
        std::string why;
        const int rc = pt_jit_translate_slot(sources[i], i, j, why);
        if (rc != PT_OK) return fail(ctx, rc, "pt_set_sdfs: SDF " + std::to_string(i) + ": " + why);
        tmp[i] = pt_sdf_plugin{PT_SDF_CUSTOM, PT_SDFMAT_DEFAULT, {0.0f, 0.0f, 0.0f}};
        custom.push_back(j);
    }
    if (n > 0) std::memcpy(ctx->plug, tmp, sizeof(pt_sdf_plugin) * (size_t)n);
    ctx->nplug = n;
    ctx->custom = custom;
    refresh_plugins(ctx);
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    PT_CUDA_TRY(ctx, sync_device_scene(ctx));
    return PT_OK;
}

int pt_upload_scene(pt_ctx* ctx, const pt_ubo* ubo) { return pt_upload_scene_ext(ctx, ubo, nullptr); }

int pt_upload_scene_ext(pt_ctx* ctx, const pt_ubo* ubo, const pt_scene_ext* ext) {
    if (!ctx) return PT_ERR_INVALID;
    if (!ubo) return fail(ctx, PT_ERR_INVALID, "pt_upload_scene: null ubo");
    {
        std::string why;
        if (!pt_ext_valid(ext, &why)) return fail(ctx, PT_ERR_INVALID, "pt_upload_scene_ext: " + why);
    }
    int n[7];
    const int caps[7] = {PT_MAX_OBJECTS_SIZE / 6, PT_MAX_OBJECTS_SIZE / 5, PT_MAX_OBJECTS_SIZE / 11,
                         PT_MAX_OBJECTS_SIZE / 12, PT_MAX_OBJECTS_SIZE / 16, PT_MAX_SDFS_SIZE / 6,
                         PT_MAX_LIGHTIDS_SIZE};
    for (int i = 0; i < 7; i++) {
        if (!integral_count(ubo->numObjects[i], caps[i], &n[i]))
            return fail(ctx, PT_ERR_INVALID, "pt_upload_scene: numObjects[" + std::to_string(i) + "] is not a valid count");
    }
    const int floats = 6 * n[0] + 5 * n[1] + 11 * n[2] + 12 * n[3] + 16 * n[4];
    if (floats > PT_MAX_OBJECTS_SIZE)
        return fail(ctx, PT_ERR_INVALID, "pt_upload_scene: objects overflow the 1024-float object array");
    if (n[5] > PT_MAX_LIVE_SDFS)
        return fail(ctx, PT_ERR_UNSUPPORTED, "pt_upload_scene: at most 32 SDFs can be evaluated (32-bit set mask)");
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));

    KScene& S = ctx->params->s;
    std::memcpy(S.numObjects, ubo->numObjects, sizeof(S.numObjects));
    std::memcpy(S.objects, ubo->objects, sizeof(S.objects));
    std::memcpy(S.sdfs, ubo->sdfs, sizeof(S.sdfs));
    std::memcpy(S.materials, ubo->materials, sizeof(S.materials));
    std::memcpy(S.lights, ubo->lights, sizeof(S.lights));
    std::memcpy(S.lightIDs, ubo->lightIDs, sizeof(S.lightIDs));
    for (int i = 0; i < 7; i++) S.meta.n[i] = n[i];
    S.meta.offset[0] = 0;
    S.meta.offset[1] = 6 * n[0];
    S.meta.offset[2] = S.meta.offset[1] + 5 * n[1];
    S.meta.offset[3] = S.meta.offset[2] + 11 * n[2];
    S.meta.offset[4] = S.meta.offset[3] + 12 * n[3];
    S.meta.total_objects = n[0] + n[1] + n[2] + n[3] + n[4];
    if (ext) {
        S.ext = *ext;
    } else {
        std::memset(&S.ext, 0, sizeof(S.ext));
    }
    refresh_plugins(ctx);

    PT_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_cie, ubo->CIEXYZ1931, sizeof(float) * PT_CIE_TABLE_SIZE,
                                     cudaMemcpyHostToDevice, ctx->stream));
    // Derive the rotation matrices on the device (the kernel's own sin/cos),
    // then carry them in the launch parameters.
    std::memset(S.rot, 0, sizeof(S.rot));
    if (S.meta.total_objects > 0) {
        PT_CUDA_TRY(ctx, ptk_rotation_setup(&S, ctx->d_rot, ctx->stream));
        PT_CUDA_TRY(ctx, cudaMemcpyAsync(S.rot, ctx->d_rot, sizeof(float) * 9 * (size_t)S.meta.total_objects,
                                         cudaMemcpyDeviceToHost, ctx->stream));
    }
    PT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->has_scene = true;
    PT_CUDA_TRY(ctx, sync_device_scene(ctx));
    return PT_OK;
}

int pt_resize_accum(pt_ctx* ctx, int width, int height) {
    if (!ctx) return PT_ERR_INVALID;
    if (width <= 0 || height <= 0 || (long long)width * (long long)height > (1ll << 31))
        return fail(ctx, PT_ERR_INVALID, "pt_resize_accum: bad size");
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = (size_t)width * (size_t)height * sizeof(float4);
    if (ctx->d_accum && width == ctx->width && height == ctx->height) {
        // the same size: zeroed in place, in stream order (no free, no allocation)
        PT_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_accum, 0, bytes, ctx->stream));
        return PT_OK;
    }
    PT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->d_accum) {
        cudaFree(ctx->d_accum);
        ctx->d_accum = nullptr;
        ctx->width = ctx->height = 0;
    }
    PT_CUDA_TRY(ctx, cudaMalloc(&ctx->d_accum, bytes));
    PT_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_accum, 0, bytes, ctx->stream));
    ctx->width = width;
    ctx->height = height;
    return PT_OK;
}

int pt_set_trace(pt_ctx* ctx, uint32_t* d_events, uint32_t* d_nevents, float* d_colors, int depth_cap) {
    if (!ctx) return PT_ERR_INVALID;
    if (depth_cap < 0 || (d_events && depth_cap == 0)) return fail(ctx, PT_ERR_INVALID, "pt_set_trace: bad depth_cap");
    ctx->trace = KTrace{d_events, d_nevents, d_colors, depth_cap};
    return PT_OK;
}

int pt_set_fp_contract(pt_ctx* ctx, int on) {
    if (!ctx) return PT_ERR_INVALID;
    ctx->fp_contract = on != 0;
    return PT_OK;
}

int pt_set_device_checks(pt_ctx* ctx, int on) {
    if (!ctx) return PT_ERR_INVALID;
    ctx->device_checks = on != 0;
    return PT_OK;
}

int pt_set_drain_limit(pt_ctx* ctx, uint64_t max_iterations) {
    if (!ctx) return PT_ERR_INVALID;
    ctx->drain_limit = max_iterations;
    return PT_OK;
}

int pt_dispatch(pt_ctx* ctx, const pt_push* push) {
    if (!ctx) return PT_ERR_INVALID;
    if (!push) return fail(ctx, PT_ERR_INVALID, "pt_dispatch: null push constants");
    if (!ctx->has_scene) return fail(ctx, PT_ERR_NO_SCENE, "pt_dispatch: no scene uploaded");
    if (!ctx->d_accum) return fail(ctx, PT_ERR_NO_SCENE, "pt_dispatch: no accumulator (pt_resize_accum)");
    if (push->resolution[0] != ctx->width || push->resolution[1] != ctx->height)
        return fail(ctx, PT_ERR_INVALID, "pt_dispatch: resolution differs from the accumulator size");
    if (push->samplesPerFrame <= 0) return fail(ctx, PT_ERR_INVALID, "pt_dispatch: samplesPerFrame must be positive");
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    KParams& P = *ctx->params;
    P.pc = *push;
    P.accum = ctx->d_accum;
    P.cie = ctx->d_cie;
    P.trace = ctx->trace;
    const bool trace = ctx->trace.events || ctx->trace.nevents || ctx->trace.colors;
    if (!ctx->custom.empty()) {
        const bool staged = ctx->engine == PT_ENGINE_WAVEFRONT && push->pathLength > 0;
        const int rc = ensure_jit(ctx, staged ? kJitMarch : kJitMegakernel);
        if (rc != PT_OK) return rc;
        ctx->last_launches = 1;
        if (!staged) return dispatch_jit(ctx, trace);
    }
    if (ctx->engine == PT_ENGINE_WAVEFRONT && push->pathLength > 0) return dispatch_wavefront(ctx, push);
    ctx->last_launches = 1;
    PT_CUDA_TRY(ctx, ptk_launch_megakernel(&P, trace, ctx->stream));
    PT_CUDA_TRY(ctx, cudaEventRecord(ctx->done, ctx->stream));
    return PT_OK;
}

int pt_render_fp64(pt_ctx* ctx, const pt_push* push, double* d_sums) {
    if (!ctx) return PT_ERR_INVALID;
    if (!push || !d_sums) return fail(ctx, PT_ERR_INVALID, "pt_render_fp64: null push constants or sums");
    if (!ctx->has_scene) return fail(ctx, PT_ERR_NO_SCENE, "pt_render_fp64: no scene uploaded");
    if (push->resolution[0] <= 0 || push->resolution[1] <= 0 || push->samplesPerFrame <= 0)
        return fail(ctx, PT_ERR_INVALID, "pt_render_fp64: bad resolution or samplesPerFrame");
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    if (!ctx->custom.empty()) {
        // scene GLSL: the FP64 megakernel compiled with the snippets in double
        const int rc = ensure_jit(ctx, kJitFp64);
        if (rc != PT_OK) return rc;
    }
    KParams& P = *ctx->params;
    P.pc = *push;
    P.accum = nullptr;
    P.sums = d_sums;
    P.cie = ctx->d_cie;
    P.trace = ctx->trace;
    const bool trace = ctx->trace.events || ctx->trace.nevents || ctx->trace.colors;
    const cudaError_t e =
        ctx->custom.empty() ? ptk_launch_fp64(&P, trace, ctx->stream)
                            : pt_jit_launch(ctx->jit[kJitFp64][(size_t)ctx->jit_cur[kJitFp64]], &P, trace, ctx->stream);
    P.sums = nullptr;
    PT_CUDA_TRY(ctx, e);
    PT_CUDA_TRY(ctx, cudaEventRecord(ctx->done, ctx->stream));
    return PT_OK;
}

int pt_set_engine(pt_ctx* ctx, int engine) {
    if (!ctx) return PT_ERR_INVALID;
    if (engine != PT_ENGINE_MEGAKERNEL && engine != PT_ENGINE_WAVEFRONT)
        return fail(ctx, PT_ERR_INVALID, "pt_set_engine: unknown engine");
    ctx->engine = engine;
    return PT_OK;
}

int pt_get_engine(pt_ctx* ctx) { return ctx ? ctx->engine : -1; }

int pt_set_wavefront_pool(pt_ctx* ctx, uint32_t slots) {
    if (!ctx) return PT_ERR_INVALID;
    if (slots < 1024 || slots > (1u << 28)) return fail(ctx, PT_ERR_INVALID, "pt_set_wavefront_pool: 1024..2^28 slots");
    ctx->pool_cap = slots;
    return PT_OK;
}

uint32_t pt_last_iterations(pt_ctx* ctx) { return ctx ? ctx->last_iterations : 0; }

uint64_t pt_last_kernel_launches(pt_ctx* ctx) { return ctx ? ctx->last_launches : 0; }

int pt_set_wavefront_engines(pt_ctx* ctx, int engines) {
    if (!ctx) return PT_ERR_INVALID;
    if (engines < 1 || engines > pt_ctx::kMaxEngines)
        return fail(ctx, PT_ERR_INVALID, "pt_set_wavefront_engines: 1..4 engines");
    ctx->wf_engines = engines;
    // engines past the new count give their pools back
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    for (int e = engines - 1; e < pt_ctx::kMaxEngines - 1; e++) {
        if (!ctx->wf_more[e]) continue;
        PT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream_more[e]));
        ctx->wf_more[e]->destroy();
        delete ctx->wf_more[e];
        ctx->wf_more[e] = nullptr;
    }
    return PT_OK;
}

int pt_get_wavefront_engines(pt_ctx* ctx) { return ctx ? ctx->wf_engines : -1; }

int pt_set_march_budget(pt_ctx* ctx, int steps) {
    if (!ctx) return PT_ERR_INVALID;
    if (steps < 1 || steps > 512) return fail(ctx, PT_ERR_INVALID, "pt_set_march_budget: 1..512 steps");
    ctx->march_budget = steps;
    return PT_OK;
}

int pt_set_stage_timing(pt_ctx* ctx, int on) {
    if (!ctx) return PT_ERR_INVALID;
    ctx->stage_timing = on != 0;
    if (ctx->wf) PT_CUDA_TRY(ctx, ctx->wf->set_stage_timing(ctx->stage_timing));  // a second engine runs untimed
    return PT_OK;
}

int pt_get_stage_times(pt_ctx* ctx, double ms[5], uint64_t* iterations) {
    if (!ctx || !ms) return PT_ERR_INVALID;
    for (int k = 0; k < PT_STAGE_COUNT; k++) ms[k] = ctx->wf ? ctx->wf->stage_ms[k] : 0.0;
    if (iterations) *iterations = ctx->wf ? ctx->wf->stage_launches : 0;
    return PT_OK;
}

int pt_get_wavefront_tuning(pt_ctx* ctx, pt_wavefront_tuning* out) {
    if (!ctx || !out) return PT_ERR_INVALID;
    out->pool_slots = ctx->pool_cap;
    out->march_budget = ctx->march_budget;
    out->refill_min = ctx->refill_min;
    out->drain_lanes = ctx->drain_lanes;
    out->blocks_per_sm = ctx->blocks_per_sm;
    out->march_inner = ctx->march_inner;
    return PT_OK;
}

int pt_set_wavefront_tuning(pt_ctx* ctx, const pt_wavefront_tuning* t) {
    if (!ctx) return PT_ERR_INVALID;
    if (!t || t->pool_slots < 1024 || t->pool_slots > (1u << 28) || t->march_budget < 1 || t->march_budget > 512 ||
        t->refill_min < 1 || t->refill_min > 32 || t->drain_lanes < 0 || t->drain_lanes > 32 || t->blocks_per_sm < 1 ||
        t->blocks_per_sm > 8 || t->march_inner < 1 || t->march_inner > 16)
        return fail(ctx, PT_ERR_INVALID, "pt_set_wavefront_tuning: a value is out of range");
    ctx->pool_cap = t->pool_slots;
    ctx->march_budget = t->march_budget;
    ctx->refill_min = t->refill_min;
    ctx->drain_lanes = t->drain_lanes;
    ctx->blocks_per_sm = t->blocks_per_sm;
    ctx->march_inner = t->march_inner;
    return PT_OK;
}

// Coordinate descent over the wavefront knobs, timing real dispatches of
// `push` (host wall clock around dispatch + wait, best of two after a
// warm-up); a setting replaces the current one only when it is at least 3 %
// faster, so run-to-run noise (about 1-2 % on GB300) does not move the
// knobs.  The accumulator is restored afterwards.
constexpr double kAutotuneGain = 0.97;
int pt_autotune_wavefront(pt_ctx* ctx, const pt_push* push, int rounds, pt_wavefront_tuning* best,
                          double* best_seconds) {
    if (!ctx) return PT_ERR_INVALID;
    if (!push || rounds < 1 || !best) return fail(ctx, PT_ERR_INVALID, "pt_autotune_wavefront: bad arguments");
    if (!ctx->has_scene || !ctx->d_accum) return fail(ctx, PT_ERR_NO_SCENE, "pt_autotune_wavefront: no scene");
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = (size_t)ctx->width * (size_t)ctx->height * sizeof(float4);
    float4* saved = nullptr;
    PT_CUDA_TRY(ctx, cudaMalloc(&saved, bytes));
    cudaError_t ce = cudaMemcpyAsync(saved, ctx->d_accum, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
    if (ce != cudaSuccess) {
        cudaFree(saved);
        return cuda_fail(ctx, ce, "pt_autotune_wavefront");
    }
    const int engine = ctx->engine;
    ctx->engine = PT_ENGINE_WAVEFRONT;
    auto time_one = [&](const pt_wavefront_tuning& t, double* secs) -> int {
        int rc = pt_set_wavefront_tuning(ctx, &t);
        double b = 1e30;
        for (int i = 0; i < 3 && rc == PT_OK; i++) {
            const auto t0 = std::chrono::steady_clock::now();
            rc = pt_dispatch(ctx, push);
            if (rc == PT_OK) rc = pt_wait(ctx, UINT64_MAX);
            const double d = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (i > 0) b = std::min(b, d);
        }
        *secs = b;
        return rc;
    };
    static const uint32_t kPools[] = {1u << 19, 1u << 20, 1u << 21, 1u << 22};
    static const int kBudgets[] = {32, 64, 128};
    static const int kRefill[] = {1, 2, 4, 8};
    static const int kDrain[] = {0, 8, 16, 24};
    static const int kBlocks[] = {2, 3, 4};
    static const int kInner[] = {2, 4, 6, 8};
    pt_wavefront_tuning cur;
    pt_get_wavefront_tuning(ctx, &cur);
    double cur_t = 0.0;
    int rc = time_one(cur, &cur_t);
    for (int r = 0; r < rounds && rc == PT_OK; r++) {
        for (int knob = 0; knob < 6 && rc == PT_OK; knob++) {
            constexpr int kCount[6] = {(int)(sizeof kPools / sizeof kPools[0]), (int)(sizeof kBudgets / sizeof kBudgets[0]),
                                       (int)(sizeof kRefill / sizeof kRefill[0]), (int)(sizeof kDrain / sizeof kDrain[0]),
                                       (int)(sizeof kBlocks / sizeof kBlocks[0]), (int)(sizeof kInner / sizeof kInner[0])};
            const int nvals = kCount[knob];
            for (int i = 0; i < nvals && rc == PT_OK; i++) {
                pt_wavefront_tuning c = cur;
                switch (knob) {
                    case 0: c.pool_slots = kPools[i]; break;
                    case 1: c.march_budget = kBudgets[i]; break;
                    case 2: c.refill_min = kRefill[i]; break;
                    case 3: c.drain_lanes = kDrain[i]; break;
                    case 4: c.blocks_per_sm = kBlocks[i]; break;
                    default: c.march_inner = kInner[i]; break;
                }
                if (std::memcmp(&c, &cur, sizeof c) == 0) continue;
                double t = 0.0;
                rc = time_one(c, &t);
                if (rc == PT_OK && t < kAutotuneGain * cur_t) {
                    cur = c;
                    cur_t = t;
                }
            }
        }
    }
    ctx->engine = engine;
    if (rc == PT_OK) rc = pt_set_wavefront_tuning(ctx, &cur);
    ce = cudaMemcpyAsync(ctx->d_accum, saved, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
    cudaFree(saved);
    if (rc != PT_OK) return rc;
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "pt_autotune_wavefront");
    *best = cur;
    if (best_seconds) *best_seconds = cur_t;
    return PT_OK;
}

int pt_wait(pt_ctx* ctx, uint64_t timeout_ns) {
    if (!ctx) return PT_ERR_INVALID;
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const auto start = std::chrono::steady_clock::now();
    auto sleep = std::chrono::microseconds(20);
    for (;;) {
        const cudaError_t e = cudaStreamQuery(ctx->stream);
        if (e == cudaSuccess) return PT_OK;
        if (e != cudaErrorNotReady) return cuda_fail(ctx, e, "pt_wait");
        const auto waited = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - start);
        if ((uint64_t)waited.count() >= timeout_ns) return fail(ctx, PT_ERR_TIMEOUT, "pt_wait: deadline passed");
        std::this_thread::sleep_for(sleep);
        if (sleep < std::chrono::microseconds(2000)) sleep *= 2;
    }
}

int pt_read_accum(pt_ctx* ctx, float* host, size_t bytes) {
    if (!ctx) return PT_ERR_INVALID;
    if (!ctx->d_accum) return fail(ctx, PT_ERR_NO_SCENE, "pt_read_accum: no accumulator");
    const size_t need = (size_t)ctx->width * (size_t)ctx->height * sizeof(float4);
    if (!host || bytes < need) return fail(ctx, PT_ERR_INVALID, "pt_read_accum: buffer too small");
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    PT_CUDA_TRY(ctx, cudaMemcpyAsync(host, ctx->d_accum, need, cudaMemcpyDeviceToHost, ctx->stream));
    PT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_write_accum(pt_ctx* ctx, const float* host, size_t bytes) {
    if (!ctx) return PT_ERR_INVALID;
    if (!ctx->d_accum) return fail(ctx, PT_ERR_NO_SCENE, "pt_write_accum: no accumulator");
    const size_t need = (size_t)ctx->width * (size_t)ctx->height * sizeof(float4);
    if (!host || bytes < need) return fail(ctx, PT_ERR_INVALID, "pt_write_accum: buffer too small");
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    PT_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_accum, host, need, cudaMemcpyHostToDevice, ctx->stream));
    PT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_read_rgb8(pt_ctx* ctx, int tonemap, uint8_t* host, size_t bytes) {
    if (!ctx) return PT_ERR_INVALID;
    if (!ctx->d_accum) return fail(ctx, PT_ERR_NO_SCENE, "pt_read_rgb8: no accumulator");
    const size_t need = (size_t)ctx->width * (size_t)ctx->height * 3;
    if (!host || bytes < need || tonemap < 0 || tonemap > 3)
        return fail(ctx, PT_ERR_INVALID, "pt_read_rgb8: bad tonemap or buffer too small");
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    if (ctx->rgb_bytes < need) {
        PT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (ctx->d_rgb) cudaFree(ctx->d_rgb);
        ctx->d_rgb = nullptr;
        ctx->rgb_bytes = 0;
        PT_CUDA_TRY(ctx, cudaMalloc(&ctx->d_rgb, need));
        ctx->rgb_bytes = need;
    }
    PT_CUDA_TRY(ctx, ptk_export_rgb8(ctx->d_accum, ctx->width, ctx->height, tonemap, ctx->d_rgb, ctx->stream));
    PT_CUDA_TRY(ctx, cudaMemcpyAsync(host, ctx->d_rgb, need, cudaMemcpyDeviceToHost, ctx->stream));
    PT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

void* pt_accum_device_ptr(pt_ctx* ctx) { return ctx ? (void*)ctx->d_accum : nullptr; }

void* pt_stream(pt_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int pt_set_stream(pt_ctx* ctx, void* stream) {
    if (!ctx) return PT_ERR_INVALID;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return PT_OK;
}

int pt_mathf_eval(pt_ctx* ctx, int fn, const float* d_x, const float* d_y, float* d_out, int n) {
    if (!ctx) return PT_ERR_INVALID;
    if (fn < 0 || fn > 10 || n < 0 || (n > 0 && (!d_x || !d_out || ((fn == 4 || fn == 8) && !d_y))))
        return fail(ctx, PT_ERR_INVALID, "pt_mathf_eval: bad arguments");
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    PT_CUDA_TRY(ctx, ptk_mathf_eval(fn, d_x, d_y, d_out, n, ctx->stream));
    PT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_quartic_surface_eval(pt_ctx* ctx, int which, const float* d_rays6, float* d_hits6, int* d_flags, int n) {
    if (!ctx) return PT_ERR_INVALID;
    if ((which != 0 && which != 1) || n < 0 || (n > 0 && (!d_rays6 || !d_hits6 || !d_flags)))
        return fail(ctx, PT_ERR_INVALID, "pt_quartic_surface_eval: bad arguments");
    PT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    PT_CUDA_TRY(ctx, ptk_quartic_surface_eval(which, d_rays6, d_hits6, d_flags, n, ctx->stream));
    PT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

const char* pt_last_error(pt_ctx* ctx) {
    if (!ctx) return "null context";
    return ctx->err.c_str();
}

}  // extern "C"

// The wavefront dispatch: one pass of one job on the context's engine,
// drained, then resolved into the accumulator.  A dispatch of at least two
// pools' worth of samples per engine is split into equal shares (in sample
// order) between up to wf_engines engines on streams of their own.
static int dispatch_wavefront(pt_ctx* ctx, const pt_push* push) {
    const uint64_t total64 = (uint64_t)push->resolution[0] * (uint64_t)push->resolution[1] *
                             (uint64_t)push->samplesPerFrame;
    if (total64 >= (1ull << 32)) return fail(ctx, PT_ERR_INVALID, "pt_dispatch: more than 2^32 samples in one dispatch");
    const uint32_t total = (uint32_t)total64;
    const bool trace = ctx->trace.events || ctx->trace.nevents || ctx->trace.colors;
    int n = 1;
    if (!trace && !ctx->stage_timing) {
        const uint64_t fit = total64 / (2ull * ctx->pool_cap);
        n = fit < (uint64_t)ctx->wf_engines ? (int)fit : ctx->wf_engines;
        if (n < 1) n = 1;
    }
    constexpr int kMax = pt_ctx::kMaxEngines;
    uint32_t base[kMax + 1];
    for (int e = 0; e <= n; e++) base[e] = (uint32_t)(total64 * (uint64_t)e / (uint64_t)n);
    WfEngine** slot[kMax] = {&ctx->wf, &ctx->wf_more[0], &ctx->wf_more[1], &ctx->wf_more[2]};
    cudaStream_t streams[kMax] = {ctx->stream, nullptr, nullptr, nullptr};
    for (int e = 1; e < n; e++) {
        if (!ctx->stream_more[e - 1]) {
            PT_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->stream_more[e - 1], cudaStreamNonBlocking));
            PT_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->join[e - 1], cudaEventDisableTiming));
        }
        streams[e] = ctx->stream_more[e - 1];
    }
    if (n > 1 && !ctx->fork) PT_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming));
    uint64_t launches0 = 0;  // engines count their launches, creation's init included
    for (int e = 0; e < kMax; e++)
        if (*slot[e]) launches0 += (*slot[e])->kernel_launches;
    // Run-time compiled SDF snippets: their march kernel (the other stages
    // evaluate no SDF); a mandelbulb: the built-in kernel with the warp-wide
    // normal pass.
    bool bulb = false;
    for (int i = 0; i < ctx->nplug; i++) bulb = bulb || ctx->plug[i].kind == PT_SDF_MANDELBULB;
    for (int e = 0; e < n; e++) {
        const uint32_t share = base[e + 1] - base[e];
        uint32_t pool = share < ctx->pool_cap ? share : ctx->pool_cap;
        if (pool < 1024u) pool = 1024u;
        WfEngine*& W = *slot[e];
        if (!W || W->pool < pool || W->pool > ctx->pool_cap) {
            PT_CUDA_TRY(ctx, cudaStreamSynchronize(streams[e]));
            if (!W) W = new (std::nothrow) WfEngine();
            if (!W) return fail(ctx, PT_ERR_OOM, "pt_dispatch: out of host memory");
            PT_CUDA_TRY(ctx, W->create(ctx->device, streams[e], pool, 4096, ctx->march_budget));
        }
        W->set_checks(ctx->device_checks);
        W->set_march_kernel(!ctx->custom.empty()
                                ? reinterpret_cast<const void*>(
                                      ctx->jit[kJitMarch][(size_t)ctx->jit_cur[kJitMarch]].kernel[0])
                                : (bulb ? W->kernels->march_warp_normals() : nullptr));
    }
    const size_t cbytes = (size_t)total * sizeof(float4);
    if (cbytes > ctx->colors_bytes) {
        PT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (ctx->d_colors) cudaFree(ctx->d_colors);
        ctx->d_colors = nullptr;
        ctx->colors_bytes = 0;
        PT_CUDA_TRY(ctx, cudaMalloc(&ctx->d_colors, cbytes));
        ctx->colors_bytes = cbytes;
    }
    // the other engines' streams start after everything queued on the context's
    if (n > 1) PT_CUDA_TRY(ctx, cudaEventRecord(ctx->fork, ctx->stream));
    for (int e = 1; e < n; e++) PT_CUDA_TRY(ctx, cudaStreamWaitEvent(streams[e], ctx->fork, 0));
    WfJob j;
    std::memset(&j, 0, sizeof j);
    j.scene = ctx->d_scene;
    j.cie = ctx->d_cie;
    j.accum = ctx->d_accum;
    j.colors = ctx->d_colors;
    j.pc = *push;
    j.variant = PT_FEAT_ALL;
    uint32_t idx0 = 0;
    WfEngine* engines[kMax];
    for (int e = 0; e < n; e++) {
        WfEngine& E = **slot[e];
        engines[e] = &E;
        E.set_stream(streams[e]);
        E.set_march_budget(ctx->march_budget);
        E.set_tuning(ctx->refill_min, ctx->drain_lanes, ctx->blocks_per_sm, ctx->march_inner);
        if (e == 0 && E.stage_timing != ctx->stage_timing) PT_CUDA_TRY(ctx, E.set_stage_timing(ctx->stage_timing));
        E.args.trace = e == 0 ? ctx->trace : KTrace{nullptr, nullptr, nullptr, 0};
        PT_CUDA_TRY(ctx, E.reset());
        uint32_t idx = 0;
        PT_CUDA_TRY(ctx, E.add_pass_part(j, base[e], base[e + 1] - base[e], &idx));
        if (e == 0) idx0 = idx;
    }
    // Every iteration moves every live path by one ray; a ray's march spans at
    // most ceil(512 / budget) + 1 iterations.
    WfEngine& E = *ctx->wf;
    const uint64_t march_iters = 512ull / (uint64_t)ctx->march_budget + 2;
    const uint64_t share_max = (total64 + (uint64_t)n - 1) / (uint64_t)n;  // the largest share
    uint64_t max_iter = (share_max / E.pool + 2) * (2ull * (uint64_t)push->pathLength + 3) * march_iters + 16;
    if (ctx->drain_limit > 0 && ctx->drain_limit < max_iter) max_iter = ctx->drain_limit;
    const cudaError_t de = n > 1 ? wf_drain_many(engines, n, max_iter) : E.drain(trace, max_iter);
    for (int e = 1; e < n; e++) {  // the resolve (and anything after it) waits for every engine
        PT_CUDA_TRY(ctx, cudaEventRecord(ctx->join[e - 1], streams[e]));
        PT_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->stream, ctx->join[e - 1], 0));
    }
    if (de == cudaErrorTimeout) return fail(ctx, PT_ERR_KERNEL, "pt_dispatch: wavefront did not drain");
    PT_CUDA_TRY(ctx, de);
    ctx->last_iterations = 0;
    for (int e = 0; e < n; e++) {
        uint32_t bad_index = 0;
        if (const uint32_t site = engines[e]->check_failed(&bad_index))
            return fail(ctx, PT_ERR_KERNEL, std::string("pt_dispatch: device index check failed: ") +
                                                pt_check_site_name(site) + " (index " + std::to_string(bad_index) + ")");
        if (engines[e]->host_counters->iterations > ctx->last_iterations)
            ctx->last_iterations = engines[e]->host_counters->iterations;
    }
    E.args.trace = KTrace{nullptr, nullptr, nullptr, 0};
    PT_CUDA_TRY(ctx, E.resolve(idx0));  // the whole pass: every share's colours
    uint64_t launches1 = 0;
    for (int e = 0; e < kMax; e++)
        if (*slot[e]) launches1 += (*slot[e])->kernel_launches;
    ctx->last_launches = launches1 - launches0;
    PT_CUDA_TRY(ctx, cudaEventRecord(ctx->done, ctx->stream));
    return PT_OK;
}

// Scenes with GLSL snippets beyond the shipped four: the megakernel (plain
// engine) or the march kernel (wavefront engine; its other stages evaluate no
// SDF) compiled at run time with their translation (pt_jit.cu) the first time
// a set of snippets is dispatched; the last 8 modules of each kind are kept.
static int ensure_jit(pt_ctx* ctx, JitKind kind) {
    constexpr size_t kJitCache = 8;
    std::vector<JitModule>& cache = ctx->jit[kind];
    // the cache key carries the contraction choice with the program text;
    // a checked march kernel is the same source with PT_DEBUG_CHECKS
    // the megakernel and march kernel of a scene whose one SDF is scene
    // GLSL evaluate it without the loop over the SDF set (PT_ONE_SDF;
    // measured faster in both)
    const bool one_sdf = (kind == kJitMegakernel || kind == kJitMarch) && ctx->nplug == 1 &&
                         ctx->custom.size() == 1 && ctx->custom[0].slot == 0;
    const std::string checks = kind == kJitMarch && ctx->device_checks ? "#define PT_DEBUG_CHECKS 1\n" : "";
    // the march kernel holds the code of the scene's plug-in kinds only (the
    // megakernel keeps every kind: without the others it measured slower)
    uint32_t kinds = 0;
    for (int i = 0; i < ctx->nplug; i++) kinds |= 1u << ctx->plug[i].kind;
    const std::string kind_mask =
        kind != kJitMarch ? std::string() : "#define PT_SDF_KINDS " + std::to_string(kinds) + "u\n";
    const std::string program = checks + (one_sdf ? "#define PT_ONE_SDF 1\n" : "") + kind_mask +
                                pt_jit_program(ctx->custom, kind) + (ctx->fp_contract ? "// fmad\n" : "");
    for (size_t i = 0; i < cache.size(); i++)
        if (cache[i].key == program) {
            ctx->jit_cur[kind] = (int)i;
            return PT_OK;
        }
    JitModule m;
    std::vector<char> cubin;
    std::string lowered[kJitMaxKernels], log;
    int rc = pt_jit_compile(ctx->device, program, kind, cubin, lowered, log, ctx->fp_contract);
    if (rc != PT_OK) return fail(ctx, rc, "compiling the scene's SDF snippets: " + log);
    rc = pt_jit_load(cubin, kind, lowered, m, log);
    if (rc != PT_OK) return fail(ctx, rc, log);
    m.key = program;
    if (cache.size() == kJitCache) {  // evict the oldest
        PT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        for (cudaStream_t s : ctx->stream_more)
            if (s) PT_CUDA_TRY(ctx, cudaStreamSynchronize(s));
        if (kind == kJitMarch) {  // no graph may keep its kernel
            if (ctx->wf) ctx->wf->set_march_kernel(nullptr);
            for (WfEngine* e : ctx->wf_more)
                if (e) e->set_march_kernel(nullptr);
        }
        pt_jit_unload(cache.front());
        cache.erase(cache.begin());
    }
    cache.push_back(m);
    ctx->jit_cur[kind] = (int)cache.size() - 1;
    return PT_OK;
}

static int dispatch_jit(pt_ctx* ctx, bool trace) {
    PT_CUDA_TRY(ctx, pt_jit_launch(ctx->jit[kJitMegakernel][(size_t)ctx->jit_cur[kJitMegakernel]], ctx->params, trace,
                                   ctx->stream));
    PT_CUDA_TRY(ctx, cudaEventRecord(ctx->done, ctx->stream));
    return PT_OK;
}
