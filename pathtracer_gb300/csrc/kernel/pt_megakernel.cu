// pt_megakernel.cu — the plain per-pixel spectral path tracer for sm_103a.
//
// One thread owns one pixel and traces its samplesPerFrame camera paths in
// order, like main()/Rendering() in src/shader.comp (SC:1509-1533), so the
// per-pixel sum and the running mean are formed in the reference's order.
// Inside the thread the path is a small state machine with ONE call site of
// intersect_all(): a primary ray, then (when next-event estimation needs it)
// the shadow ray of the same bounce, then the next bounce or the next sample.
// Lanes of a warp that are at different bounces, samples or ray kinds still
// execute the scene intersection and SDF march together, instead of
// splitting into a primary-ray pass and a shadow-ray pass.
#include <cuda_runtime.h>

#include "pt_megakernel.h"
#include "pt_path.cuh"

namespace {

template <bool TRACE, int FEAT>
__global__ void __launch_bounds__(PT_MK_THREADS) megakernel(const __grid_constant__ KParams P) {
    const KScene& S = P.s;
    const pt_push& pc = P.pc;
    __shared__ CamInfo camS;
    if (threadIdx.x == 0 && threadIdx.y == 0) camS = make_camera(pc);
    __syncthreads();

    const int W = pc.resolution[0], H = pc.resolution[1];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;  // SC:1526 uses '>'; the extra row/column would write out of bounds

    const uint32_t xx = (uint32_t)x;
    const uint32_t yy = (uint32_t)H - (uint32_t)y;  // SC:1510
    const float uvx = (2.0f * (float)xx - (float)W) / (float)H;
    const float uvy = (2.0f * (float)yy - (float)H) / (float)H;
    const int spf = pc.samplesPerFrame;
    const int depth = pc.pathLength;
    const size_t pix = (size_t)y * (size_t)W + (size_t)x;

    float3 sum = f3(0.0f, 0.0f, 0.0f);
    int k = 0;
    PathState ps;
    bool active = false, shadow = false;
    for (;;) {
        if (!active) {
            // Finish sample k-1 (SC:1477-1489, SC:1514-1516) and start sample k.
            if (k > 0) {
                const float3 color = sample_color(ps, P.cie);
                if (TRACE) {
                    const size_t p = pix * (size_t)spf + (size_t)(k - 1);
                    if (P.trace.nevents) P.trace.nevents[p] = (uint32_t)ps.bounce;
                    if (P.trace.colors) {
                        P.trace.colors[3 * p] = color.x;
                        P.trace.colors[3 * p + 1] = color.y;
                        P.trace.colors[3 * p + 2] = color.z;
                    }
                }
                sum = sum + color;
            }
            if (k >= spf) break;
            start_sample(ps, pc, camS, xx, yy, uvx, uvy, k);
            k++;
            shadow = false;
            active = depth > 0;
            continue;
        }
        // ---- the single scene intersection of the loop ----
        Hit h;
        h.hitdist = PT_MAXDIST;
        h.normal = f3(0.0f, 0.0f, 0.0f);
        h.materialID = 0.0f;
        h.lightID = -1.0f;
        int objectID = -1;
        intersect_all<FEAT>(S, ps.org, shadow ? ps.shDir : ps.dir, h, objectID);
        const StepResult r =
            shadow ? shade_shadow<TRACE>(ps, S, objectID, depth) : shade_primary<TRACE>(ps, S, h, objectID, depth);
        shadow = (r == STEP_SHADOW);
        if (TRACE && r != STEP_SHADOW) {
            const size_t p = pix * (size_t)spf + (size_t)(k - 1);
            const int b = ps.bounce - 1;
            if (P.trace.events && b < P.trace.cap) P.trace.events[p * (size_t)P.trace.cap + b] = ps.ev;
        }
        if (r == STEP_TERMINATED) active = false;
    }
    P.accum[pix] = accumulate(pc, sum, P.accum[pix]);
}

// Per-upload derivation of the rotation matrices of boxes, lenses and cyclides.
__global__ void rotation_setup_kernel(const __grid_constant__ KScene S, float* __restrict__ out) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= S.meta.total_objects) return;
    const int* n = S.meta.n;
    int base = -1;
    if (g >= n[0] + n[1]) {
        int i = g - n[0] - n[1];
        if (i < n[2]) {
            base = S.meta.offset[2] + 11 * i;
        } else if ((i -= n[2]) < n[3]) {
            base = S.meta.offset[3] + 12 * i;
        } else {
            i -= n[3];
            base = S.meta.offset[4] + 16 * i;
        }
    }
    float r[9] = {1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f};
    if (base >= 0) {
        const m3 m = rotation_matrix(f3(S.objects[base + 3], S.objects[base + 4], S.objects[base + 5]));
        r[0] = m.c0.x; r[1] = m.c0.y; r[2] = m.c0.z;
        r[3] = m.c1.x; r[4] = m.c1.y; r[5] = m.c1.z;
        r[6] = m.c2.x; r[7] = m.c2.y; r[8] = m.c2.z;
    }
#pragma unroll
    for (int j = 0; j < 9; j++) out[9 * g + j] = r[j];
}

}  // namespace

namespace {
__global__ void mathf_eval_kernel(int fn, const float* __restrict__ x, const float* __restrict__ y,
                                  float* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float r;
    switch (fn) {
        case 0: r = ptm_sinf(x[i]); break;
        case 1: r = ptm_cosf(x[i]); break;
        case 2: r = ptm_expf(x[i]); break;
        case 3: r = ptm_logf(x[i]); break;
        case 4: r = ptm_powf(x[i], y[i]); break;
        default: r = ptm_acosf(x[i]); break;
    }
    out[i] = r;
}
}  // namespace

cudaError_t ptk_mathf_eval(int fn, const float* x, const float* y, float* out, int n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    mathf_eval_kernel<<<(n + 255) / 256, 256, 0, stream>>>(fn, x, y, out, n);
    return cudaGetLastError();
}

cudaError_t ptk_rotation_setup(const KScene* scene, float* d_out, cudaStream_t stream) {
    const int n = scene->meta.total_objects;
    if (n <= 0) return cudaSuccess;
    rotation_setup_kernel<<<(n + 127) / 128, 128, 0, stream>>>(*scene, d_out);
    return cudaGetLastError();
}

cudaError_t ptk_launch_megakernel(const KParams* params, bool trace, cudaStream_t stream) {
    const int W = params->pc.resolution[0], H = params->pc.resolution[1];
    const dim3 block(PT_MK_BLOCK_X, PT_MK_BLOCK_Y);
    const dim3 grid((W + PT_MK_BLOCK_X - 1) / PT_MK_BLOCK_X, (H + PT_MK_BLOCK_Y - 1) / PT_MK_BLOCK_Y);
    if (trace) {
        megakernel<true, PT_FEAT_ALL><<<grid, block, 0, stream>>>(*params);
        return cudaGetLastError();
    }
    // The smallest variant that covers the scene's primitive classes.
    switch (pt_feature_variant(params->s.meta.n)) {
        case 0: megakernel<false, 0><<<grid, block, 0, stream>>>(*params); break;
        case PT_FEAT_BOX: megakernel<false, PT_FEAT_BOX><<<grid, block, 0, stream>>>(*params); break;
        case PT_FEAT_ANALYTIC: megakernel<false, PT_FEAT_ANALYTIC><<<grid, block, 0, stream>>>(*params); break;
        default: megakernel<false, PT_FEAT_ALL><<<grid, block, 0, stream>>>(*params); break;
    }
    return cudaGetLastError();
}
