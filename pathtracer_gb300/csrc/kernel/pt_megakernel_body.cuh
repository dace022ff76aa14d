// pt_megakernel_body.cuh — the plain megakernel, shared by the translation
// units that instantiate its variants (pt_megakernel.cu: SDF scenes and
// traces; pt_megakernel_analytic.cu: analytic scenes, with the larger math
// functions called out of line).
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
#pragma once

#include "pt_megakernel.h"
#include "pt_path.cuh"

// The run-time compiled module (pt_jit.cu) names its kernels ptjit::...
#if defined(PT_JIT_USER_SDF)
namespace ptjit {
#else
namespace {
#endif

// R = float: the shader's method, into the float accumulator.  R = double:
// the FP64 reference renderer (pt_fp64.cu), the same method in double
// precision, adding each pixel's exposed colour sum and sample count to
// P.sums.
template <bool TRACE, int FEAT, typename R = float>
__global__ void __launch_bounds__(PT_MK_THREADS) megakernel(const __grid_constant__ KParams P) {
    const KScene& S = P.s;
    const pt_push& pc = P.pc;
    __shared__ CamInfoT<R> camS;
    if (threadIdx.x == 0 && threadIdx.y == 0) camS = make_camera<R>(pc);
    __syncthreads();

    const int W = pc.resolution[0], H = pc.resolution[1];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;  // SC:1526 uses '>'; the extra row/column would write out of bounds

    const uint32_t xx = (uint32_t)x;
    const uint32_t yy = (uint32_t)H - (uint32_t)y;  // SC:1510
    const R uvx = (R(2) * (R)xx - (R)W) / (R)H;
    const R uvy = (R(2) * (R)yy - (R)H) / (R)H;
    const int spf = pc.samplesPerFrame;
    const int depth = pc.pathLength;
    const size_t pix = (size_t)y * (size_t)W + (size_t)x;

    V3<R> sum = v3<R>(R(0), R(0), R(0));
    int k = 0;
    PathStateT<R> ps;
    bool active = false, shadow = false;
    for (;;) {
        if (!active) {
            // Finish sample k-1 (SC:1477-1489, SC:1514-1516) and start sample k.
            if (k > 0) {
                const V3<R> color = sample_color(ps, S, P.cie);
                if (TRACE) {
                    const size_t p = pix * (size_t)spf + (size_t)(k - 1);
                    if (P.trace.nevents) P.trace.nevents[p] = (uint32_t)ps.bounce;
                    if (P.trace.colors) {
                        P.trace.colors[3 * p] = (float)color.x;
                        P.trace.colors[3 * p + 1] = (float)color.y;
                        P.trace.colors[3 * p + 2] = (float)color.z;
                    }
                }
                sum = sum + color;
            }
            if (k >= spf) break;
            start_sample(ps, S, pc, camS, xx, yy, uvx, uvy, k);
            k++;
            shadow = false;
            active = depth > 0;
            continue;
        }
        // ---- the single scene intersection of the loop ----
        HitT<R> h;
        h.hitdist = R(PT_MAXDIST);
        h.normal = v3<R>(R(0), R(0), R(0));
        h.materialID = R(0);
        h.lightID = R(-1);
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
    if constexpr (sizeof(R) == 4) {
        P.accum[pix] = accumulate(pc, sum, P.accum[pix]);
    } else {
        // Rendering's exposure (SC:1517), each sample's colour summed at full precision.
        const double exposure = (double)pc.apertureSize * (double)pc.apertureSize * (double)pc.ISO;
        double* s4 = P.sums + 4 * pix;
        s4[0] += (double)sum.x * exposure;
        s4[1] += (double)sum.y * exposure;
        s4[2] += (double)sum.z * exposure;
        s4[3] += (double)spf;
    }
}

}  // namespace
