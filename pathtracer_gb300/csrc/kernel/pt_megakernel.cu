// pt_megakernel.cu — the plain per-pixel spectral path tracer for sm_103a
// (pt_megakernel_body.cuh): its variants for SDF scenes and traced
// dispatches, with all math inlined, plus the per-upload rotation setup and
// the math verification kernel.  The analytic-scene variants live in
// pt_megakernel_analytic.cu.
#include <cuda_runtime.h>

#include "pt_megakernel_body.cuh"

namespace {

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
        case 5: r = ptm_acosf(x[i]); break;
        case 6: r = ptm_asinf(x[i]); break;
        case 7: r = ptm_atanf(x[i]); break;
        case 8: r = ptm_atan2f(x[i], y[i]); break;
        case 9: r = ptm_exp2f(x[i]); break;
        default: r = ptm_log2f(x[i]); break;
    }
    out[i] = r;
}
}  // namespace

namespace {
__global__ void quartic_surface_kernel(int which, const float* __restrict__ rays, float* __restrict__ hits,
                                       int* __restrict__ flags, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = rays + 6 * (size_t)i;
    float* hp = hits + 6 * (size_t)i;
    Hit h;
    h.hitdist = hp[0];
    h.normal = f3(hp[1], hp[2], hp[3]);
    h.materialID = hp[4];
    h.lightID = hp[5];
    const float3 o = f3(r[0], r[1], r[2]), d = f3(r[3], r[4], r[5]);
    const bool hit = (which == 0) ? thritorius_intersect(o, d, h) : smooth_cuboid_intersect(o, d, h);
    hp[0] = h.hitdist;
    hp[1] = h.normal.x;
    hp[2] = h.normal.y;
    hp[3] = h.normal.z;
    hp[4] = h.materialID;
    hp[5] = h.lightID;
    flags[i] = hit ? 1 : 0;
}
}  // namespace

cudaError_t ptk_quartic_surface_eval(int which, const float* rays6, float* hits6, int* flags, int n,
                                     cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    quartic_surface_kernel<<<(n + 127) / 128, 128, 0, stream>>>(which, rays6, hits6, flags, n);
    return cudaGetLastError();
}

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
    const int variant = pt_feature_variant(params->s.meta.n);
    if (variant != PT_FEAT_ALL) return ptk_launch_megakernel_analytic(params, variant, grid, block, stream);
    megakernel<false, PT_FEAT_ALL><<<grid, block, 0, stream>>>(*params);
    return cudaGetLastError();
}
