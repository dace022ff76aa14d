// pt_megakernel.h — host entry points of the megakernel translation unit.
#pragma once

#if !defined(__CUDACC_RTC__)
#include <cuda_runtime.h>
#endif

#include "pt_scene.cuh"

// Block shape of the plain megakernel: 16 x 8 pixels, one warp = 16 x 2 pixels.
#define PT_MK_BLOCK_X 16
#define PT_MK_BLOCK_Y 8
#define PT_MK_THREADS (PT_MK_BLOCK_X * PT_MK_BLOCK_Y)

#if !defined(__CUDACC_RTC__)
// Writes 9 floats per object (column-major RotationMatrix of its rotation;
// identity for spheres and planes) to d_out[9 * total_objects].
cudaError_t ptk_rotation_setup(const KScene* scene, float* d_out, cudaStream_t stream);

// One dispatch of the plain megakernel over params->pc.resolution.
cudaError_t ptk_launch_megakernel(const KParams* params, bool trace, cudaStream_t stream);
// One dispatch of the FP64 reference renderer (pt_fp64.cu): the same paths
// in double precision, adding exposed colour sums and sample counts to
// params->sums (4 doubles per pixel).
cudaError_t ptk_launch_fp64(const KParams* params, bool trace, cudaStream_t stream);
// The analytic-scene variants (PT_FEAT_* 0, BOX, ANALYTIC), from their own
// translation unit.
cudaError_t ptk_launch_megakernel_analytic(const KParams* params, int variant, dim3 grid, dim3 block,
                                           cudaStream_t stream);

// Evaluates a pt_mathf function over device arrays (verification hook):
// fn 0 sin, 1 cos, 2 exp, 3 log, 4 pow(x, y), 5 acos.
cudaError_t ptk_mathf_eval(int fn, const float* x, const float* y, float* out, int n, cudaStream_t stream);
// thritorius_intersect (which 0) or smooth_cuboid_intersect (1) per ray:
// rays6 origin + direction, hits6 the hit record in and out, flags the result.
cudaError_t ptk_quartic_surface_eval(int which, const float* rays6, float* hits6, int* flags, int n,
                                     cudaStream_t stream);
#endif
