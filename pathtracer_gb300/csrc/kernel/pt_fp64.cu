// pt_fp64.cu — the FP64 reference renderer: the plain megakernel's
// per-pixel path loop (pt_megakernel_body.cuh) instantiated in double
// precision.  The path arithmetic is the same templates as the FP32 kernels
// (pt_path.cuh, pt_geometry.cuh) with R = double: every intermediate value
// carries 53 bits, transcendentals are CUDA's double-precision functions,
// the RNG draws the same 32-bit stream (converted exactly, so a draw never
// rounds up to 1.0), and the scene's values are the same floats widened.
// Images it renders are the references the FP32 method's error is measured
// against.  SDF text compiled at run time has no double form, so scenes with
// such snippets are refused by the host.
#include <cuda_runtime.h>

#include "pt_megakernel_body.cuh"

cudaError_t ptk_launch_fp64(const KParams* params, bool trace, cudaStream_t stream) {
    const int W = params->pc.resolution[0], H = params->pc.resolution[1];
    const dim3 block(PT_MK_BLOCK_X, PT_MK_BLOCK_Y);
    const dim3 grid((W + PT_MK_BLOCK_X - 1) / PT_MK_BLOCK_X, (H + PT_MK_BLOCK_Y - 1) / PT_MK_BLOCK_Y);
    if (trace) {
        megakernel<true, PT_FEAT_ALL, double><<<grid, block, 0, stream>>>(*params);
    } else {
        megakernel<false, PT_FEAT_ALL, double><<<grid, block, 0, stream>>>(*params);
    }
    return cudaGetLastError();
}
