// pt_megakernel_analytic.cu — the plain megakernel's variants for scenes
// without SDFs (pt_megakernel_body.cuh).  Their shading calls the larger
// pt_mathf functions out of line: the loop stays small enough for the
// instruction cache, which these compute-bound variants measurably need.
#define PTM_OUTLINE
#include <cuda_runtime.h>

#include "pt_megakernel_body.cuh"

cudaError_t ptk_launch_megakernel_analytic(const KParams* params, int variant, dim3 grid, dim3 block,
                                           cudaStream_t stream) {
    switch (variant) {
        case 0: megakernel<false, 0><<<grid, block, 0, stream>>>(*params); break;
        case PT_FEAT_BOX: megakernel<false, PT_FEAT_BOX><<<grid, block, 0, stream>>>(*params); break;
        default: megakernel<false, PT_FEAT_ANALYTIC><<<grid, block, 0, stream>>>(*params); break;
    }
    return cudaGetLastError();
}
