// pt_export.cu — SaveRender's tonemap chain on the device (pt_export.cuh):
// W*H float4 XYZ in, W*H*3 bytes out.  HBM-bound: 16 B read and 3 B written
// per pixel; each thread converts four pixels and, when the output is
// 4-byte aligned, writes their 12 bytes as three 32-bit words.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/pt_cuda.h"
#include "pt_export.cuh"

namespace {

constexpr int kExportThreads = 256;

__global__ void __launch_bounds__(kExportThreads)
    export_rgb8_kernel(const float4* __restrict__ accum, uint32_t n, int tonemap, uint8_t* __restrict__ rgb,
                       bool words) {
    const uint32_t i = 4u * (blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    if (words && i + 4 <= n) {
        uint8_t b[12];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float4 c = accum[i + k];
            ptx_pixel(c.x, c.y, c.z, tonemap, b + 3 * k);
        }
        uint32_t* out = reinterpret_cast<uint32_t*>(rgb + 3 * (size_t)i);
#pragma unroll
        for (int w = 0; w < 3; w++)
            out[w] = (uint32_t)b[4 * w] | ((uint32_t)b[4 * w + 1] << 8) | ((uint32_t)b[4 * w + 2] << 16) |
                     ((uint32_t)b[4 * w + 3] << 24);
        return;
    }
    for (uint32_t p = i; p < n && p < i + 4; p++) {
        const float4 c = accum[p];
        ptx_pixel(c.x, c.y, c.z, tonemap, rgb + 3 * (size_t)p);
    }
}

}  // namespace

cudaError_t ptk_export_rgb8(const void* d_accum, int width, int height, int tonemap, void* d_rgb,
                            cudaStream_t stream) {
    const uint32_t n = (uint32_t)width * (uint32_t)height;
    const uint32_t threads = (n + 3) / 4;
    const bool words = (reinterpret_cast<uintptr_t>(d_rgb) & 3u) == 0;
    export_rgb8_kernel<<<(threads + kExportThreads - 1) / kExportThreads, kExportThreads, 0, stream>>>(
        static_cast<const float4*>(d_accum), n, tonemap, static_cast<uint8_t*>(d_rgb), words);
    return cudaGetLastError();
}

extern "C" int pt_export_rgb8_device(const void* d_accum, int width, int height, int tonemap, void* d_rgb,
                                     void* stream) {
    if (!d_accum || !d_rgb || width <= 0 || height <= 0 || tonemap < 0 || tonemap > 3 ||
        (long long)width * height >= (1ll << 31))
        return PT_ERR_INVALID;
    return ptk_export_rgb8(d_accum, width, height, tonemap, d_rgb, static_cast<cudaStream_t>(stream)) ==
                   cudaSuccess
               ? PT_OK
               : PT_ERR_CUDA;
}
