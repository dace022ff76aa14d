// pt_export.cuh — SaveRender's per-pixel chain (src/pathtracer.cpp:3491-3518):
// Bradford E->D65 (:971-978), XYZ->linear sRGB (:980-987), max(0), the
// tonemap (Reinhard :989-997, ACES fit :999-1021, DEUCES :1023-1033), sRGB
// companding (:1061-1071) and byte truncation.  Shared by the host export
// (libpt_host) and the device kernel (libpt_cuda), with pt_mathf's exp and
// pow on both, so the two give the same bytes.
#pragma once

#include <stdint.h>

#include "../../include/pt_mathf.h"

#if defined(__CUDACC__)
#define PTX_FN static __device__ __forceinline__
#else
#define PTX_FN static inline
#endif

// glm: vec3 * mat3 (column-major) = dot with each column.
PTX_FN void ptx_row_times(float& x, float& y, float& z, const float* m) {
    const float a = x * m[0] + y * m[1] + z * m[2];
    const float b = x * m[3] + y * m[4] + z * m[5];
    const float c = x * m[6] + y * m[7] + z * m[8];
    x = a;
    y = b;
    z = c;
}

PTX_FN float ptx_tonemap(float x, int tonemap) {
    if (tonemap == 1) x = x / (1.0f + x);
    if (tonemap == 2) {
        const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f;
        x = x * (a * x + b) / (x * (c * x + d) + e);
    }
    if (tonemap == 3) x = ptm_expf(-0.25f / x);
    return x;
}

PTX_FN float ptx_srgb(float x) {
    x = (x < 0.0f) ? 0.0f : ((1.0f < x) ? 1.0f : x);
    if (x <= 0.0031308f) return 12.92f * x;
    return 1.055f * ptm_powf(x, 1.0f / 2.4f) - 0.055f;
}

PTX_FN uint8_t ptx_byte(float x) { return (uint8_t)(int)((double)x * 255.0); }

// One pixel: XYZ in, three bytes out.
PTX_FN void ptx_pixel(float x, float y, float z, int tonemap, uint8_t* out) {
    // IlluminantEToD65 and XYZToRGB, column-major as glm holds them.
    const float kEToD65[9] = {0.9531874f, -0.0265906f, 0.0238731f, -0.0382467f, 1.0288406f,
                              0.0094060f, 0.0026068f,  -0.0030332f, 1.0892565f};
    const float kXYZToRGB[9] = {3.2404542f, -1.5371385f, -0.4985314f, -0.9692660f, 1.8760108f,
                                0.0415560f, 0.0556434f,  -0.2040259f, 1.0572252f};
    ptx_row_times(x, y, z, kEToD65);
    ptx_row_times(x, y, z, kXYZToRGB);
    x = (x < 0.0f) ? 0.0f : x;  // glm::max(rgb, 0)
    y = (y < 0.0f) ? 0.0f : y;
    z = (z < 0.0f) ? 0.0f : z;
    out[0] = ptx_byte(ptx_srgb(ptx_tonemap(x, tonemap)));
    out[1] = ptx_byte(ptx_srgb(ptx_tonemap(y, tonemap)));
    out[2] = ptx_byte(ptx_srgb(ptx_tonemap(z, tonemap)));
}
