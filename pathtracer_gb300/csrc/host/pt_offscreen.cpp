// pt_offscreen.cpp — the offscreen progressive loop, the export tonemap and
// PPM writer, and an analytic CIE table for callers without the tabulated
// one.  Headless restatement of src/pathtracer.cpp (PT) :918-933, :971-1071,
// :3491-3518, :3965-4093.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

#include "../../../include/pt_host.h"
#include "pt_scene_model.h"

namespace {

struct v3 {
    float x, y, z;
};

// glm: vec3 * mat3 with mat3 given column-major = dot with each column.
v3 row_times(v3 c, const float m[9]) {
    return v3{c.x * m[0] + c.y * m[1] + c.z * m[2], c.x * m[3] + c.y * m[4] + c.z * m[5],
              c.x * m[6] + c.y * m[7] + c.z * m[8]};
}

// IlluminantEToD65 (Bradford), PT:971-978, and XYZToRGB, PT:980-987.
const float kEToD65[9] = {0.9531874f, -0.0265906f, 0.0238731f, -0.0382467f, 1.0288406f,
                          0.0094060f, 0.0026068f,  -0.0030332f, 1.0892565f};
const float kXYZToRGB[9] = {3.2404542f, -1.5371385f, -0.4985314f, -0.9692660f, 1.8760108f,
                            0.0415560f, 0.0556434f,  -0.2040259f, 1.0572252f};

float tonemap1(float x, int tonemap) {
    if (tonemap == 1) x = x / (1.0f + x);  // Reinhard, PT:989-997
    if (tonemap == 2) {                    // ACES filmic fit, PT:999-1021
        const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f;
        x = x * (a * x + b) / (x * (c * x + d) + e);
    }
    if (tonemap == 3) x = std::exp(-0.25f / x);  // DEUCES, PT:1023-1033
    return x;
}

// sRGBCompanding, PT:1061-1071.
float srgb_companding(float x) {
    x = (x < 0.0f) ? 0.0f : ((1.0f < x) ? 1.0f : x);  // std::clamp
    if (x <= 0.0031308f) {
        x = 12.92f * x;
    } else {
        x = 1.055f * std::pow(x, 1.0f / 2.4f) - 0.055f;
    }
    return x;
}

// g(x; mu, s1, s2) of the multi-lobe fit: a Gaussian with a different width
// on each side of its peak.
double lobe(double x, double mu, double s1, double s2) {
    const double s = x < mu ? s1 : s2;
    const double t = (x - mu) / s;
    return std::exp(-0.5 * t * t);
}

}  // namespace

extern "C" {

int pt_export_rgb8(const float* accum, int width, int height, int tonemap, uint8_t* rgb) {
    if (!accum || !rgb || width <= 0 || height <= 0) return PT_ERR_INVALID;
    const size_t n = (size_t)width * (size_t)height;
    for (size_t i = 0; i < n; i++) {
        v3 c{accum[4 * i], accum[4 * i + 1], accum[4 * i + 2]};
        c = row_times(c, kEToD65);
        c = row_times(c, kXYZToRGB);
        c = v3{(c.x < 0.0f) ? 0.0f : c.x, (c.y < 0.0f) ? 0.0f : c.y, (c.z < 0.0f) ? 0.0f : c.z};  // glm::max
        c = v3{tonemap1(c.x, tonemap), tonemap1(c.y, tonemap), tonemap1(c.z, tonemap)};
        c = v3{srgb_companding(c.x), srgb_companding(c.y), srgb_companding(c.z)};
        rgb[3 * i] = (uint8_t)(int)((double)c.x * 255.0);
        rgb[3 * i + 1] = (uint8_t)(int)((double)c.y * 255.0);
        rgb[3 * i + 2] = (uint8_t)(int)((double)c.z * 255.0);
    }
    return PT_OK;
}

int pt_save_ppm(const char* path, const uint8_t* rgb, int width, int height) {
    if (!path || !rgb || width <= 0 || height <= 0) return PT_ERR_INVALID;
    FILE* f = std::fopen(path, "wb");
    if (!f) return PT_ERR_INVALID;
    std::fprintf(f, "P6\n%d\n%d\n255\n", width, height);
    const size_t n = (size_t)width * (size_t)height * 3;
    const size_t w = std::fwrite(rgb, 1, n, f);
    const int rc = std::fclose(f);
    return (w == n && rc == 0) ? PT_OK : PT_ERR_INVALID;
}

void pt_cie_analytic_table(float out[PT_CIE_TABLE_SIZE]) {
    for (int i = 0; i < PT_CIE_TABLE_SIZE / 3; i++) {
        const double l = 360.0 + (double)i;
        const double x = 1.056 * lobe(l, 599.8, 37.9, 31.0) + 0.362 * lobe(l, 442.0, 16.0, 26.7) -
                         0.065 * lobe(l, 501.1, 20.4, 26.2);
        const double y = 0.821 * lobe(l, 568.8, 46.9, 40.5) + 0.286 * lobe(l, 530.9, 16.3, 31.1);
        const double z = 1.217 * lobe(l, 437.0, 11.8, 36.0) + 0.681 * lobe(l, 459.0, 26.0, 13.8);
        out[3 * i] = (float)x;
        out[3 * i + 1] = (float)y;
        out[3 * i + 2] = (float)z;
    }
}

// MainLoop with OFFSCREENRENDER (PT:3965-4093): frame += spf and
// currentSamples += spf per dispatch until currentSamples >= numSamples.
int pt_render_offscreen(pt_ctx* ctx, const pt_scene* scene, const float* cie, const pt_offscreen_opts* o,
                        float* accum_out, size_t accum_bytes, double* seconds_out) {
    if (!ctx || !scene || !cie || !o) return PT_ERR_INVALID;
    if (o->width <= 0 || o->height <= 0 || o->samplesPerFrame <= 0 || o->numSamples <= 0) return PT_ERR_INVALID;
    int rc = pt_scene_bind(ctx, scene, cie);
    if (rc != PT_OK) return rc;
    rc = pt_resize_accum(ctx, o->width, o->height);
    if (rc != PT_OK) return rc;
    pt_frame_state st{};
    st.width = o->width;
    st.height = o->height;
    st.samplesPerFrame = o->samplesPerFrame;
    st.FPS = 1.0f / 0.0166f;  // frameTime initial value, PT:1167
    st.persistence = 0.0625f;
    st.pathLength = o->pathLength;
    st.cameraShotIndex = o->cameraShotIndex;
    st.tonemap = o->tonemap;
    int frame = o->frameOffset;
    int currentSamples = 0;
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        frame += o->samplesPerFrame;
        currentSamples += o->samplesPerFrame;
        st.frame = frame;
        st.currentSamples = currentSamples;
        pt_push push;
        rc = pt_scene_push_constants(scene, &st, &push);
        if (rc != PT_OK) return rc;
        rc = pt_dispatch(ctx, &push);
        if (rc != PT_OK) return rc;
        if (currentSamples >= o->numSamples) break;
    }
    rc = pt_wait(ctx, UINT64_MAX);
    if (rc != PT_OK) return rc;
    const auto t1 = std::chrono::steady_clock::now();
    if (seconds_out) *seconds_out = std::chrono::duration<double>(t1 - t0).count();
    if (accum_out) rc = pt_read_accum(ctx, accum_out, accum_bytes);
    return rc;
}

}  // extern "C"
