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
#include "../pt_export.cuh"
#include "pt_scene_model.h"

namespace {

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
    for (size_t i = 0; i < n; i++) ptx_pixel(accum[4 * i], accum[4 * i + 1], accum[4 * i + 2], tonemap, rgb + 3 * i);
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
