/* user_sdfs.c — TEST INFRASTRUCTURE ONLY: hand restatements, in C, of the
 * GLSL SDF snippets the tests use for scenes beyond the reference's four
 * shipped ones (their GLSL text is in tests/user_snippets.py).  The product
 * compiles such text at run time (pt_glsl_translate + NVRTC); the oracle
 * renders the same scene with these functions registered per SDF slot
 * (pto_set_user_sdf), so a parity failure points at the translation or the
 * run-time compile, not at a shared helper.
 *
 * Arithmetic follows GLSL's meaning of each expression in source order, with
 * the shader's conventions: single precision, no contraction (built with
 * -ffp-contract=off), mod(a, b) = a - b * floor(a / b), length = sqrt(dot),
 * and the transcendentals through the shared pt_mathf routines (tan as sin / cos
 * of one reduction). */
#include <math.h>
#include <stdint.h>

#include "../include/pt_mathf.h"

/* Work counters of the restatements below (loop iterations by snippet),
 * summed over all threads while counting is on; the work model of a
 * workload reads them beside the oracle's own counters. */
enum { USER_C_BULB8_ITERS = 0, USER_C_MANDELBULB_ITERS, USER_C_COUNT };
uint64_t user_counters[USER_C_COUNT];
static int g_counting;

void user_count(int on) {
    g_counting = on;
    for (int k = 0; k < USER_C_COUNT; k++) user_counters[k] = 0;
}

static void user_add(int k, int n) {
    if (g_counting) __atomic_fetch_add(&user_counters[k], (uint64_t)n, __ATOMIC_RELAXED);
}

/* ---- "twisted torus": torus (R 0.8, r 0.25) with a sin ripple ---------- */
static float torus(float px, float py, float pz, float tx, float ty, float* ring) {
    const float qx = sqrtf(px * px + pz * pz) - tx;
    const float qy = py;
    *ring = qx;
    return sqrtf(qx * qx + qy * qy) - ty;
}

float user_torus_sdf(float x, float y, float z) {
    float ring;
    const float d = torus(x, y, z, 0.8f, 0.25f, &ring);
    return d + 0.02f * ptm_sinf(8.0f * x) * ptm_sinf(8.0f * z);
}

float user_torus_material(float x, float y, float z) {
    float ring;
    (void)torus(x, y, z, 0.8f, 0.25f, &ring);
    return ring > 0.0f ? 2.0f : 3.0f;
}

/* ---- "lattice": rounded cubes repeated every 0.6, clipped to a box ----- */
static float box(float px, float py, float pz, float bx, float by, float bz) {
    const float qx = fabsf(px) - bx, qy = fabsf(py) - by, qz = fabsf(pz) - bz;
    const float mx = fmaxf(qx, 0.0f), my = fmaxf(qy, 0.0f), mz = fmaxf(qz, 0.0f);
    return sqrtf(mx * mx + my * my + mz * mz) + fminf(fmaxf(qx, fmaxf(qy, qz)), 0.0f);
}

static float glsl_mod(float a, float b) { return a - b * floorf(a / b); }

float user_lattice_sdf(float x, float y, float z) {
    const float c = 0.6f;
    const float h = 0.5f * c;
    const float rx = glsl_mod(x + h, c) - h;
    const float ry = glsl_mod(y + h, c) - h;
    const float rz = glsl_mod(z + h, c) - h;
    return fmaxf(box(rx, ry, rz, 0.18f, 0.18f, 0.18f) - 0.04f, box(x, y, z, 0.9f, 0.9f, 0.9f));
}

float user_lattice_material(float x, float y, float z) {
    (void)x;
    (void)z;
    return floorf(fminf(fmaxf(y + 1.0f, 0.0f), 1.5f)) + 1.0f;
}

/* ---- "spiral": a ring twisted by its polar angle ----------------------- */
float user_spiral_sdf(float x, float y, float z) {
    const float a = ptm_atan2f(z, x);
    const float r = sqrtf(x * x + z * z);
    const float twist = 0.25f * ptm_sinf(3.0f * a + 2.0f * y);
    const float qx = r - 0.7f - 0.1f * twist;
    const float qy = y;
    const float k = ptm_exp2f(-2.0f) + 0.01f * ptm_log2f(1.0f + r);
    float s, c;
    ptm_sincosf(0.3f * y, &s, &c);
    return sqrtf(qx * qx + qy * qy) - 0.2f - k * 0.1f + 0.02f * ptm_asinf(fminf(fmaxf(y, -1.0f), 1.0f)) +
           0.001f * (s / c);
}

float user_spiral_material(float x, float y, float z) {
    (void)y;
    (void)z;
    return roundf(ptm_atanf(x) + 2.0f);
}

/* ---- "bulb8": power-8 mandelbulb, 12 iterations, bailout 2 ------------
 * The SDF of pathtracer_gb300/scenes/mandelbulb12_plane.json: z -> z^8 + p
 * in spherical form with the 8-fold angles from Chebyshev polynomials of the
 * cosines (cos 8a = T8(cos a), sin 8a = sin a * U7(cos a)). */
typedef struct {
    float t8, u7;
} cheb8_t;

static cheb8_t cheb8(float c) {
    const float c2 = c * c;
    cheb8_t o;
    o.t8 = PTM_FMA(PTM_FMA(PTM_FMA(PTM_FMA(128.0f, c2, -256.0f), c2, 160.0f), c2, -32.0f), c2, 1.0f);
    o.u7 = PTM_FMA(PTM_FMA(PTM_FMA(128.0f, c2, -192.0f), c2, 80.0f), c2, -8.0f) * c;
    return o;
}

float user_bulb8_sdf(float x, float y, float z) {
    float zx = x, zy = y, zz = z;
    float r = sqrtf(zx * zx + zy * zy + zz * zz);
    float dr = 1.0f;
    int i;
    for (i = 0; i < 12; i++) {
        if (r > 2.0f) break;
        const float r2 = r * r;
        const float r4 = r2 * r2;
        dr = 8.0f * (r4 * r2 * r) * dr + 1.0f;
        const float l = sqrtf(zx * zx + zz * zz);
        const float q = 1.0f / (l * r); /* one division for 1/l and 1/r */
        const float il = r * q;
        const float ir = l * q;
        const cheb8_t a = cheb8(zz * il);
        const cheb8_t b = cheb8(zy * ir);
        const float st8 = a.u7 * (zx * il);
        const float sp8 = b.u7 * (l * ir);
        const float r8 = r4 * r4;
        zx = r8 * (st8 * sp8) + x;
        zy = r8 * b.t8 + y;
        zz = r8 * (a.t8 * sp8) + z;
        r = sqrtf(zx * zx + zy * zy + zz * zz);
    }
    user_add(USER_C_BULB8_ITERS, i);
    return 0.5f * ptm_logf(r) * r / dr;
}

float user_bulb8_material(float x, float y, float z) {
    const float f = x * x + y * y + z * z;
    const float t = f / (0.8f + f);
    return 4.0f * (1.0f - t) + 3.0f * t;
}

/* ---- generated scenes (PT_GEN_SDF_VARIED): mandelbulb of any power ------
 * The text pt_scene_generate writes for a mandelbulb of power `power` and
 * `iter` iterations; the parameters are set with user_mandelbulb_set. */
static float g_mb_power = 8.0f;
static int g_mb_iter = 4;

void user_mandelbulb_set(float power, int iter) {
    g_mb_power = power;
    g_mb_iter = iter;
}

float user_mandelbulb_sdf(float x, float y, float z) {
    float zx = x, zy = y, zz = z;
    float dr = 1.0f;
    float r = sqrtf(zx * zx + zy * zy + zz * zz);
    int i;
    for (i = 0; i < g_mb_iter; i++) {
        if (r > 2.0f) break;
        const float theta = ptm_acosf(fminf(fmaxf(zy / r, -1.0f), 1.0f)) * g_mb_power;
        const float phi = ptm_atan2f(zz, zx) * g_mb_power;
        dr = ptm_powf(r, g_mb_power - 1.0f) * g_mb_power * dr + 1.0f;
        const float zr = ptm_powf(r, g_mb_power);
        const float st = ptm_sinf(theta), ct = ptm_cosf(theta), sp = ptm_sinf(phi), cp = ptm_cosf(phi);
        zx = zr * (st * cp) + x;
        zy = zr * ct + y;
        zz = zr * (st * sp) + z;
        r = sqrtf(zx * zx + zy * zy + zz * zz);
    }
    user_add(USER_C_MANDELBULB_ITERS, i);
    return 0.5f * ptm_logf(r) * r / dr;
}

float user_mandelbulb_material(float x, float y, float z) {
    const float f = x * x + y * y + z * z;
    const float t = f / (0.8f + f);
    return 0.0f * (1.0f - t) + 1.0f * t;
}

/* ---- generated scenes: Menger sponge with `levels` levels ---------------- */
static int g_menger_levels = 3;

void user_menger_set(int levels) { g_menger_levels = levels; }

float user_menger_sdf(float x, float y, float z) {
    float d = box(x, y, z, 1.0f, 1.0f, 1.0f);
    float s = 1.0f;
    for (int m = 0; m < g_menger_levels; m++) {
        const float ax = glsl_mod(x * s, 2.0f) - 1.0f;
        const float ay = glsl_mod(y * s, 2.0f) - 1.0f;
        const float az = glsl_mod(z * s, 2.0f) - 1.0f;
        s *= 3.0f;
        const float hx = fabsf(1.0f - 3.0f * fabsf(ax));
        const float hy = fabsf(1.0f - 3.0f * fabsf(ay));
        const float hz = fabsf(1.0f - 3.0f * fabsf(az));
        const float c = (fminf(fmaxf(hx, hy), fminf(fmaxf(hy, hz), fmaxf(hz, hx))) - 1.0f) / s;
        d = fmaxf(d, c);
    }
    return d;
}

float user_menger_material(float x, float y, float z) {
    (void)x;
    (void)y;
    (void)z;
    return 2.0f;
}

/* ---- "fbm terrain": 8-octave value-noise height field ------------------
 * The terrain SDF of pathtracer_gb300/scenes/menger_terrain_full.json: value
 * noise on the integer lattice of the xz plane (an integer hash of the
 * lattice point and the seed 7 to [0, 1)), smoothstep-weighted bilinear
 * interpolation, 8 octaves of doubling frequency and halving amplitude,
 * height scale 0.3; distance = half the vertical gap to the surface. */
static float fbm_lattice(int ix, int iz) {
    uint32_t h = (uint32_t)ix * 1597334677u + (uint32_t)iz * 3812015801u + 7u * 2654435761u;
    h = (h ^ (h >> 16u)) * 2246822519u;
    h = (h ^ (h >> 13u)) * 3266489917u;
    h = h ^ (h >> 16u);
    return (float)(h >> 8u) * (1.0f / 16777216.0f);
}

static float fbm_value_noise(float qx, float qz) {
    const float ix = floorf(qx), iz = floorf(qz);
    const float fx = qx - ix, fz = qz - iz;
    const float ux = fx * fx * (3.0f - 2.0f * fx), uz = fz * fz * (3.0f - 2.0f * fz);
    const int jx = (int)ix, jz = (int)iz;
    const float a = fbm_lattice(jx, jz);
    const float b = fbm_lattice(jx + 1, jz);
    const float c = fbm_lattice(jx, jz + 1);
    const float d = fbm_lattice(jx + 1, jz + 1);
    const float ab = a * (1.0f - ux) + b * ux;
    const float cd = c * (1.0f - ux) + d * ux;
    return ab * (1.0f - uz) + cd * uz;
}

static float fbm_height(float x, float z) {
    float h = 0.0f, amp = 0.5f, freq = 1.0f;
    for (int o = 0; o < 8; o++) {
        h += amp * (2.0f * fbm_value_noise(x * freq, z * freq) - 1.0f);
        freq *= 2.0f;
        amp *= 0.5f;
    }
    return 0.3f * h;
}

float user_fbm_sdf(float x, float y, float z) { return 0.5f * (y - fbm_height(x, z)); }

float user_fbm_material(float x, float y, float z) {
    (void)x;
    (void)y;
    (void)z;
    return 0.0f;
}
