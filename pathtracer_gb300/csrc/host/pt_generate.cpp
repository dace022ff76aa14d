// pt_generate.cpp — seeded synthetic render jobs (pt_host.h, pt_scene_generate).
//
// Stand-ins for a stream of user scenes: every job (scene, resolution,
// samples per pixel, path length) follows from a 64-bit seed through
// std::mt19937_64, whose output sequence the C++ standard fixes, and a few
// transforms written here with additions and multiplications only (no libm),
// so a seed gives the same scene on every platform.
//
// PT_GEN_SPHERES, PT_GEN_SDF and PT_GEN_SDF_VARIED are expressible in the
// reference's scene schema (src/pathtracer.cpp:110-185) and render with its
// unmodified method.  The reference's only surface model is the Lambertian
// Gaussian-spectrum BRDF (src/shader.comp:1030-1038, 1075-1091), so there
// the "mirror" and "dielectric" material classes of a job mix map to
// Lambertian spectra of their own: flat (sigma 1000) and inverted-bump.
// PT_GEN_SPHERES_FULL draws the same scenes (the same random stream) and
// gives those two classes their full-form surface models (extension
// "bsdf"): a conductor mirror of reflectance 0.9, and a Cauchy dielectric
// whose A in [1.4, 1.7] and B in [0.002, 0.008] um^2 follow from the
// inverted bump's two draws.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <random>
#include <string>

#include "../../../include/pt_host.h"
#include "pt_scene_model.h"

namespace {

struct Rng {
    std::mt19937_64 g;
    explicit Rng(uint64_t seed) : g(seed) {}
    // [0, 1) with 53 random bits.
    double u() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }
    double range(double a, double b) { return a + (b - a) * u(); }
    // Integer in [0, n) (n small: the modulo bias is below 2^-58).
    uint32_t below(uint32_t n) { return (uint32_t)(g() % n); }
    // Approximately standard normal: Irwin-Hall sum of 12 uniforms minus 6.
    double normal() {
        double s = 0.0;
        for (int i = 0; i < 12; i++) s += u();
        return s - 6.0;
    }
};

// e^x for |x| <= 8 from the Taylor series of e^(x/16), squared four times.
double exp_series(double x) {
    const double y = x / 16.0;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 14; k++) {
        term = term * y / (double)k;
        sum += term;
    }
    for (int i = 0; i < 4; i++) sum *= sum;
    return sum;
}

constexpr double kLn2 = 0.69314718055994530942;

// Camera block of the reference's default scene (lens, sensor, aperture).
void default_camera(pt_scene& S, float px, float py, float pz, float yaw, float pitch) {
    S.camera.ISO = 1600;
    S.camera.size = 0.057f;
    S.camera.apertureSize = 0.0025f;
    S.camera.apertureDist = 0.049f;
    S.camera.lensRadius = 0.01f;
    S.camera.lensFocalLength = 0.03f;
    S.camera.lensThickness = 0.0f;
    S.camera.lensDistance = 0.05f;
    ShotD shot{};
    shot.pos[0] = px;
    shot.pos[1] = py;
    shot.pos[2] = pz;
    shot.angle[0] = yaw;
    shot.angle[1] = pitch;
    S.shots.push_back(shot);
}

int add_material(pt_scene& S, float peak, float sigma, bool invert) {
    MaterialD m{};
    m.reflection[0] = peak;
    m.reflection[1] = sigma;
    m.reflection[2] = invert ? 1.0f : 0.0f;
    S.materials.push_back(m);
    return (int)S.materials.size();  // 1-based, as objects reference materials
}

int add_light(pt_scene& S, float temperature, float luminosity) {
    LightD l{};
    l.emission[0] = temperature;
    l.emission[1] = luminosity;
    S.lights.push_back(l);
    return (int)S.lights.size();
}

void add_sphere(pt_scene& S, float x, float y, float z, float r, int material, int light) {
    SphereD s{};
    s.pos[0] = x;
    s.pos[1] = y;
    s.pos[2] = z;
    s.radius = r;
    s.materialID = material;
    s.lightID = light;
    S.spheres.push_back(s);
}

// 4-64 spheres (centres uniform in [-2,2]^3, radii lognormal(-1.5, 0.5)
// clamped to [0.03, 1]) on a ground plane at y = -2, lit by one blackbody
// sphere light at 3000-9000 K; resolution uniform over {128, 256, 512,
// 1024}^2, samples per pixel log-uniform over [4, 256], path length 8.
void spheres_job(Rng& r, pt_scene& S, pt_job_spec& spec, bool full) {
    static const int kRes[4] = {128, 256, 512, 1024};
    const int res = kRes[r.below(4)];
    spec.width = spec.height = res;
    spec.spp = (int)(4.0 * exp_series(6.0 * kLn2 * r.u()) + 0.5);
    spec.pathLength = 8;
    spec.sdf_kind = PT_SDF_NONE;
    const int n = 4 + (int)r.below(61);
    spec.objects = n;
    default_camera(S, 0.0f, 1.0f, 8.0f, 180.0f, -7.125016f);  // looking at the origin
    for (int i = 0; i < n; i++) {
        const float x = (float)r.range(-2.0, 2.0), y = (float)r.range(-2.0, 2.0), z = (float)r.range(-2.0, 2.0);
        double rad = exp_series(-1.5 + 0.5 * r.normal());
        if (rad < 0.03) rad = 0.03;
        if (rad > 1.0) rad = 1.0;
        int mat;
        switch (r.below(3)) {
            case 0:  // Gaussian-bump Lambertian
                mat = add_material(S, (float)r.range(400.0, 700.0), (float)r.range(4.0, 12.0), false);
                break;
            case 1:  // "mirror" class: flat spectrum
                mat = add_material(S, 550.0f, 1000.0f, false);
                if (full) {
                    S.materials.back().bsdf = PT_BSDF_MIRROR;
                    S.materials.back().bsdf_p[0] = 0.9f;
                }
                break;
            default: {  // "dielectric" class: inverted bump
                mat = add_material(S, (float)r.range(400.0, 700.0), (float)r.range(6.0, 12.0), true);
                if (full) {
                    MaterialD& m = S.materials.back();
                    m.bsdf = PT_BSDF_CAUCHY;
                    m.bsdf_p[0] = 1.4f + 0.3f * (m.reflection[0] - 400.0f) / 300.0f;
                    m.bsdf_p[1] = 0.002f + 0.006f * (m.reflection[1] - 6.0f) / 6.0f;
                }
                break;
            }
        }
        add_sphere(S, x, y, z, (float)rad, mat, 0);
    }
    const int ground = add_material(S, 550.0f, 1000.0f, false);
    PlaneD p{};
    p.pos[1] = -2.0f;
    p.materialID = ground;
    p.lightID = 0;
    S.planes.push_back(p);
    const int lmat = add_material(S, 550.0f, 1000.0f, false);
    const float temperature = (float)r.range(3000.0, 9000.0);
    const int light = add_light(S, temperature, (float)r.range(15.0, 40.0));
    add_sphere(S, (float)r.range(-2.0, 2.0), (float)r.range(3.0, 4.0), (float)r.range(-2.0, 2.0),
               (float)r.range(0.4, 0.8), lmat, light);
}

// GLSL of a mandelbulb of any power (the spherical-coordinate form: r^n,
// angles times n), `iter` iterations, bailout 2.
std::string mandelbulb_glsl(double power, int iter) {
    char pw[32];
    std::snprintf(pw, sizeof pw, "%.2f", power);
    return std::string("// Mandelbulb of power ") + pw + ", " + std::to_string(iter) +
           " iterations (spherical coordinates).\n"
           "const float POWER = " + pw + ";\n"
           "float sdf(vec3 p)\n{\n"
           "    vec3 z = p;\n    float dr = 1.0;\n    float r = length(z);\n"
           "    for (int i = 0; i < " + std::to_string(iter) + "; i++) {\n"
           "        if (r > 2.0) break;\n"
           "        float theta = acos(clamp(z.y / r, -1.0, 1.0)) * POWER;\n"
           "        float phi = atan(z.z, z.x) * POWER;\n"
           "        dr = pow(r, POWER - 1.0) * POWER * dr + 1.0;\n"
           "        float zr = pow(r, POWER);\n"
           "        z = zr * vec3(sin(theta) * cos(phi), cos(theta), sin(theta) * sin(phi)) + p;\n"
           "        r = length(z);\n    }\n"
           "    return 0.5 * log(r) * r / dr;\n}\n"
           "float sdfmaterial(vec3 p)\n{\n    float f = dot(p, p);\n    return mix(0.0, 1.0, f / (0.8 + f));\n}\n";
}

// GLSL of a Menger sponge with `levels` levels of holes (unit half-size).
std::string menger_glsl(int levels) {
    return "// Menger sponge, " + std::to_string(levels) + " levels.\n"
           "float box(vec3 p, vec3 b)\n{\n    vec3 q = abs(p) - b;\n"
           "    return length(max(q, 0.0)) + min(max(q.x, max(q.y, q.z)), 0.0);\n}\n"
           "float sdf(vec3 p)\n{\n    float d = box(p, vec3(1.0));\n    float s = 1.0;\n"
           "    for (int m = 0; m < " + std::to_string(levels) + "; m++) {\n"
           "        vec3 a = mod(p * s, 2.0) - 1.0;\n        s *= 3.0;\n"
           "        vec3 h = abs(1.0 - 3.0 * abs(a));\n"
           "        float c = (min(max(h.x, h.y), min(max(h.y, h.z), max(h.z, h.x))) - 1.0) / s;\n"
           "        d = max(d, c);\n    }\n    return d;\n}\n"
           "float sdfmaterial(vec3 p)\n{\n    return 2.0;\n}\n";
}

// One SDF plug-in (mandelbulb, menger or blob, with its own material
// constants) over a ground plane, under a sky sphere and a sun sphere, both
// blackbody emitters; resolution uniform over {256, 512, 1024}^2; samples per
// pixel open (refined until a target error), path length 8.  The plug-ins'
// iteration counts and powers are those of the reference snippets, or with
// `varied` drawn per job (GLSL text compiled at run time).
void sdf_job(Rng& r, pt_scene& S, pt_job_spec& spec, bool varied) {
    static const int kRes[3] = {256, 512, 1024};
    const int res = kRes[r.below(3)];
    spec.width = spec.height = res;
    spec.spp = 0;
    spec.pathLength = 8;
    spec.objects = 1;
    default_camera(S, 0.0f, 2.0f, 4.5f, 180.0f, -12.528808f);  // looking at (0, 1, 0)
    // Materials 1-3 (0-based 0-2 inside the plug-ins): three random bumps.
    for (int i = 0; i < 3; i++) add_material(S, (float)r.range(420.0, 680.0), (float)r.range(5.0, 12.0), false);
    SdfD d{};
    d.pos[1] = 1.0f;
    d.is_builtin_key = true;
    switch (r.below(3)) {
        case 0:
            spec.sdf_kind = PT_SDF_MANDELBULB;
            d.size[0] = d.size[1] = d.size[2] = 2.5f;
            d.pos[1] = 1.15f;
            d.source = "builtin:mandelbulb:0,1";
            if (varied) {
                const double power = r.range(4.0, 10.0);
                d.source = mandelbulb_glsl(power, 4 + (int)r.below(3));
                d.is_builtin_key = false;
                spec.sdf_kind = PT_SDF_CUSTOM;
            }
            break;
        case 1:
            spec.sdf_kind = PT_SDF_MENGER;
            d.size[0] = d.size[1] = d.size[2] = 2.0f;
            d.source = "builtin:menger:" + std::to_string(r.below(3));
            if (varied) {
                d.source = menger_glsl(3 + (int)r.below(3));
                d.is_builtin_key = false;
                spec.sdf_kind = PT_SDF_CUSTOM;
            }
            break;
        default:
            spec.sdf_kind = PT_SDF_BLOB;
            d.size[0] = 3.0f;
            d.size[1] = 4.0f;
            d.size[2] = 3.0f;
            d.source = "builtin:blob:0,1,2";
            break;
    }
    S.sdfs.push_back(d);
    const int ground = add_material(S, 550.0f, 1000.0f, false);
    PlaneD p{};
    p.materialID = ground;
    p.lightID = 0;
    S.planes.push_back(p);
    const int white = add_material(S, 550.0f, 1000.0f, false);
    const int sky = add_light(S, (float)r.range(3000.0, 9000.0), 0.6f);
    add_sphere(S, 0.0f, 0.0f, 0.0f, 50.0f, white, sky);
    const int sun = add_light(S, (float)r.range(3000.0, 9000.0), 10.0f);
    add_sphere(S, (float)r.range(-4.0, 4.0), 5.0f, (float)r.range(-4.0, 4.0), 1.0f, white, sun);
}

}  // namespace

extern "C" {

int pt_scene_generate(int kind, uint64_t seed, pt_scene** out, pt_job_spec* spec) {
    if (!out || !spec ||
        (kind != PT_GEN_SPHERES && kind != PT_GEN_SDF && kind != PT_GEN_SDF_VARIED && kind != PT_GEN_SPHERES_FULL))
        return PT_ERR_INVALID;
    *out = nullptr;
    pt_scene* S = new (std::nothrow) pt_scene();
    if (!S) return PT_ERR_OOM;
    std::memset(spec, 0, sizeof *spec);
    spec->kind = kind;
    spec->seed = seed;
    Rng r(seed);
    try {
        if (kind == PT_GEN_SPHERES || kind == PT_GEN_SPHERES_FULL) {
            spheres_job(r, *S, *spec, kind == PT_GEN_SPHERES_FULL);
        } else {
            sdf_job(r, *S, *spec, kind == PT_GEN_SDF_VARIED);
        }
    } catch (const std::bad_alloc&) {
        delete S;
        return PT_ERR_OOM;
    }
    *out = S;
    return PT_OK;
}

}  // extern "C"
