// pt_scene_model.h — the in-memory scene, field for field the reference's
// scene structs (src/pathtracer.cpp:110-185).
#pragma once

#include <string>
#include <vector>

struct SphereD {
    float pos[3];
    float radius;
    int materialID, lightID;  // 1-based; lightID 0 = not emissive
};
struct PlaneD {
    float pos[3];
    int materialID, lightID;
};
struct BoxD {
    float pos[3], rotation[3], size[3];
    int materialID, lightID;
};
struct LensD {
    float pos[3], rotation[3];
    float radius, focalLength, thickness;
    bool isConverging;
    int materialID, lightID;
};
struct CyclideD {
    float pos[3], rotation[3], scale[3];
    float a, b, c, d, brad;
    int materialID, lightID;
};
struct SdfD {
    float pos[3], size[3];
    std::string source;   // GLSL text or "builtin:..." spec
    bool is_builtin_key;  // loaded from "builtin" (saved back under that key)
};
struct MaterialD {
    float reflection[3];  // peak wavelength, sigma, isInvert (0/1)
    // Full-form extension ("bsdf" key, not read by the reference):
    // PT_BSDF_* and its parameters (pt_cuda.h, pt_material_ext).
    int bsdf = 0;
    float bsdf_p[6] = {0, 0, 0, 0, 0, 0};
};
struct LightD {
    float emission[2];  // temperature, luminosity
};
struct ShotD {
    float pos[3];
    float angle[2];
};
struct CameraD {
    int ISO;
    float size, apertureSize, apertureDist, lensRadius, lensFocalLength, lensThickness, lensDistance;
};

// Scene-level full-form extensions ("environment", "spectral", "march" keys,
// not read by the reference): pt_scene_ext without the material table.
struct ExtD {
    bool sky = false;
    float sky_temperature = 0, sky_luminosity = 0;
    bool range = false;
    float lambda_min = 0, lambda_max = 0;
    bool analytic_cmf = false;
    bool march = false;
    int march_max_steps = 512;
    float march_epsilon = 1e-4f, march_max_distance = 0;
};

struct pt_scene {
    CameraD camera{};
    ExtD ext;
    std::vector<ShotD> shots;
    std::vector<SphereD> spheres;
    std::vector<PlaneD> planes;
    std::vector<BoxD> boxes;
    std::vector<LensD> lenses;
    std::vector<CyclideD> cyclides;
    std::vector<SdfD> sdfs;
    std::vector<MaterialD> materials;
    std::vector<LightD> lights;
};
