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

struct pt_scene {
    CameraD camera{};
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
