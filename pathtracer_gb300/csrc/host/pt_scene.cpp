// pt_scene.cpp — scene model, JSON load/save, uniform-buffer packing and push
// constants: the headless restatement of src/pathtracer.cpp (PT) :110-218,
// :2576-2858, :3642-3834.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../../include/pt_host.h"
#include "pt_json.h"
#include "pt_scene_model.h"

using ptjson::Value;

namespace {

struct LoadError {
    std::string msg;
};

const Value& req(const Value& v, const char* key, const char* where) {
    const Value* x = v.find(key);
    if (!x || x->type == Value::Null) throw LoadError{std::string(where) + ": missing \"" + key + "\""};
    return *x;
}
float num_f(const Value& v, const std::string& where) {
    if (!v.is_number()) throw LoadError{where + ": expected a number"};
    return (float)v.number();
}
int num_i(const Value& v, const std::string& where) {
    if (v.type == Value::Int) return (int)v.i;
    if (v.type == Value::Bool) return v.b ? 1 : 0;
    if (v.type == Value::Float) return (int)v.d;  // truncation, like a static_cast
    throw LoadError{where + ": expected an integer"};
}
bool num_b(const Value& v, const std::string& where) {
    if (v.type == Value::Bool) return v.b;
    if (v.type == Value::Int) return v.i != 0;
    if (v.type == Value::Float) return v.d != 0.0;
    throw LoadError{where + ": expected a boolean"};
}
void vec_f(const Value& v, float* out, int n, const std::string& where) {
    if (v.type != Value::Array || (int)v.arr.size() < n) throw LoadError{where + ": expected an array of " + std::to_string(n)};
    for (int i = 0; i < n; i++) out[i] = num_f(v.arr[(size_t)i], where);
}
// `scene["sphere"].size()` on a missing key is 0 in the reference.
const std::vector<Value>& list(const Value& root, const char* key) {
    static const std::vector<Value> empty;
    const Value* x = root.find(key);
    if (!x || x->type == Value::Null) return empty;
    if (x->type != Value::Array) throw LoadError{std::string(key) + ": expected an array"};
    return x->arr;
}

// A material's "bsdf" object (full-form extension): {"type": "flat",
// "albedo"}, {"type": "smooth", "base", "amplitude", "center", "width"},
// {"type": "mirror", "reflectance"}, {"type": "cauchy", "A", "B"},
// {"type": "sellmeier", "B": [3], "C": [3]}.
void load_bsdf(const Value& b, MaterialD& d) {
    if (b.type == Value::Null) return;
    const Value& t = req(b, "type", "material.bsdf");
    if (t.type != Value::String) throw LoadError{"material.bsdf.type: expected a string"};
    const std::string& k = t.s;
    if (k == "flat") {
        d.bsdf = PT_BSDF_FLAT;
        d.bsdf_p[0] = num_f(req(b, "albedo", "material.bsdf"), "material.bsdf.albedo");
    } else if (k == "smooth") {
        d.bsdf = PT_BSDF_SMOOTH;
        d.bsdf_p[0] = num_f(req(b, "base", "material.bsdf"), "material.bsdf.base");
        d.bsdf_p[1] = num_f(req(b, "amplitude", "material.bsdf"), "material.bsdf.amplitude");
        d.bsdf_p[2] = num_f(req(b, "center", "material.bsdf"), "material.bsdf.center");
        d.bsdf_p[3] = num_f(req(b, "width", "material.bsdf"), "material.bsdf.width");
    } else if (k == "mirror") {
        d.bsdf = PT_BSDF_MIRROR;
        d.bsdf_p[0] = num_f(req(b, "reflectance", "material.bsdf"), "material.bsdf.reflectance");
    } else if (k == "cauchy") {
        d.bsdf = PT_BSDF_CAUCHY;
        d.bsdf_p[0] = num_f(req(b, "A", "material.bsdf"), "material.bsdf.A");
        d.bsdf_p[1] = num_f(req(b, "B", "material.bsdf"), "material.bsdf.B");
    } else if (k == "sellmeier") {
        d.bsdf = PT_BSDF_SELLMEIER;
        vec_f(req(b, "B", "material.bsdf"), d.bsdf_p, 3, "material.bsdf.B");
        vec_f(req(b, "C", "material.bsdf"), d.bsdf_p + 3, 3, "material.bsdf.C");
    } else if (k == "reference") {
        d.bsdf = PT_BSDF_REFERENCE;
    } else {
        throw LoadError{"material.bsdf.type: unknown \"" + k + "\""};
    }
}

void load(const Value& root, pt_scene& S) {
    if (root.type != Value::Object) throw LoadError{"scene: expected an object"};
    // Camera, PT:2576-2613.
    const Value& cam = req(root, "camera", "scene");
    const int nshots = num_i(req(cam, "numShots", "camera"), "camera.numShots");
    if (nshots < 0) throw LoadError{"camera.numShots: negative"};
    const Value& positions = req(cam, "position", "camera");
    const Value& angles = req(cam, "angle", "camera");
    S.shots.resize((size_t)nshots);
    for (int i = 0; i < nshots; i++) {
        if (positions.type != Value::Array || angles.type != Value::Array || (int)positions.arr.size() <= i ||
            (int)angles.arr.size() <= i)
            throw LoadError{"camera: fewer positions/angles than numShots"};
        vec_f(positions.arr[(size_t)i], S.shots[(size_t)i].pos, 3, "camera.position");
        vec_f(angles.arr[(size_t)i], S.shots[(size_t)i].angle, 2, "camera.angle");
    }
    S.camera.ISO = num_i(req(cam, "ISO", "camera"), "camera.ISO");
    S.camera.size = num_f(req(cam, "size", "camera"), "camera.size");
    S.camera.apertureSize = num_f(req(cam, "apertureSize", "camera"), "camera.apertureSize");
    S.camera.apertureDist = num_f(req(cam, "apertureDistance", "camera"), "camera.apertureDistance");
    S.camera.lensRadius = num_f(req(cam, "lensRadius", "camera"), "camera.lensRadius");
    S.camera.lensFocalLength = num_f(req(cam, "lensFocalLength", "camera"), "camera.lensFocalLength");
    S.camera.lensThickness = num_f(req(cam, "lensThickness", "camera"), "camera.lensThickness");
    S.camera.lensDistance = num_f(req(cam, "lensDistance", "camera"), "camera.lensDistance");

    // Objects, PT:2615-2722.
    for (const Value& o : list(root, "sphere")) {
        SphereD d{};
        vec_f(req(o, "position", "sphere"), d.pos, 3, "sphere.position");
        d.radius = num_f(req(o, "radius", "sphere"), "sphere.radius");
        d.materialID = num_i(req(o, "materialID", "sphere"), "sphere.materialID");
        d.lightID = num_i(req(o, "lightID", "sphere"), "sphere.lightID");
        S.spheres.push_back(d);
    }
    for (const Value& o : list(root, "plane")) {
        PlaneD d{};
        vec_f(req(o, "position", "plane"), d.pos, 3, "plane.position");
        d.materialID = num_i(req(o, "materialID", "plane"), "plane.materialID");
        d.lightID = num_i(req(o, "lightID", "plane"), "plane.lightID");
        S.planes.push_back(d);
    }
    for (const Value& o : list(root, "box")) {
        BoxD d{};
        vec_f(req(o, "position", "box"), d.pos, 3, "box.position");
        vec_f(req(o, "rotation", "box"), d.rotation, 3, "box.rotation");
        vec_f(req(o, "size", "box"), d.size, 3, "box.size");
        d.materialID = num_i(req(o, "materialID", "box"), "box.materialID");
        d.lightID = num_i(req(o, "lightID", "box"), "box.lightID");
        S.boxes.push_back(d);
    }
    for (const Value& o : list(root, "lens")) {
        LensD d{};
        vec_f(req(o, "position", "lens"), d.pos, 3, "lens.position");
        vec_f(req(o, "rotation", "lens"), d.rotation, 3, "lens.rotation");
        d.radius = num_f(req(o, "radius", "lens"), "lens.radius");
        d.focalLength = num_f(req(o, "focalLength", "lens"), "lens.focalLength");
        d.thickness = num_f(req(o, "thickness", "lens"), "lens.thickness");
        d.isConverging = num_b(req(o, "isConverging", "lens"), "lens.isConverging");
        d.materialID = num_i(req(o, "materialID", "lens"), "lens.materialID");
        d.lightID = num_i(req(o, "lightID", "lens"), "lens.lightID");
        S.lenses.push_back(d);
    }
    for (const Value& o : list(root, "cyclide")) {
        CyclideD d{};
        vec_f(req(o, "position", "cyclide"), d.pos, 3, "cyclide.position");
        vec_f(req(o, "rotation", "cyclide"), d.rotation, 3, "cyclide.rotation");
        vec_f(req(o, "scale", "cyclide"), d.scale, 3, "cyclide.scale");
        d.a = num_f(req(o, "a", "cyclide"), "cyclide.a");
        d.b = num_f(req(o, "b", "cyclide"), "cyclide.b");
        d.c = num_f(req(o, "c", "cyclide"), "cyclide.c");
        d.d = num_f(req(o, "d", "cyclide"), "cyclide.d");
        d.brad = num_f(req(o, "boundingRadius", "cyclide"), "cyclide.boundingRadius");
        d.materialID = num_i(req(o, "materialID", "cyclide"), "cyclide.materialID");
        d.lightID = num_i(req(o, "lightID", "cyclide"), "cyclide.lightID");
        S.cyclides.push_back(d);
    }
    for (const Value& o : list(root, "sdf")) {
        SdfD d{};
        vec_f(req(o, "position", "sdf"), d.pos, 3, "sdf.position");
        vec_f(req(o, "boundingSize", "sdf"), d.size, 3, "sdf.boundingSize");
        const Value* g = o.find("glsl");
        const Value* b = o.find("builtin");
        if (g && g->type == Value::String) {
            d.source = g->s;
            d.is_builtin_key = false;
        } else if (b && b->type == Value::String) {
            d.source = (b->s.rfind("builtin:", 0) == 0) ? b->s : "builtin:" + b->s;
            d.is_builtin_key = true;
        } else {
            throw LoadError{"sdf: needs a \"glsl\" or \"builtin\" string"};
        }
        S.sdfs.push_back(d);
    }
    for (const Value& o : list(root, "material")) {
        MaterialD d{};
        const Value& r = req(o, "reflection", "material");
        d.reflection[0] = num_f(req(r, "peakWavelength", "material.reflection"), "material.peakWavelength");
        d.reflection[1] = num_f(req(r, "sigma", "material.reflection"), "material.sigma");
        d.reflection[2] = num_b(req(r, "isInvert", "material.reflection"), "material.isInvert") ? 1.0f : 0.0f;
        if (const Value* b = o.find("bsdf")) load_bsdf(*b, d);
        S.materials.push_back(d);
    }
    for (const Value& o : list(root, "light")) {
        LightD d{};
        const Value& e = req(o, "emission", "light");
        d.emission[0] = num_f(req(e, "temperature", "light.emission"), "light.temperature");
        d.emission[1] = num_f(req(e, "luminosity", "light.emission"), "light.luminosity");
        S.lights.push_back(d);
    }
    // Full-form extensions (keys the reference's loader does not read).
    if (const Value* env = root.find("environment"); env && env->type != Value::Null) {
        S.ext.sky = true;
        S.ext.sky_temperature = num_f(req(*env, "temperature", "environment"), "environment.temperature");
        S.ext.sky_luminosity = num_f(req(*env, "luminosity", "environment"), "environment.luminosity");
    }
    if (const Value* sp = root.find("spectral"); sp && sp->type != Value::Null) {
        if (const Value* r = sp->find("range"); r && r->type != Value::Null) {
            float lr[2];
            vec_f(*r, lr, 2, "spectral.range");
            S.ext.range = true;
            S.ext.lambda_min = lr[0];
            S.ext.lambda_max = lr[1];
        }
        if (const Value* c = sp->find("cmf"); c && c->type != Value::Null) {
            if (c->type != Value::String || (c->s != "analytic" && c->s != "table"))
                throw LoadError{"spectral.cmf: \"analytic\" or \"table\""};
            S.ext.analytic_cmf = c->s == "analytic";
        }
    }
    if (const Value* m = root.find("march"); m && m->type != Value::Null) {
        S.ext.march = true;
        S.ext.march_max_steps = num_i(req(*m, "maxSteps", "march"), "march.maxSteps");
        S.ext.march_epsilon = num_f(req(*m, "epsilon", "march"), "march.epsilon");
        S.ext.march_max_distance = num_f(req(*m, "maxDistance", "march"), "march.maxDistance");
    }
}

void set_err(char* err, size_t cap, const std::string& msg) {
    if (err && cap > 0) {
        std::snprintf(err, cap, "%s", msg.c_str());
    }
}

// RoundDecimal, PT:935-943, without the int overflow for |x| >= 21474.
double round_decimal(double number, double precision) {
    if (number >= 0.0) {
        number = (double)(long long)(number * precision + 0.5);
    } else {
        number = (double)(long long)(number * precision - 0.5);
    }
    return number / precision;
}

Value rnum(float f) { return Value::make_float(round_decimal((double)f, 1e5)); }
Value rvec(const float* v, int n) {
    Value a = Value::make_array();
    for (int i = 0; i < n; i++) a.arr.push_back(rnum(v[i]));
    return a;
}

}  // namespace

extern "C" {

int pt_scene_parse(const char* json, size_t len, pt_scene** out, char* err, size_t err_cap) {
    if (!json || !out) return PT_ERR_INVALID;
    *out = nullptr;
    Value root;
    std::string perr;
    if (!ptjson::parse(std::string(json, len), root, perr)) {
        set_err(err, err_cap, "JSON: " + perr);
        return PT_ERR_INVALID;
    }
    pt_scene* s = new pt_scene();
    try {
        load(root, *s);
    } catch (const LoadError& e) {
        set_err(err, err_cap, e.msg);
        delete s;
        return PT_ERR_INVALID;
    } catch (...) {
        set_err(err, err_cap, "scene: out of memory");
        delete s;
        return PT_ERR_OOM;
    }
    *out = s;
    return PT_OK;
}

int pt_scene_load_file(const char* path, pt_scene** out, char* err, size_t err_cap) {
    if (!path || !out) return PT_ERR_INVALID;
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        set_err(err, err_cap, std::string("Failed To Open The JSON File With Directory ") + path);
        return PT_ERR_INVALID;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    return pt_scene_parse(text.data(), text.size(), out, err, err_cap);
}

void pt_scene_free(pt_scene* scene) { delete scene; }

int pt_scene_counts(const pt_scene* s, int counts[9]) {
    if (!s || !counts) return PT_ERR_INVALID;
    counts[0] = (int)s->spheres.size();
    counts[1] = (int)s->planes.size();
    counts[2] = (int)s->boxes.size();
    counts[3] = (int)s->lenses.size();
    counts[4] = (int)s->cyclides.size();
    counts[5] = (int)s->sdfs.size();
    counts[6] = (int)s->materials.size();
    counts[7] = (int)s->lights.size();
    counts[8] = (int)s->shots.size();
    return PT_OK;
}

// UpdateUniformBuffer, PT:3642-3811.
int pt_scene_pack_ubo(const pt_scene* s, const float* cie, pt_ubo* out) {
    if (!s || !out) return PT_ERR_INVALID;
    std::vector<float> objects, sdfs, materials, lights, lightIDs;
    for (size_t i = 0; i < s->spheres.size(); i++) {
        const SphereD& o = s->spheres[i];
        objects.insert(objects.end(), {o.pos[0], o.pos[1], o.pos[2], o.radius, (float)o.materialID, (float)o.lightID});
        if (o.lightID > 0) lightIDs.push_back((float)i);
    }
    for (size_t i = 0; i < s->planes.size(); i++) {
        const PlaneD& o = s->planes[i];
        objects.insert(objects.end(), {o.pos[0], o.pos[1], o.pos[2], (float)o.materialID, (float)o.lightID});
        if (o.lightID > 0) lightIDs.push_back((float)(s->spheres.size() + i));
    }
    for (size_t i = 0; i < s->boxes.size(); i++) {
        const BoxD& o = s->boxes[i];
        objects.insert(objects.end(), {o.pos[0], o.pos[1], o.pos[2], o.rotation[0], o.rotation[1], o.rotation[2],
                                       o.size[0], o.size[1], o.size[2], (float)o.materialID, (float)o.lightID});
        if (o.lightID > 0) lightIDs.push_back((float)(s->spheres.size() + s->planes.size() + i));
    }
    for (size_t i = 0; i < s->lenses.size(); i++) {
        const LensD& o = s->lenses[i];
        objects.insert(objects.end(), {o.pos[0], o.pos[1], o.pos[2], o.rotation[0], o.rotation[1], o.rotation[2],
                                       o.radius, o.focalLength, o.thickness, (float)o.isConverging,
                                       (float)o.materialID, (float)o.lightID});
        // PT:3704 tests planes[i].lightID here; past the end of the plane list
        // (undefined in the reference) no light is added.
        if (i < s->planes.size() && s->planes[i].lightID > 0)
            lightIDs.push_back((float)(s->spheres.size() + s->planes.size() + s->boxes.size() + i));
    }
    for (size_t i = 0; i < s->cyclides.size(); i++) {
        const CyclideD& o = s->cyclides[i];
        const float m = std::max(std::max(o.scale[0], o.scale[1]), o.scale[2]);
        objects.insert(objects.end(), {o.pos[0], o.pos[1], o.pos[2], o.rotation[0], o.rotation[1], o.rotation[2],
                                       o.scale[0], o.scale[1], o.scale[2], o.a, o.b, o.c, o.d,
                                       o.brad * o.brad * (m * m), (float)o.materialID, (float)o.lightID});
        // PT:3728 tests planes[i].lightID here as well.
        if (i < s->planes.size() && s->planes[i].lightID > 0)
            lightIDs.push_back(
                (float)(s->spheres.size() + s->planes.size() + s->boxes.size() + s->lenses.size() + i));
    }
    for (const SdfD& d : s->sdfs) sdfs.insert(sdfs.end(), {d.pos[0], d.pos[1], d.pos[2], d.size[0], d.size[1], d.size[2]});
    for (const MaterialD& d : s->materials) materials.insert(materials.end(), {d.reflection[0], d.reflection[1], d.reflection[2]});
    for (const LightD& d : s->lights) lights.insert(lights.end(), {d.emission[0], d.emission[1]});

    if (objects.size() > PT_MAX_OBJECTS_SIZE || sdfs.size() > PT_MAX_SDFS_SIZE ||
        materials.size() > PT_MAX_MATERIALS_SIZE || lights.size() > PT_MAX_LIGHTS_SIZE ||
        lightIDs.size() > PT_MAX_LIGHTIDS_SIZE)
        return PT_ERR_INVALID;

    std::memset(out, 0, sizeof(pt_ubo));
    out->numObjects[0] = (float)s->spheres.size();
    out->numObjects[1] = (float)s->planes.size();
    out->numObjects[2] = (float)s->boxes.size();
    out->numObjects[3] = (float)s->lenses.size();
    out->numObjects[4] = (float)s->cyclides.size();
    out->numObjects[5] = (float)s->sdfs.size();
    out->numObjects[6] = (float)lightIDs.size();
    std::copy(objects.begin(), objects.end(), out->objects);
    std::copy(sdfs.begin(), sdfs.end(), out->sdfs);
    std::copy(materials.begin(), materials.end(), out->materials);
    std::copy(lights.begin(), lights.end(), out->lights);
    std::copy(lightIDs.begin(), lightIDs.end(), out->lightIDs);
    if (cie) std::memcpy(out->CIEXYZ1931, cie, sizeof(out->CIEXYZ1931));
    return PT_OK;
}

// The scene's full-form extensions as the kernels take them; a scene
// without any gives a zeroed block (the reference's method).
int pt_scene_pack_ext(const pt_scene* s, pt_scene_ext* out) {
    if (!s || !out) return PT_ERR_INVALID;
    std::memset(out, 0, sizeof(pt_scene_ext));
    const ExtD& x = s->ext;
    if (x.sky) {
        out->flags |= PT_EXT_SKY;
        out->sky_temperature = x.sky_temperature;
        out->sky_luminosity = x.sky_luminosity;
    }
    if (x.range) {
        out->flags |= PT_EXT_WAVELENGTHS;
        out->lambda_min = x.lambda_min;
        out->lambda_max = x.lambda_max;
    }
    if (x.analytic_cmf) out->flags |= PT_EXT_ANALYTIC_CMF;
    if (x.march) {
        out->flags |= PT_EXT_MARCH;
        out->march_max_steps = x.march_max_steps;
        out->march_epsilon = x.march_epsilon;
        out->march_max_distance = x.march_max_distance;
    }
    int last = 0;  // materials up to the last one with a model of its own
    for (size_t i = 0; i < s->materials.size(); i++)
        if (s->materials[i].bsdf != PT_BSDF_REFERENCE) last = (int)i + 1;
    if (last > PT_MAX_EXT_MATERIALS) return PT_ERR_INVALID;
    if (last > 0) {
        out->flags |= PT_EXT_MATERIALS;
        out->nmat = last;
        for (int i = 0; i < last; i++) {
            out->mat[i].type = s->materials[(size_t)i].bsdf;
            std::memcpy(out->mat[i].p, s->materials[(size_t)i].bsdf_p, sizeof(out->mat[i].p));
        }
    }
    return PT_OK;
}

// UpdatePushConstant, PT:3813-3834.
int pt_scene_push_constants(const pt_scene* s, const pt_frame_state* st, pt_push* out) {
    if (!s || !st || !out) return PT_ERR_INVALID;
    if (st->cameraShotIndex < 1 || st->cameraShotIndex > (int)s->shots.size()) return PT_ERR_INVALID;
    const ShotD& shot = s->shots[(size_t)st->cameraShotIndex - 1];
    std::memset(out, 0, sizeof(pt_push));
    out->resolution[0] = st->width;
    out->resolution[1] = st->height;
    out->frame = st->frame;
    out->currentSamples = st->currentSamples;
    out->samplesPerFrame = st->samplesPerFrame;
    out->FPS = st->FPS;
    out->persistence = st->persistence;
    out->pathLength = st->pathLength;
    out->cameraAngle[0] = -shot.angle[1];
    out->cameraAngle[1] = shot.angle[0];
    out->cameraPosX = shot.pos[0];
    out->cameraPosY = shot.pos[1];
    out->cameraPosZ = shot.pos[2];
    out->ISO = s->camera.ISO;
    out->cameraSize = s->camera.size;
    out->apertureSize = s->camera.apertureSize;
    out->apertureDist = s->camera.apertureDist;
    out->lensRadius = s->camera.lensRadius;
    out->lensFocalLength = s->camera.lensFocalLength;
    out->lensThickness = s->camera.lensThickness;
    out->lensDistance = s->camera.lensDistance;
    out->tonemap = st->tonemap;
    return PT_OK;
}

const char* pt_scene_sdf_source(const pt_scene* s, int i) {
    if (!s || i < 0 || i >= (int)s->sdfs.size()) return nullptr;
    return s->sdfs[(size_t)i].source.c_str();
}

int pt_scene_sdf_plugins(const pt_scene* s, pt_sdf_plugin* out, int cap, int* count) {
    if (!s || !count || cap < 0 || (cap > 0 && !out)) return PT_ERR_INVALID;
    const int n = (int)s->sdfs.size();
    *count = n;
    for (int i = 0; i < n && i < cap; i++) {
        const int rc = pt_parse_sdf_source(s->sdfs[(size_t)i].source.c_str(), &out[i]);
        if (rc != PT_OK) return rc;
    }
    return PT_OK;
}

// UpdateToJSON, PT:2724-2858, then dump(4).
int pt_scene_to_json(const pt_scene* s, char* buf, size_t cap, size_t* needed) {
    if (!s) return PT_ERR_INVALID;
    Value root = Value::make_object();
    Value& cam = root.at_or_insert("camera");
    cam.at_or_insert("numShots") = Value::make_int((int64_t)s->shots.size());
    if (!s->shots.empty()) {
        Value pos = Value::make_array();
        Value ang = Value::make_array();
        for (const ShotD& sh : s->shots) {
            pos.arr.push_back(rvec(sh.pos, 3));
            ang.arr.push_back(rvec(sh.angle, 2));
        }
        cam.at_or_insert("position") = pos;  // (references into the object are not kept across inserts)
        cam.at_or_insert("angle") = ang;
    }
    cam.at_or_insert("ISO") = Value::make_int(s->camera.ISO);
    cam.at_or_insert("size") = rnum(s->camera.size);
    cam.at_or_insert("apertureSize") = rnum(s->camera.apertureSize);
    cam.at_or_insert("apertureDistance") = rnum(s->camera.apertureDist);
    cam.at_or_insert("lensRadius") = rnum(s->camera.lensRadius);
    cam.at_or_insert("lensFocalLength") = rnum(s->camera.lensFocalLength);
    cam.at_or_insert("lensThickness") = rnum(s->camera.lensThickness);
    cam.at_or_insert("lensDistance") = rnum(s->camera.lensDistance);
    auto arr = [&root](const char* key) -> Value& {
        Value& a = root.at_or_insert(key);
        if (a.type != Value::Array) a = Value::make_array();
        return a;
    };
    auto ids = [](Value& o, int m, int l) {
        o.at_or_insert("materialID") = Value::make_int(m);
        o.at_or_insert("lightID") = Value::make_int(l);
    };
    if (!s->spheres.empty()) {
        Value& a = arr("sphere");
        for (const SphereD& d : s->spheres) {
            Value o = Value::make_object();
            o.at_or_insert("position") = rvec(d.pos, 3);
            o.at_or_insert("radius") = rnum(d.radius);
            ids(o, d.materialID, d.lightID);
            a.arr.push_back(o);
        }
    }
    if (!s->planes.empty()) {
        Value& a = arr("plane");
        for (const PlaneD& d : s->planes) {
            Value o = Value::make_object();
            o.at_or_insert("position") = rvec(d.pos, 3);
            ids(o, d.materialID, d.lightID);
            a.arr.push_back(o);
        }
    }
    if (!s->boxes.empty()) {
        Value& a = arr("box");
        for (const BoxD& d : s->boxes) {
            Value o = Value::make_object();
            o.at_or_insert("position") = rvec(d.pos, 3);
            o.at_or_insert("rotation") = rvec(d.rotation, 3);
            o.at_or_insert("size") = rvec(d.size, 3);
            ids(o, d.materialID, d.lightID);
            a.arr.push_back(o);
        }
    }
    if (!s->lenses.empty()) {
        Value& a = arr("lens");
        for (const LensD& d : s->lenses) {
            Value o = Value::make_object();
            o.at_or_insert("position") = rvec(d.pos, 3);
            o.at_or_insert("rotation") = rvec(d.rotation, 3);
            o.at_or_insert("radius") = rnum(d.radius);
            o.at_or_insert("focalLength") = rnum(d.focalLength);
            o.at_or_insert("thickness") = rnum(d.thickness);
            o.at_or_insert("isConverging") = Value::make_bool(d.isConverging);
            ids(o, d.materialID, d.lightID);
            a.arr.push_back(o);
        }
    }
    if (!s->cyclides.empty()) {
        Value& a = arr("cyclide");
        for (const CyclideD& d : s->cyclides) {
            Value o = Value::make_object();
            o.at_or_insert("position") = rvec(d.pos, 3);
            o.at_or_insert("rotation") = rvec(d.rotation, 3);
            o.at_or_insert("scale") = rvec(d.scale, 3);
            o.at_or_insert("a") = rnum(d.a);
            o.at_or_insert("b") = rnum(d.b);
            o.at_or_insert("c") = rnum(d.c);
            o.at_or_insert("d") = rnum(d.d);
            o.at_or_insert("boundingRadius") = rnum(d.brad);
            ids(o, d.materialID, d.lightID);
            a.arr.push_back(o);
        }
    }
    if (!s->sdfs.empty()) {
        Value& a = arr("sdf");
        for (const SdfD& d : s->sdfs) {
            Value o = Value::make_object();
            o.at_or_insert("position") = rvec(d.pos, 3);
            o.at_or_insert("boundingSize") = rvec(d.size, 3);
            if (d.is_builtin_key) {
                o.at_or_insert("builtin") = Value::make_string(d.source);
            } else {
                o.at_or_insert("glsl") = Value::make_string(d.source);
            }
            a.arr.push_back(o);
        }
    }
    if (!s->materials.empty()) {
        Value& a = arr("material");
        for (const MaterialD& d : s->materials) {
            Value o = Value::make_object();
            Value& r = o.at_or_insert("reflection");
            r.at_or_insert("peakWavelength") = rnum(d.reflection[0]);
            r.at_or_insert("sigma") = rnum(d.reflection[1]);
            r.at_or_insert("isInvert") = Value::make_bool(d.reflection[2] != 0.0f);
            if (d.bsdf != PT_BSDF_REFERENCE) {
                Value& b = o.at_or_insert("bsdf");
                const float* p = d.bsdf_p;
                switch (d.bsdf) {
                    case PT_BSDF_FLAT:
                        b.at_or_insert("type") = Value::make_string("flat");
                        b.at_or_insert("albedo") = rnum(p[0]);
                        break;
                    case PT_BSDF_SMOOTH:
                        b.at_or_insert("type") = Value::make_string("smooth");
                        b.at_or_insert("base") = rnum(p[0]);
                        b.at_or_insert("amplitude") = rnum(p[1]);
                        b.at_or_insert("center") = rnum(p[2]);
                        b.at_or_insert("width") = rnum(p[3]);
                        break;
                    case PT_BSDF_MIRROR:
                        b.at_or_insert("type") = Value::make_string("mirror");
                        b.at_or_insert("reflectance") = rnum(p[0]);
                        break;
                    case PT_BSDF_CAUCHY:
                        b.at_or_insert("type") = Value::make_string("cauchy");
                        b.at_or_insert("A") = rnum(p[0]);
                        b.at_or_insert("B") = rnum(p[1]);
                        break;
                    default:
                        b.at_or_insert("type") = Value::make_string("sellmeier");
                        b.at_or_insert("B") = rvec(p, 3);
                        b.at_or_insert("C") = rvec(p + 3, 3);
                        break;
                }
            }
            a.arr.push_back(o);
        }
    }
    if (!s->lights.empty()) {
        Value& a = arr("light");
        for (const LightD& d : s->lights) {
            Value o = Value::make_object();
            Value& e = o.at_or_insert("emission");
            e.at_or_insert("temperature") = rnum(d.emission[0]);
            e.at_or_insert("luminosity") = rnum(d.emission[1]);
            a.arr.push_back(o);
        }
    }
    const ExtD& x = s->ext;
    if (x.sky) {
        Value& e = root.at_or_insert("environment");
        e = Value::make_object();
        e.at_or_insert("temperature") = rnum(x.sky_temperature);
        e.at_or_insert("luminosity") = rnum(x.sky_luminosity);
    }
    if (x.range || x.analytic_cmf) {
        Value& sp = root.at_or_insert("spectral");
        sp = Value::make_object();
        if (x.range) {
            const float lr[2] = {x.lambda_min, x.lambda_max};
            sp.at_or_insert("range") = rvec(lr, 2);
        }
        if (x.analytic_cmf) sp.at_or_insert("cmf") = Value::make_string("analytic");
    }
    if (x.march) {
        Value& m = root.at_or_insert("march");
        m = Value::make_object();
        m.at_or_insert("maxSteps") = Value::make_int(x.march_max_steps);
        m.at_or_insert("epsilon") = Value::make_float((double)x.march_epsilon);
        m.at_or_insert("maxDistance") = rnum(x.march_max_distance);
    }
    const std::string text = ptjson::dump(root, 4);
    if (needed) *needed = text.size() + 1;
    if (!buf || cap < text.size() + 1) return buf ? PT_ERR_INVALID : PT_OK;
    std::memcpy(buf, text.c_str(), text.size() + 1);
    return PT_OK;
}

int pt_scene_bind(pt_ctx* ctx, const pt_scene* s, const float* cie) {
    if (!ctx || !s || !cie) return PT_ERR_INVALID;
    pt_ubo* ubo = new (std::nothrow) pt_ubo;
    if (!ubo) return PT_ERR_OOM;
    int rc = pt_scene_pack_ubo(s, cie, ubo);
    if (rc == PT_OK) {
        std::vector<const char*> src;
        for (const SdfD& d : s->sdfs) src.push_back(d.source.c_str());
        rc = pt_set_sdfs(ctx, src.data(), (int)src.size());
    }
    pt_scene_ext* ext = nullptr;
    if (rc == PT_OK) {
        ext = new (std::nothrow) pt_scene_ext;
        if (!ext) rc = PT_ERR_OOM;
    }
    if (rc == PT_OK) rc = pt_scene_pack_ext(s, ext);
    if (rc == PT_OK) rc = pt_upload_scene_ext(ctx, ubo, ext->flags ? ext : nullptr);
    delete ext;
    delete ubo;
    return rc;
}

}  // extern "C"
