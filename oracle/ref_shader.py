"""Builds the reference's own compute shader (src/shader.comp of the reference
tree) for the CPU, in two forms, into oracle/_ref/ (git-ignored).

TEST INFRASTRUCTURE ONLY.  The reference cannot run here as a program (it is
Vulkan), but its shader is plain GLSL that the repository's translator
(pt_glsl_translate) and shim (pt_glsl_shim.h) take:
- libref_shader.so: single functions cut out of the source (RNG, sampling,
  spectra, refraction, MIS, the polynomial solvers, the rotation matrix,
  smin, and the analytic intersections with the structs they take), the
  source's numeric #defines as constants and its push constants as
  variables;
- libref_scene_<key>.so: the whole shader without its interface and `main`,
  with a scene's SDF snippets spliced in as the reference's host does
  (splice_sdfs), the uniform buffer and push constants as variables bound
  from a packed scene, and Scene(), Rendering() and Intersection() exposed.
Both compile with g++ -ffp-contract=off.  tests/test_oracle_reference.py
checks the oracle (oracle/pt_oracle.c) against them bit for bit, and
bench.py times the whole shader as the CPU baseline.  Nothing of the
reference is committed: the source is read from the reference tree at build
time; where the tree is absent (the GPU machine) a whole-shader C++ text
generated before is compiled instead.

    python oracle/ref_shader.py [reference-root]
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libref_shader.so")
DEFAULT_REFERENCE = "/root/reference"

# The shader functions built, every overload of each name.
FUNCTIONS = [
    "PCG32", "RandomFloatPCG32", "GenerateSeed", "SampleHeroWavelength", "InverseSampleWavelengthPDF",
    "SampleWavelengths", "SampleUniformUnitDisk", "SampleUniformUnitSphere", "SampleCosineDirectionHemisphere",
    "CosineDirectionPDF", "SampleCosineUnitCone", "CosineUnitConePDF", "SpectralPowerDistribution",
    "BlackBodyRadiation", "BlackBodyRadiationPeak", "RefractiveIndexWavelength", "RefractiveIndexBK7Glass",
    "OrthonormalBasis", "ToWorld", "MISPowerHeuristicsBeta2", "EvalQuadratic", "EvalCubic",
    "EvalQuartic", "SolveCubic", "SolveQuartic", "minMaterial", "smin", "RotationMatrix", "SortMinMax",
    "BoundingSphere", "RayIntersectAABB", "SphereIntersection", "PlaneIntersection", "BoxIntersection",
    "SphereSliceIntersection", "LensIntersection", "DupinCyclide", "Thritorius", "SmoothCuboid",
]
# The shader's structs those functions take.
STRUCTS = ["Ray", "sphere", "plane", "box", "sphereSlice", "lens", "cyclide"]

# C entry points (refsh_*) over the translated functions (namespace ptg::ref_).
WRAPPERS = r"""
using namespace ptg;
using namespace ptg::ref_;
extern "C" {
uint32_t refsh_pcg32(uint32_t s) { uint x = s; ref_PCG32(x); return x; }
float refsh_random_float(uint32_t* s) { uint x = *s; const float r = ref_RandomFloatPCG32(x); *s = x; return r; }
uint32_t refsh_generate_seed(uint32_t x, uint32_t y, int fr, int spf, int k, int width) {
    frame = fr;
    samplesPerFrame = spf;
    resolution = ivec2(width, 0);
    return ref_GenerateSeed(uvec2(x, y), k);
}
float refsh_hero_wavelength(float lmin, float lmax, uint32_t* s) {
    uint x = *s;
    const float r = ref_SampleHeroWavelength(lmin, lmax, x);
    *s = x;
    return r;
}
float refsh_inverse_wavelength_pdf(float lmin, float lmax) { return ref_InverseSampleWavelengthPDF(lmin, lmax); }
void refsh_sample_wavelengths(float lh, float* o) {
    const vec4 v = ref_SampleWavelengths(lh);
    o[0] = v.x, o[1] = v.y, o[2] = v.z, o[3] = v.w;
}
void refsh_sample_disk(uint32_t* s, float* o) {
    uint x = *s;
    const vec2 v = ref_SampleUniformUnitDisk(x);
    *s = x;
    o[0] = v.x, o[1] = v.y;
}
void refsh_sample_sphere(uint32_t* s, float* o) {
    uint x = *s;
    const vec3 v = ref_SampleUniformUnitSphere(x);
    *s = x;
    o[0] = v.x, o[1] = v.y, o[2] = v.z;
}
void refsh_sample_hemisphere(const float* n, uint32_t* s, float* o) {
    uint x = *s;
    const vec3 v = ref_SampleCosineDirectionHemisphere(vec3(n[0], n[1], n[2]), x);
    *s = x;
    o[0] = v.x, o[1] = v.y, o[2] = v.z;
}
float refsh_cosine_pdf(float c) { return ref_CosineDirectionPDF(c); }
void refsh_sample_cone(uint32_t* s, float cmax, float* o) {
    uint x = *s;
    const vec3 v = ref_SampleCosineUnitCone(x, cmax);
    *s = x;
    o[0] = v.x, o[1] = v.y, o[2] = v.z;
}
float refsh_cone_pdf(float c, float cmax) { return ref_CosineUnitConePDF(c, cmax); }
void refsh_spd(const float* l, float peak, float d, int invert, float* o) {
    const vec4 v = ref_SpectralPowerDistribution(vec4(l[0], l[1], l[2], l[3]), peak, d, invert);
    o[0] = v.x, o[1] = v.y, o[2] = v.z, o[3] = v.w;
}
void refsh_blackbody(const float* l, float T, float* o) {
    const vec4 v = ref_BlackBodyRadiation(vec4(l[0], l[1], l[2], l[3]), T);
    o[0] = v.x, o[1] = v.y, o[2] = v.z, o[3] = v.w;
}
float refsh_blackbody_peak(float T) { return ref_BlackBodyRadiationPeak(T); }
float refsh_bk7_index(float l) { return ref_RefractiveIndexBK7Glass(l); }
void refsh_to_world(const float* v, const float* n, float* o) {
    const vec3 r = ref_ToWorld(vec3(v[0], v[1], v[2]), vec3(n[0], n[1], n[2]));
    o[0] = r.x, o[1] = r.y, o[2] = r.z;
}
float refsh_mis(float a, float b) { return ref_MISPowerHeuristicsBeta2(a, b); }
float refsh_smin(float x, float y) { return ref_smin(x, y); }
void refsh_smin2(const float* x, const float* y, float* o) {
    const vec2 v = ref_smin(vec2(x[0], x[1]), vec2(y[0], y[1]));
    o[0] = v.x, o[1] = v.y;
}
float refsh_min_material(float x, float y, float m1, float m2) { return ref_minMaterial(x, y, m1, m2); }
int refsh_solve_cubic(float b, float c, float d, float* r) {
    vec3 v(r[0], r[1], r[2]);
    const bvec3 real = ref_SolveCubic(b, c, d, v);
    r[0] = v.x, r[1] = v.y, r[2] = v.z;
    return (int)real.x + (int)real.y + (int)real.z;
}
void refsh_solve_quartic(float a, float b, float c, float d, float e, float* r, int* real) {
    vec4 v(r[0], r[1], r[2], r[3]);
    const bvec4 q = ref_SolveQuartic(a, b, c, d, e, v);
    r[0] = v.x, r[1] = v.y, r[2] = v.z, r[3] = v.w;
    real[0] = q.x, real[1] = q.y, real[2] = q.z, real[3] = q.w;
}
void refsh_rotation(const float* angle, float* o) {
    const mat3 m = ref_RotationMatrix(vec3(angle[0], angle[1], angle[2]));
    const vec3 c[3] = {m.c0, m.c1, m.c2};
    for (int j = 0; j < 3; j++) o[3 * j] = c[j].x, o[3 * j + 1] = c[j].y, o[3 * j + 2] = c[j].z;
}
static Ray ray_of(const float* r) {
    Ray ray;
    ray.origin = vec3(r[0], r[1], r[2]);
    ray.dir = vec3(r[3], r[4], r[5]);
    return ray;
}
// hit = hitdist, normal, materialID, lightID: the inout arguments of an intersection
struct Hit {
    float d;
    vec3 n;
    float m, l;
    explicit Hit(const float* h) : d(h[0]), n(h[1], h[2], h[3]), m(h[4]), l(h[5]) {}
    void put(float* h) const { h[0] = d, h[1] = n.x, h[2] = n.y, h[3] = n.z, h[4] = m, h[5] = l; }
};
int refsh_bounding_sphere(const float* r, const float* pos, float radius2) {
    return ref_BoundingSphere(ray_of(r), vec3(pos[0], pos[1], pos[2]), radius2);
}
void refsh_aabb(const float* origin, const float* invdir, const float* pos, const float* size, float* o) {
    box b;
    b.pos = vec3(pos[0], pos[1], pos[2]);
    b.size = vec3(size[0], size[1], size[2]);
    const vec2 v = ref_RayIntersectAABB(vec3(origin[0], origin[1], origin[2]), vec3(invdir[0], invdir[1], invdir[2]), b);
    o[0] = v.x, o[1] = v.y;
}
int refsh_sphere(const float* r, const float* o, float* h) {
    sphere s;
    s.pos = vec3(o[0], o[1], o[2]);
    s.radius = o[3];
    s.materialID = (int)o[4];
    s.lightID = (int)o[5];
    Hit t(h);
    const bool hit = ref_SphereIntersection(ray_of(r), s, t.d, t.n, t.m, t.l);
    t.put(h);
    return hit;
}
int refsh_plane(const float* r, const float* o, float* h) {
    plane p;
    p.pos = vec3(o[0], o[1], o[2]);
    p.materialID = (int)o[3];
    p.lightID = (int)o[4];
    Hit t(h);
    const bool hit = ref_PlaneIntersection(ray_of(r), p, t.d, t.n, t.m, t.l);
    t.put(h);
    return hit;
}
int refsh_box(const float* r, const float* o, float* h) {
    box b;
    b.pos = vec3(o[0], o[1], o[2]);
    b.rotation = vec3(o[3], o[4], o[5]);
    b.size = vec3(o[6], o[7], o[8]);
    b.materialID = (int)o[9];
    b.lightID = (int)o[10];
    Hit t(h);
    const bool hit = ref_BoxIntersection(ray_of(r), b, t.d, t.n, t.m, t.l);
    t.put(h);
    return hit;
}
int refsh_lens(const float* r, const float* o, float* h, int* isOutside) {
    lens l;
    l.pos = vec3(o[0], o[1], o[2]);
    l.rotation = vec3(o[3], o[4], o[5]);
    l.radius = o[6];
    l.focalLength = o[7];
    l.thickness = o[8];
    l.isConverging = o[9] != 0.0f;
    l.materialID = (int)o[10];
    l.lightID = (int)o[11];
    Hit t(h);
    int out = *isOutside;
    const bool hit = ref_LensIntersection(ray_of(r), l, t.d, t.n, out, t.m, t.l);
    t.put(h);
    *isOutside = out;
    return hit;
}
int refsh_cyclide(const float* r, const float* o, float* h) {
    cyclide c;
    c.pos = vec3(o[0], o[1], o[2]);
    c.rotation = vec3(o[3], o[4], o[5]);
    c.scale = vec3(o[6], o[7], o[8]);
    c.a = o[9], c.b = o[10], c.c = o[11], c.d = o[12], c.brad = o[13];
    c.materialID = (int)o[14];
    c.lightID = (int)o[15];
    Hit t(h);
    const bool hit = ref_DupinCyclide(ray_of(r), c, t.d, t.n, t.m, t.l);
    t.put(h);
    return hit;
}
int refsh_thritorius(const float* r, const float*, float* h) {
    Hit t(h);
    const bool hit = ref_Thritorius(ray_of(r), t.d, t.n, t.m, t.l);
    t.put(h);
    return hit;
}
int refsh_smooth_cuboid(const float* r, const float*, float* h) {
    Hit t(h);
    const bool hit = ref_SmoothCuboid(ray_of(r), t.d, t.n, t.m, t.l);
    t.put(h);
    return hit;
}
}
"""


def reference_root(arg: str | None = None) -> str:
    return arg or os.environ.get("PT_REFERENCE_ROOT", DEFAULT_REFERENCE)


def shader_path(reference: str | None = None) -> str:
    """The reference's compute shader source (present only where the
    reference tree is mounted)."""
    return os.path.join(reference_root(reference), "src", "shader.comp")


def extract(src: str) -> str:
    """The GLSL text handed to the translator: the source's numeric #defines as
    constants, the push constants the functions read as variables, then every
    definition of each FUNCTIONS name in source order."""
    out = []
    for m in re.finditer(r"^#define\s+(\w+)\s+([-+0-9.eE]+)\s*$", src, re.M):
        name, value = m.group(1), m.group(2)
        kind = "float" if re.search(r"[.eE]", value) else "int"
        out.append(f"const {kind} {name} = {value};")
    out.append("int frame = 0;\nint samplesPerFrame = 1;\nivec2 resolution = ivec2(0);")
    for name in STRUCTS:
        m = re.search(r"^struct\s+" + name + r"\s*\{.*?\};", src, re.M | re.S)
        if not m:
            raise ValueError(f"struct {name} not found in the shader source")
        out.append(m.group(0))
    starts = []
    for name in FUNCTIONS:
        found = [m.start() for m in re.finditer(r"^\w+\s+" + name + r"\s*\(", src, re.M)]
        if not found:
            raise ValueError(f"{name} not found in the shader source")
        starts.extend(found)
    for s in sorted(starts):
        depth, i = 0, src.index("{", s)
        while True:
            if src[i] == "{":
                depth += 1
            elif src[i] == "}":
                depth -= 1
                if depth == 0:
                    break
            i += 1
        out.append(src[s:i + 1])
    # the translator wants the two SDF entry points of a scene snippet
    out.append("float sdf(vec3 p) { return 0.0; }\nfloat sdfmaterial(vec3 p) { return 0.0; }")
    return "\n\n".join(out) + "\n"


def build(reference: str | None = None) -> str:
    """Builds (when the shader source is newer) and returns the library path."""
    shader = shader_path(reference)
    if not os.path.exists(shader):
        raise FileNotFoundError(shader)
    deps = [shader, __file__, os.path.join(ROOT, "pathtracer_gb300", "csrc", "kernel", "pt_glsl_shim.h"),
            os.path.join(ROOT, "pathtracer_gb300", "csrc", "pt_glsl.cpp"), os.path.join(ROOT, "include", "pt_mathf.h")]
    if os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    sys.path.insert(0, ROOT)
    from pathtracer_gb300 import glsl_translate

    with open(shader) as f:
        glsl = extract(f.read())
    code = glsl_translate(glsl, "ref_")
    os.makedirs(OUT, exist_ok=True)
    cpp = os.path.join(OUT, "ref_shader.cpp")
    with open(cpp, "w") as f:
        f.write("#include <stdint.h>\n#include \"pt_glsl_shim.h\"\n" + code + WRAPPERS)
    subprocess.run([os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-fno-fast-math", "-I", os.path.join(ROOT, "pathtracer_gb300", "csrc", "kernel"), "-o", LIB, cpp],
                   check=True)
    return LIB


def load(reference: str | None = None) -> ctypes.CDLL:
    return ctypes.CDLL(build(reference))


# ---- the whole path tracer: Scene() of the shader for one sample ---------

# The uniform buffer and the push constants (src/shader.comp:19-52) as
# variables of the translated unit.  Buffer reads outside an array give 0,
# as robust buffer access does on the device (the oracle reads them the same
# way).
SCENE_PRELUDE = r"""
#include <omp.h>
#include <stdint.h>
#include <string.h>
#include "pt_cuda.h"
#include "pt_glsl_shim.h"
namespace ptg {
namespace rs_ {
template <int N> struct Robust {
    float v[N];
    float operator[](int i) const { return (i >= 0 && i < N) ? v[i] : 0.0f; }
};
Robust<7> numObjects;
Robust<PT_MAX_OBJECTS_SIZE> objects;
Robust<PT_MAX_SDFS_SIZE> sdfs;
Robust<PT_MAX_MATERIALS_SIZE> materials;
Robust<PT_MAX_LIGHTS_SIZE> lights;
Robust<PT_MAX_LIGHTIDS_SIZE> lightIDs;
Robust<PT_CIE_TABLE_SIZE> CIEXYZ1931;
ivec2 resolution;
int frame, currentSamples, samplesPerFrame;
float FPS, persistence;
int pathLength;
vec2 cameraAngle;
float cameraPosX, cameraPosY, cameraPosZ;
int ISO;
float cameraSize, apertureSize, apertureDist, lensRadius, lensFocalLength, lensThickness, lensDistance;
int tonemap;
uvec3 gl_GlobalInvocationID;  // the invocation Rendering() runs for
}  // namespace rs_
}  // namespace ptg
"""

SCENE_WRAPPERS = r"""
using namespace ptg;
using namespace ptg::rs_;
extern "C" {
// Binds a packed scene (pt_ubo) and the push constants (pt_push), as the
// descriptor set and vkCmdPushConstants do.
void refsc_bind(const pt_ubo* u, const pt_push* pc) {
    memcpy(numObjects.v, u->numObjects, sizeof numObjects.v);
    memcpy(objects.v, u->objects, sizeof objects.v);
    memcpy(sdfs.v, u->sdfs, sizeof sdfs.v);
    memcpy(materials.v, u->materials, sizeof materials.v);
    memcpy(lights.v, u->lights, sizeof lights.v);
    memcpy(lightIDs.v, u->lightIDs, sizeof lightIDs.v);
    memcpy(CIEXYZ1931.v, u->CIEXYZ1931, sizeof CIEXYZ1931.v);
    resolution = ivec2(pc->resolution[0], pc->resolution[1]);
    frame = pc->frame, currentSamples = pc->currentSamples, samplesPerFrame = pc->samplesPerFrame;
    FPS = pc->FPS, persistence = pc->persistence, pathLength = pc->pathLength;
    cameraAngle = vec2(pc->cameraAngle[0], pc->cameraAngle[1]);
    cameraPosX = pc->cameraPosX, cameraPosY = pc->cameraPosY, cameraPosZ = pc->cameraPosZ;
    ISO = pc->ISO;
    cameraSize = pc->cameraSize, apertureSize = pc->apertureSize, apertureDist = pc->apertureDist;
    lensRadius = pc->lensRadius, lensFocalLength = pc->lensFocalLength, lensThickness = pc->lensThickness;
    lensDistance = pc->lensDistance, tonemap = pc->tonemap;
    cameraPos = vec3(cameraPosX, cameraPosY, cameraPosZ);  // the shader's per-invocation global
}
// Scene() for invocation (x, y) and sample k, with the pixel mapping of
// Rendering (src/shader.comp:1509-1511).
void refsc_scene(uint32_t x, uint32_t y, int k, float* out3) {
    const uvec2 xy = uvec2(x, (uint)resolution.y - y);
    const vec2 uv = (2.0f * vec2((float)xy.x, (float)xy.y) - vec2((float)resolution.x, (float)resolution.y)) /
                    (float)resolution.y;
    const vec3 c = rs_Scene(xy, uv, k);
    out3[0] = c.x, out3[1] = c.y, out3[2] = c.z;
}
// Rendering's sample loop over the rows listed in rows[0..n) of the bound
// frame: Scene() for every pixel and sample k < samplesPerFrame, the colours
// summed per pixel into out (3 floats a pixel, row by row in list order);
// OpenMP over all (row, pixel) pairs.
void refsc_render_rows(const int* rows, int n, float* out, int nthreads) {
    const int W = resolution.x, spf = samplesPerFrame;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 8)
    for (long q = 0; q < (long)n * W; q++) {
        const int r = (int)(q / W), x = (int)(q % W);
        float* o = out + 3 * q;
        for (int k = 0; k < spf; k++) {
            float c[3];
            refsc_scene((uint32_t)x, (uint32_t)rows[r], k, c);
            o[0] += c[0], o[1] += c[1], o[2] += c[2];
        }
    }
}
// Rendering() of invocation (x, y): the pixel's samples of this dispatch,
// exposure and Accumulate() over the pixel's previous value in3 (what main
// loads from and stores to the texel buffer).
void refsc_rendering(uint32_t x, uint32_t y, const float* in3, float* out3) {
    gl_GlobalInvocationID = uvec3(x, y, 0u);
    const vec3 c = rs_Rendering(vec3(in3[0], in3[1], in3[2]));
    out3[0] = c.x, out3[1] = c.y, out3[2] = c.z;
}
// Intersection() of one ray: out6 = hitdist, normal, materialID, lightID.
void refsc_intersection(const float* r, float* out6) {
    Ray ray;
    ray.origin = vec3(r[0], r[1], r[2]);
    ray.dir = vec3(r[3], r[4], r[5]);
    vec3 normal = vec3(0.0f);
    float materialID = 0.0f, lightID = -1.0f;
    const float d = rs_Intersection(ray, normal, materialID, lightID);
    out6[0] = d, out6[1] = normal.x, out6[2] = normal.y, out6[3] = normal.z, out6[4] = materialID, out6[5] = lightID;
}
}
"""


def extract_scene(src: str) -> str:
    """The shader without its interface and entry point: the #version,
    #extension, precision and layout lines, the uniform and push-constant
    blocks (SCENE_PRELUDE declares them) and main (it reads and writes the
    texel buffer) are left out; numeric #defines become constants."""
    text = src
    for pat in (r"^#version[^\n]*\n", r"^#extension[^\n]*\n", r"^precision[^\n]*\n", r"^layout\([^)]*\)\s*in;\s*\n",
                r"^layout\([^)]*\)\s*uniform\s+\w+\s*\{.*?\};", r"^layout\([^)]*\)\s*uniform\s+imageBuffer[^;]*;"):
        text = re.sub(pat, "", text, flags=re.M | re.S)
    consts = []

    def define(m):
        value = m.group(2)
        kind = "float" if re.search(r"[.eE]", value) else "int"
        consts.append(f"const {kind} {m.group(1)} = {value};")
        return ""

    text = re.sub(r"^#define\s+(\w+)\s+([-+0-9.eE]+)\s*$", define, text, flags=re.M)
    for name in ("main",):
        m = re.search(r"^\w+\s+" + name + r"\s*\(", text, re.M)
        if not m:
            raise ValueError(f"{name} not found in the shader source")
        depth, i = 0, text.index("{", m.start())
        while True:
            depth += (text[i] == "{") - (text[i] == "}")
            if depth == 0:
                break
            i += 1
        text = text[:m.start()] + text[i + 1:]
    if "#" in text:
        raise ValueError("a preprocessor line is left in the shader text")
    return "\n".join(consts) + "\n" + text + "\nfloat sdf(vec3 p) { return 0.0; }\nfloat sdfmaterial(vec3 p) { return 0.0; }\n"


def splice_sdfs(src: str, texts: list[str]) -> str:
    """The shader with a scene's SDF snippets spliced in, as the reference's
    host does before compiling it (InsertSDF, src/pathtracer.cpp:2004-2054):
    snippet i (1-based n) has its first "sdf" renamed SDFn and then its first
    "sdfmaterial" SDFnMATERIAL, and goes after the "All SDF Are Inserted
    Here" comment; SDF() gains `if ((set1 & 2^i) == 2^i) sdf = min(sdf,
    SDFn(p - pos_i));` and SDFMATERIAL() the material line
    `sdfmaterial = minMaterial(sdf, SDFn(p - pos_i), sdfmaterial,
    SDFnMATERIAL(p - pos_i));` followed by the same distance line, snippet 0
    first.  (The host inserts at character offsets that land after those
    comment lines with CRLF line ends; here the text goes after the comment
    line, the same place.)"""
    code = src

    def after_line(marker):
        j = code.find(marker)
        if j < 0:
            raise ValueError(f"marker {marker!r} not found")
        return j + len(marker)

    for i in reversed(range(len(texts))):
        t = texts[i]
        n = str(i + 1)
        bit = str(1 << (i % 32))
        j = t.find("sdf")
        t = t[:j] + "SDF" + n + t[j + 3:]
        j = t.find("sdfmaterial")
        t = t[:j] + "SDF" + n + "MATERIAL" + t[j + 11:] + "\n"
        pos = f"(p - vec3(sdfs[{6 * i}], sdfs[{6 * i + 1}], sdfs[{6 * i + 2}]))"
        test = f"\n    if ((set{i // 32 + 1} & {bit}) == {bit}) sdf"
        dist = test + f" = min(sdf, SDF{n}{pos});"
        mat = test + f"material = minMaterial(sdf, SDF{n}{pos}, sdfmaterial, SDF{n}MATERIAL{pos});"
        k = after_line("// Put SDF Functions Here")
        code = code[:k] + dist + code[k:]
        k = after_line("// Put SDFMATERIAL Functions Here")
        code = code[:k] + mat + dist + code[k:]
        k = after_line("// All SDF Are Inserted Here")
        code = code[:k] + "\n" + t + code[k:]
    return code


def scene_key(sdf_texts: list[str] | None) -> str:
    import hashlib

    texts = list(sdf_texts or [])
    return hashlib.sha1("\0".join(texts).encode()).hexdigest()[:12] if texts else "nosdf"


def build_scene(reference: str | None = None, sdf_texts: list[str] | None = None) -> str:
    """The shader's path tracer for a scene's SDF snippets (none: the SDF
    hooks stay empty, as in the source), as oracle/_ref/libref_scene_<key>.so.
    Where the reference tree is mounted the C++ text is (re)generated from
    it; elsewhere a text generated before is compiled, and without one this
    raises FileNotFoundError."""
    texts = list(sdf_texts or [])
    key = scene_key(texts)
    cpp = os.path.join(OUT, f"ref_scene_{key}.cpp")
    lib = os.path.join(OUT, f"libref_scene_{key}.so")
    shader = shader_path(reference)
    kernel = os.path.join(ROOT, "pathtracer_gb300", "csrc", "kernel")
    if os.path.exists(shader):
        deps = [shader, __file__, os.path.join(kernel, "pt_glsl_shim.h"),
                os.path.join(ROOT, "pathtracer_gb300", "csrc", "pt_glsl.cpp")]
        if not os.path.exists(cpp) or any(os.path.getmtime(d) > os.path.getmtime(cpp) for d in deps):
            sys.path.insert(0, ROOT)
            from pathtracer_gb300 import glsl_translate

            with open(shader) as f:
                code = glsl_translate(extract_scene(splice_sdfs(f.read(), texts)), "rs_")
            os.makedirs(OUT, exist_ok=True)
            with open(cpp, "w") as f:
                f.write(SCENE_PRELUDE + code + SCENE_WRAPPERS)
    elif not os.path.exists(cpp):
        raise FileNotFoundError(shader)
    cdeps = [cpp, os.path.join(kernel, "pt_glsl_shim.h"), os.path.join(ROOT, "include", "pt_mathf.h"),
             os.path.join(ROOT, "include", "pt_cuda.h")]
    if not os.path.exists(lib) or any(os.path.getmtime(d) > os.path.getmtime(lib) for d in cdeps):
        subprocess.run([os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                        "-fno-fast-math", "-fopenmp", "-I", kernel, "-I", os.path.join(ROOT, "include"), "-o", lib,
                        cpp], check=True)
    return lib


def load_scene(reference: str | None = None, sdf_texts: list[str] | None = None) -> ctypes.CDLL:
    return ctypes.CDLL(build_scene(reference, sdf_texts))


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
    print(build_scene(sys.argv[1] if len(sys.argv) > 1 else None))
