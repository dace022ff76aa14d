"""The GLSL SDF snippet path without a GPU: pt_glsl_translate's rewrite, its
rejections, the translation's CPU build against the oracle (bit-exact), and
pt_jit_check (NVRTC compiles the run-time megakernel for sm_103a)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import REFERENCE, ROOT, reference_available
from user_snippets import LATTICE, SNIPPETS, SPIRAL, TORUS

KERNEL_DIR = os.path.join(ROOT, "pathtracer_gb300", "csrc", "kernel")
BUILD_DIR = os.path.join(ROOT, "oracle", "_build")


@pytest.fixture(scope="module")
def pt(built):
    import pathtracer_gb300 as pt

    return pt


def _cpu_build(pt, name: str, snippets: dict) -> ctypes.CDLL:
    """The translations of `snippets` (name -> GLSL) compiled with g++ over the
    shim, each exported as c_<name>_sdf / c_<name>_mat(float, float, float)."""
    code = '#include "pt_glsl_shim.h"\n'
    for n, glsl in snippets.items():
        code += pt.glsl_translate(glsl, n + "_")
        code += (f'extern "C" float c_{n}_sdf(float x, float y, float z) '
                 f'{{ return ptg::{n}_::{n}_sdf(ptg::vec3(x, y, z)); }}\n')
        code += (f'extern "C" float c_{n}_mat(float x, float y, float z) '
                 f'{{ return ptg::{n}_::{n}_sdfmaterial(ptg::vec3(x, y, z)); }}\n')
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(BUILD_DIR, f"glsl_{name}.cpp")
    lib = os.path.join(BUILD_DIR, f"glsl_{name}.so")
    with open(src, "w") as f:
        f.write(code)
    subprocess.run([os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-I", KERNEL_DIR, "-o", lib, src], check=True)
    return ctypes.CDLL(lib)


def _fn(lib, name):
    f = getattr(lib, name)
    f.restype = ctypes.c_float
    f.argtypes = [ctypes.c_float] * 3
    return f


def _points(n=20000, scale=1.5, seed=1):
    return (np.random.default_rng(seed).standard_normal((n, 3)) * scale).astype(np.float32)


def _bits(x: float) -> int:
    return int(np.float32(x).view(np.uint32))


def test_translation_rewrites_glsl(pt):
    out = pt.glsl_translate(TORUS, "u3_")
    assert out.startswith("namespace ptg {")
    out = " ".join(out.split())  # whitespace is kept as written; compare without it
    assert "constexpr float R = 0.8f;" in out
    assert "PTG_FN float u3_sdTorus( vec3 p, vec2 t, float& ring)" in out
    assert "length(p.xz())" in out
    assert "vec2(R, 0.25f)" in out and "sin(8.0f * p.z)" in out
    assert "u3_sdTorus(p, vec2(R, 0.25f), ring);" in out
    assert "PTG_FN float u3_sdf(vec3 p)" in out and "PTG_FN float u3_sdfmaterial(vec3 p)" in out
    assert "//" not in out.replace("} // namespace u3_ } // namespace ptg", "")
    assert out.startswith("namespace ptg { namespace u3_ {")
    lat = pt.glsl_translate(LATTICE, "u0_")
    assert "max(q.x, max(q.y, q.z))" in lat  # .g .b name fields
    assert "/*" not in lat
    assert "1e-3f" in pt.glsl_translate("float sdf(vec3 p){return 1e-3;} float sdfmaterial(vec3 p){return 2.;}", "a_")
    with pytest.raises(pt.PathTracerError):
        pt.glsl_translate(TORUS, "9bad")


@pytest.mark.parametrize("text,why", [
    ("layout(std430) buffer B { float a; }; float sdf(vec3 p){return 0.0;} float sdfmaterial(vec3 p){return 0.0;}",
     "layout"),
    ("uniform float t; float sdf(vec3 p){return t;} float sdfmaterial(vec3 p){return 0.0;}", "uniform"),
    ("#define K 2.0\nfloat sdf(vec3 p){return K;} float sdfmaterial(vec3 p){return 0.0;}", "preprocessor"),
    ("float sdf(vec3 p){(p).xy = vec2(0.0); return 0.0;} float sdfmaterial(vec3 p){return 0.0;}", "swizzle"),
    ("float sdf(vec3 p){return length(p) - 1.0;}", "must define"),
    ("float sdf(vec3 p){return 0.0;} float sdfmaterial(vec3 p){return 0.0;", "unbalanced"),
    ("float sdf(vec3 p){return 0.0; /* open", "unterminated"),
    ("const vec3 C = vec3(1.0); float sdf(vec3 p){return 0.0;} float sdfmaterial(vec3 p){return 0.0;}", "constants"),
])
def test_translation_rejects_what_the_shim_lacks(pt, text, why):
    from pathtracer_gb300 import native

    with pytest.raises(pt.PathTracerError) as e:
        pt.glsl_translate(text)
    assert e.value.code == native.PT_ERR_UNSUPPORTED
    assert why in str(e.value)


def test_user_snippets_match_their_c_restatement(pt):
    """The translation of each test snippet, built for the CPU, agrees bit for
    bit with the hand restatement the oracle renders with."""
    from oracle import oracle

    lib = _cpu_build(pt, "user", {n: g for n, (g, _, _) in SNIPPETS.items()})
    pts = _points()
    for n, (_, sdf_name, mat_name) in SNIPPETS.items():
        fs, fm = _fn(lib, f"c_{n}_sdf"), _fn(lib, f"c_{n}_mat")
        rs, rm = oracle.user_fn(sdf_name), oracle.user_fn(mat_name)
        bad_s = sum(_bits(fs(*map(float, p))) != _bits(rs(*map(float, p))) for p in pts)
        bad_m = sum(_bits(fm(*map(float, p))) != _bits(rm(*map(float, p))) for p in pts)
        assert bad_s == 0 and bad_m == 0, (n, bad_s, bad_m)


@pytest.mark.skipif(not reference_available(), reason="needs the reference's sdfs/*.glsl")
def test_shipped_snippets_translate_to_the_builtins(pt):
    """The reference's four snippets, run through the translator and built for
    the CPU, give the oracle's built-in plug-ins bit for bit (distance and
    material) — the translator and shim carry the shader's arithmetic."""
    from oracle import oracle
    from pathtracer_gb300 import native

    kinds = {"blob": native.PT_SDF_BLOB, "mandelbulb": native.PT_SDF_MANDELBULB,
             "menger": native.PT_SDF_MENGER, "terrain": native.PT_SDF_TERRAIN}
    texts = {n: open(os.path.join(REFERENCE, "sdfs", n + ".glsl")).read() for n in kinds}
    lib = _cpu_build(pt, "shipped", texts)
    olib = oracle.lib()
    pts = _points()
    for n, kind in kinds.items():
        fs, fm = _fn(lib, f"c_{n}_sdf"), _fn(lib, f"c_{n}_mat")
        pl = native.PtSdfPlugin()
        assert native.cuda().pt_parse_sdf_source(texts[n].encode(), ctypes.byref(pl)) == native.PT_OK
        bad_s = bad_m = 0
        for p in pts:
            a = fs(*map(float, p))
            b = olib.pto_sdf_eval(ctypes.byref(pl), p.ctypes.data)
            bad_s += _bits(a) != _bits(b)
            if kind in (native.PT_SDF_BLOB, native.PT_SDF_MANDELBULB):
                bad_m += _bits(fm(*map(float, p))) != _bits(olib.pto_sdf_material(ctypes.byref(pl), p.ctypes.data))
        assert bad_s == 0 and bad_m == 0, (n, bad_s, bad_m)


def test_jit_check_compiles_the_megakernel(pt):
    """NVRTC builds the run-time megakernel (both trace variants) and march
    kernel for sm_103a with user snippets in slots 0-3, one of them twice
    (each slot's text has its own namespace)."""
    log = pt.jit_check([TORUS, LATTICE, SPIRAL, TORUS], sm=103)
    assert "error" not in log.lower()


def test_jit_check_reports_compiler_errors(pt):
    from pathtracer_gb300 import native

    bad = "float sdf(vec3 p){ return wobble(p); } float sdfmaterial(vec3 p){ return 0.0; }"
    with pytest.raises(pt.PathTracerError) as e:
        pt.jit_check([bad], sm=103)
    assert e.value.code == native.PT_ERR_UNSUPPORTED
    assert "wobble" in str(e.value)


def test_generated_snippets_match_their_c_restatement(pt):
    """The GLSL that pt_scene_generate writes for PT_GEN_SDF_VARIED jobs
    (mandelbulbs of any power, Menger sponges of 3-5 levels), translated and
    built for the CPU, agrees bit for bit with the oracle's restatement."""
    from oracle import oracle
    from pathtracer_gb300 import Scene, native
    from user_snippets import generated_params, set_generated

    texts = {}
    for seed in range(2000, 2040):
        sc, spec = Scene.generate(native.PT_GEN_SDF_VARIED, seed)
        src = sc.sdf_sources()[0]
        if generated_params(src):
            texts.setdefault(generated_params(src)[0], []).append(src)
    assert len(texts.get("mandelbulb", [])) >= 2 and len(texts.get("menger", [])) >= 2
    pts = _points(n=4000, scale=0.9)
    for kind, srcs in texts.items():
        for k, src in enumerate(srcs[:3]):
            lib = _cpu_build(pt, f"gen_{kind}_{k}", {"g": src})
            fs, fm = _fn(lib, "c_g_sdf"), _fn(lib, "c_g_mat")
            rs_name, rm_name = set_generated(src)
            rs, rm = oracle.user_fn(rs_name), oracle.user_fn(rm_name)
            bad = sum(_bits(fs(*map(float, p))) != _bits(rs(*map(float, p))) for p in pts)
            bad += sum(_bits(fm(*map(float, p))) != _bits(rm(*map(float, p))) for p in pts)
            assert bad == 0, (kind, generated_params(src), bad)


def test_scene_snippet_matches_its_c_restatement(pt):
    """The power-8, 12-iteration mandelbulb of scenes/mandelbulb12_plane.json,
    translated and built for the CPU, agrees bit for bit with the oracle's
    restatement; near the surface most points run many iterations."""
    import os

    from conftest import SCENES
    from oracle import oracle
    from pathtracer_gb300 import Scene

    src = Scene.load(os.path.join(SCENES, "mandelbulb12_plane.json")).sdf_sources()[0]
    assert oracle.restatement_for(src) == ("user_bulb8_sdf", "user_bulb8_material")
    lib = _cpu_build(pt, "bulb8", {"b": src})
    fs, fm = _fn(lib, "c_b_sdf"), _fn(lib, "c_b_mat")
    rs, rm = oracle.user_fn("user_bulb8_sdf"), oracle.user_fn("user_bulb8_material")
    pts = _points(n=6000, scale=1.2)
    bad = sum(_bits(fs(*map(float, p))) != _bits(rs(*map(float, p))) for p in pts)
    bad += sum(_bits(fm(*map(float, p))) != _bits(rm(*map(float, p))) for p in pts)
    assert bad == 0, bad
    u = oracle.user_sdfs()
    u.user_count(1)
    for p in pts[:1000]:
        rs(*map(float, p))
    import ctypes

    iters = (ctypes.c_uint64 * len(oracle.USER_COUNTERS)).in_dll(u, "user_counters")[0]
    u.user_count(0)
    assert 1000 < iters < 12 * 1000


def test_fbm_terrain_matches_its_c_restatement(pt):
    """The value-noise fBm terrain of scenes/menger_terrain_full.json (uint
    hashing, int lattice coordinates, 8 octaves), translated and built for the
    CPU, agrees bit for bit with the oracle's restatement, negative lattice
    coordinates included."""
    import os

    from conftest import SCENES
    from oracle import oracle
    from pathtracer_gb300 import Scene

    src = Scene.load(os.path.join(SCENES, "menger_terrain_full.json")).sdf_sources()[1]
    assert oracle.restatement_for(src) == ("user_fbm_sdf", "user_fbm_material")
    lib = _cpu_build(pt, "fbm", {"t": src})
    fs, fm = _fn(lib, "c_t_sdf"), _fn(lib, "c_t_mat")
    rs, rm = oracle.user_fn("user_fbm_sdf"), oracle.user_fn("user_fbm_material")
    pts = _points(n=6000, scale=20.0)
    bad = sum(_bits(fs(*map(float, p))) != _bits(rs(*map(float, p))) for p in pts)
    bad += sum(_bits(fm(*map(float, p))) != _bits(rm(*map(float, p))) for p in pts)
    assert bad == 0, bad
    vals = [rs(float(x), 0.0, float(z)) for x, _, z in pts[:500]]
    assert max(abs(v) for v in vals) < 0.2 and len(set(vals)) > 400  # heights within +-0.3, a varied field


HASHED = """
// A hashed jitter: uint arithmetic, a side-effecting helper in a vector
// constructor, swizzle assignment and boolean vectors.
void pcg(inout uint s)
{
    uint state = s * 747796405u + 2891336453u;
    uint word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    s = (word >> 22u) ^ word;
}
float rnd(inout uint s) { pcg(s); return float(s) / 0xFFFFFFFFu; }
float sdf(vec3 p)
{
    uint s = uint(floor(p.x * 4.0) + 64.0) * 97u + uint(floor(p.z * 4.0) + 64.0);
    vec2 j = vec2(rnd(s), rnd(s));
    vec4 q = vec4(p, 1.0);
    q.xy -= 0.1 * j;
    q.zw = vec2(q.z, 0.5);
    bvec2 in2 = bvec2(q.x > 0.0, q.y > 0.0);
    float r = in2.x ? 0.5 : 0.45;
    return length(q.xyz) - r;
}
float sdfmaterial(vec3 p) { return 1.0; }
"""


def test_integer_boolean_and_swizzle_vocabulary(pt):
    """uint hashing, bvec, swizzle assignment and a vector constructor whose
    arguments draw random numbers: translated as GLSL means them (arguments
    left to right through a braced constructor), compiled by NVRTC for
    sm_103 and by g++, and the CPU build matches a Python restatement."""
    import numpy as np

    out = " ".join(pt.glsl_translate(HASHED, "h_").split())
    assert "vec2{h_rnd(s), h_rnd(s)}" in out
    assert "q.set_xy(q.xy() - ( 0.1f * j));" in out and "q.set_zw( vec2(q.z, 0.5f));" in out
    assert "uint& s" in out and "bvec2 in2" in out
    pt.jit_check([HASHED], sm=103)
    lib = _cpu_build(pt, "hashed", {"h": HASHED})
    f = _fn(lib, "c_h_sdf")

    def pcg(s):
        state = (s * 747796405 + 2891336453) & 0xFFFFFFFF
        word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & 0xFFFFFFFF
        return ((word >> 22) ^ word) & 0xFFFFFFFF

    f32 = np.float32
    for x, y, z in _points(n=300, scale=1.0):
        x, y, z = f32(x), f32(y), f32(z)
        s = (int(np.floor(x * f32(4.0)) + f32(64.0)) * 97 + int(np.floor(z * f32(4.0)) + f32(64.0))) & 0xFFFFFFFF
        s = pcg(s)
        jx = f32(s) / f32(4294967295.0)
        s = pcg(s)
        jy = f32(s) / f32(4294967295.0)
        qx, qy = x - f32(0.1) * jx, y - f32(0.1) * jy
        r = f32(0.5) if qx > 0 else f32(0.45)
        want = np.sqrt(f32(qx * qx + qy * qy) + z * z, dtype=np.float32) - r
        assert abs(f(float(x), float(y), float(z)) - want) <= 1e-6 * max(1.0, abs(want))


def test_structs_keep_member_names(pt):
    """A struct declared in a snippet passes through; its members named like
    colour components (`a`, `b`) keep their names (in such a snippet `.a` and
    `.b` are not read as vector components), an `inout` parameter of the
    struct type becomes a reference, and the result matches GLSL."""
    text = """
struct Shape { vec3 c; float a, b; };
void grow(inout Shape s, float k) { s.a *= k; s.b += k; }
float sdf(vec3 p)
{
    Shape s;
    s.c = vec3(0.0, 0.5, 0.0);
    s.a = 0.5;
    s.b = 0.1;
    grow(s, 2.0);
    vec4 q = vec4(p - s.c, 1.0);
    return length(q.xyz) - s.a;
}
float sdfmaterial(vec3 p) { return 1.0; }
"""
    out = " ".join(pt.glsl_translate(text, "s_").split())
    assert "s.a *= k; s.b += k;" in out and "Shape& s" in out
    pt.jit_check([text], sm=103)
    f = _fn(_cpu_build(pt, "shape", {"s": text}), "c_s_sdf")
    for x, y, z in _points(n=50, scale=1.0):
        want = np.sqrt(np.float32(x * x + (y - 0.5) ** 2 + z * z), dtype=np.float32) - 1.0
        assert abs(f(float(x), float(y), float(z)) - want) < 1e-5
