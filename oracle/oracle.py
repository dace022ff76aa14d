"""ctypes wrapper of the CPU restatement of src/shader.comp (oracle/pt_oracle.c).

TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU-baseline
leg of bench.py use it as the oracle.  The product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libpt_oracle.so")


class PtoTrace(ctypes.Structure):
    _fields_ = [
        ("depth_cap", ctypes.c_int),
        ("events", ctypes.c_void_p),
        ("nevents", ctypes.c_void_p),
        ("colors", ctypes.c_void_p),
        ("counters", ctypes.c_void_p),
    ]


_lib = None


def build() -> str:
    src = os.path.join(HERE, "pt_oracle.c")
    deps = [src, os.path.join(HERE, "pt_oracle.h"), os.path.join(HERE, "..", "include", "pt_cuda.h"),
            os.path.join(HERE, "..", "include", "pt_mathf.h")]
    if not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        subprocess.run([os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-std=c11", "-ffp-contract=off",
                        "-fno-fast-math", "-fopenmp", "-shared", "-o", LIB, src, "-lm"], check=True)
    return LIB


USER_LIB = os.path.join(HERE, "_build", "libpt_user_sdfs.so")
_user = None


def user_sdfs() -> ctypes.CDLL:
    """The C restatements of the test snippets (oracle/user_sdfs.c)."""
    global _user
    if _user is None:
        src = os.path.join(HERE, "user_sdfs.c")
        deps = [src, os.path.join(HERE, "..", "include", "pt_mathf.h")]
        if not os.path.exists(USER_LIB) or any(os.path.getmtime(d) > os.path.getmtime(USER_LIB) for d in deps):
            os.makedirs(os.path.dirname(USER_LIB), exist_ok=True)
            subprocess.run([os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-std=c11", "-ffp-contract=off",
                            "-fno-fast-math", "-shared", "-o", USER_LIB, src, "-lm"], check=True)
        _user = ctypes.CDLL(USER_LIB)
    return _user


def user_fn(name: str):
    """A float(float, float, float) function of user_sdfs.c."""
    f = getattr(user_sdfs(), name)
    f.restype = ctypes.c_float
    f.argtypes = [ctypes.c_float] * 3
    return f


def set_user_sdf(slot: int, sdf_name: str | None, material_name: str | None = None) -> None:
    """Registers user_sdfs.c functions for a PT_SDF_CUSTOM slot (None clears it)."""
    fs = ctypes.cast(getattr(user_sdfs(), sdf_name), ctypes.c_void_p) if sdf_name else None
    fm = ctypes.cast(getattr(user_sdfs(), material_name), ctypes.c_void_p) if material_name else None
    if lib().pto_set_user_sdf(slot, fs, fm) != 0:
        raise ValueError(f"bad SDF slot {slot}")


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.pto_dispatch.restype = ctypes.c_int
        L.pto_dispatch.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(PtoTrace), ctypes.c_int]
        L.pto_dispatch_ext.restype = ctypes.c_int
        L.pto_dispatch_ext.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.POINTER(PtoTrace), ctypes.c_int]
        L.pto_pcg32.restype = ctypes.c_uint32
        L.pto_pcg32.argtypes = [ctypes.c_uint32]
        L.pto_random_float.restype = ctypes.c_float
        L.pto_random_float.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
        L.pto_generate_seed.restype = ctypes.c_uint32
        L.pto_generate_seed.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int]
        L.pto_bk7_index.restype = ctypes.c_float
        L.pto_bk7_index.argtypes = [ctypes.c_float]
        L.pto_blackbody.restype = None
        L.pto_blackbody.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p]
        L.pto_blackbody_peak.restype = ctypes.c_float
        L.pto_blackbody_peak.argtypes = [ctypes.c_float]
        L.pto_set_user_sdf.restype = ctypes.c_int
        L.pto_set_user_sdf.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.pto_sdf_eval.restype = ctypes.c_float
        L.pto_sdf_eval.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.pto_sdf_material.restype = ctypes.c_float
        L.pto_sdf_material.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.pto_wave_to_xyz.restype = None
        L.pto_wave_to_xyz.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p]
        L.pto_mathf_eval.restype = ctypes.c_int
        L.pto_mathf_eval.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib = L
    return _lib


def dispatch(ubo: np.ndarray, push, plugins: list, accum: np.ndarray, rect=None, trace_depth: int = 0,
             nthreads: int = 0, ext=None):
    """Runs the shader over rect=(x0, y0, x1, y1) (default: the whole frame).

    Returns (events, nevents, colors) when trace_depth > 0, else None.
    accum is updated in place (H x W x 4 float32).
    """
    W, H = push.resolution[0], push.resolution[1]
    x0, y0, x1, y1 = rect if rect is not None else (0, 0, W, H)
    spf = push.samplesPerFrame
    npaths = (x1 - x0) * (y1 - y0) * spf
    tr = None
    out = None
    if trace_depth > 0:
        ev = np.zeros(npaths * trace_depth, np.uint32)
        nev = np.zeros(npaths, np.uint32)
        col = np.zeros(npaths * 3, np.float32)
        tr = PtoTrace(trace_depth, ev.ctypes.data, nev.ctypes.data, col.ctypes.data, None)
        out = (ev.reshape(npaths, trace_depth), nev, col.reshape(npaths, 3))
    arr = _plugin_array(plugins)
    assert accum.dtype == np.float32 and accum.flags["C_CONTIGUOUS"] and accum.size == W * H * 4
    rc = lib().pto_dispatch_ext(ubo.ctypes.data, _ext_ptr(ext), ctypes.addressof(push), ctypes.addressof(arr),
                                len(plugins), accum.ctypes.data, x0, y0, x1, y1, ctypes.byref(tr) if tr else None,
                                nthreads)
    if rc != 0:
        raise RuntimeError(f"pto_dispatch failed: {rc}")
    return out


def _ext_ptr(ext):
    """The address of a scene extension block (any ctypes struct of the
    pt_scene_ext layout) or None for the reference's method."""
    if ext is None or not ext.flags:
        return None
    return ctypes.addressof(ext)


def _plugin_array(plugins: list):
    """The plug-ins as a C array of the oracle's slot struct (same layout as
    pt_sdf_plugin: kind, material mode, three material constants)."""
    from .pack import PtoSdfPlugin

    arr = (PtoSdfPlugin * max(1, len(plugins)))()
    for i, p in enumerate(plugins):
        arr[i].kind, arr[i].material_mode = p.kind, p.material_mode
        arr[i].material[:] = list(p.material)
    return arr


# atan2 takes (y, x) like GLSL's atan(y, x): the first array is y.
MATHF = {"sin": 0, "cos": 1, "exp": 2, "log": 3, "pow": 4, "acos": 5, "asin": 6, "atan": 7, "atan2": 8, "exp2": 9,
         "log2": 10}


def mathf(fn: str, x: np.ndarray, y: np.ndarray | None = None) -> np.ndarray:
    """pt_mathf function `fn` on the CPU over float32 arrays."""
    x = np.ascontiguousarray(x, np.float32)
    yy = np.ascontiguousarray(y if y is not None else x, np.float32)
    out = np.empty_like(x)
    rc = lib().pto_mathf_eval(MATHF[fn], x.ctypes.data, yy.ctypes.data, out.ctypes.data, x.size)
    if rc != 0:
        raise ValueError(fn)
    return out


COUNTERS = ["samples", "path_rays", "shadow_rays", "sphere", "plane", "bounding_sphere", "box", "lens_slice",
            "cyclide", "aabb", "march_steps", "sdf_blob", "sdf_mandelbulb", "mandelbulb_iters", "sdf_menger",
            "sdf_terrain", "sdf_material", "emit", "brdf", "surface_hits", "sdf_custom"]
# Loop iterations inside the C restatements of GLSL snippets (user_sdfs.c).
USER_COUNTERS = ["bulb8_iters", "user_mandelbulb_iters"]


def count_work(ubo: np.ndarray, push, plugins: list, rect=None, nthreads: int = 0, ext=None) -> dict:
    """Runs the shader over rect with the work counters on; returns them by name."""
    W, H = push.resolution[0], push.resolution[1]
    x0, y0, x1, y1 = rect if rect is not None else (0, 0, W, H)
    cnt = np.zeros(len(COUNTERS), np.uint64)
    tr = PtoTrace(0, None, None, None, cnt.ctypes.data)
    arr = _plugin_array(plugins)
    accum = np.zeros((H, W, 4), np.float32)
    user = user_sdfs()
    user.user_count(1)
    try:
        rc = lib().pto_dispatch_ext(ubo.ctypes.data, _ext_ptr(ext), ctypes.addressof(push), ctypes.addressof(arr),
                                    len(plugins), accum.ctypes.data, x0, y0, x1, y1, ctypes.byref(tr), nthreads)
        ucnt = list((ctypes.c_uint64 * len(USER_COUNTERS)).in_dll(user, "user_counters"))
    finally:
        user.user_count(0)
    if rc != 0:
        raise RuntimeError(f"pto_dispatch failed: {rc}")
    out = {k: int(v) for k, v in zip(COUNTERS, cnt)}
    out.update({k: int(v) for k, v in zip(USER_COUNTERS, ucnt)})
    return out


def generated_params(text: str):
    """(kind, parameters) of an SDF text pt_scene_generate writes for
    PT_GEN_SDF_VARIED, read from its first line, or None for other text."""
    import re

    m = re.match(r"// Mandelbulb of power ([0-9.]+), ([0-9]+) iterations", text)
    if m:
        return "mandelbulb", (float(m.group(1)), int(m.group(2)))
    m = re.match(r"// Menger sponge, ([0-9]+) levels", text)
    if m:
        return "menger", (int(m.group(1)),)
    return None


def set_generated(text: str):
    """Points the restatement of a generated snippet at its parameters;
    returns the names of its sdf and sdfmaterial functions."""
    kind, prm = generated_params(text)
    u = user_sdfs()
    if kind == "mandelbulb":
        u.user_mandelbulb_set.argtypes = [ctypes.c_float, ctypes.c_int]
        u.user_mandelbulb_set(float(np.float32(prm[0])), prm[1])
        return "user_mandelbulb_sdf", "user_mandelbulb_material"
    u.user_menger_set.argtypes = [ctypes.c_int]
    u.user_menger_set(prm[0])
    return "user_menger_sdf", "user_menger_material"


def plugins_for_sources(sources: list[str]) -> list:
    """The oracle's plug-in per SDF slot from the scene's texts alone (no
    product library): shipped snippets and builtin keys by oracle/pack.py,
    other text by its C restatement in user_sdfs.c (restatement_for)."""
    from . import pack

    out = []
    for slot, src in enumerate(sources):
        p = pack.plugin_for(src)
        if p.kind == pack.SDF_CUSTOM:
            names = restatement_for(src)
            if names is None:
                raise ValueError(f"no C restatement of the SDF text: {src[:60]!r}")
            set_user_sdf(slot, *names)
        out.append(p)
    return out


# First line of the SDF text of pathtracer_gb300/scenes/mandelbulb12_plane.json.
BULB8_HEADER = "// Mandelbulb of power 8 in Chebyshev form, 12 iterations, bailout 2."
# First line of the terrain text of pathtracer_gb300/scenes/menger_terrain_full.json.
FBM_HEADER = "// Terrain: 8-octave value-noise fBm height field, amplitude 0.3, seed 7."


def restatement_for(text: str):
    """(sdf, sdfmaterial) names in user_sdfs.c of the C restatement of a
    scene's GLSL text that the repository's scenes and generator write
    (the generated mandelbulbs and sponges with their parameters set), or
    None for other text."""
    if text.startswith(BULB8_HEADER):
        return "user_bulb8_sdf", "user_bulb8_material"
    if text.startswith(FBM_HEADER):
        return "user_fbm_sdf", "user_fbm_material"
    if generated_params(text) is not None:
        return set_generated(text)
    return None
