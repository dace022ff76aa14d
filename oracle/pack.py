"""The reference host's scene loading, uniform-buffer packing and push
constants, restated in Python for the oracle's side.

TEST INFRASTRUCTURE ONLY: the tests and the CPU legs of bench.py use it so
that the oracle (and the reference's own shader built for the CPU) can be fed
without the product's libraries.  It follows src/pathtracer.cpp of the
reference:
- `load_scene`: UpdateFromJSON (src/pathtracer.cpp:2576-2722), the scene JSON
  schema read with nlohmann's conversions: numbers to float, IDs to int
  (truncating), `isConverging` / `isInvert` booleans, a missing array as
  empty (`scene["sphere"].size()` is 0 for a missing key);
- `pack_ubo`: UpdateUniformBuffer (src/pathtracer.cpp:3642-3811), with the
  light list's quirk of testing `planes[i].lightID` for lenses and cyclides
  (:3704, :3728; past the end of the plane list no light is added);
- `push_constants`: UpdatePushConstant (src/pathtracer.cpp:3813-3834) with
  the host's defaults (frameTime 0.0166, persistence 0.0625, :1164-1173);
- `cie_analytic`: a CIE 1931 matching-function table from the multi-lobe
  Gaussian fit of Wyman, Sloan and Shirley (2013) at 1 nm over 360-800 nm,
  for callers without the reference's tabulated CIEXYZ1931 (which is not
  redistributed here);
- `plugins`: which shipped SDF snippet (sdfs/*.glsl and the scene files'
  copies) a scene's `glsl` text is, by the hash of its whitespace-normalised
  text, or a `builtin:<name>` key; other text is a run-time compiled slot.

Float arithmetic is done in numpy float32 where the reference computes in
float, so the packed bytes equal the reference host's.
"""
from __future__ import annotations

import ctypes
import json
import math

import numpy as np

MAX_OBJECTS_SIZE = 1024
MAX_SDFS_SIZE = 768
MAX_MATERIALS_SIZE = 783
MAX_LIGHTS_SIZE = 128
MAX_LIGHTIDS_SIZE = 64
CIE_TABLE_SIZE = 1323
UBO_FLOATS = 7 + MAX_OBJECTS_SIZE + MAX_SDFS_SIZE + MAX_MATERIALS_SIZE + MAX_LIGHTS_SIZE + MAX_LIGHTIDS_SIZE + \
    CIE_TABLE_SIZE
_OFF = {"numObjects": 0, "objects": 7}
_OFF["sdfs"] = _OFF["objects"] + MAX_OBJECTS_SIZE
_OFF["materials"] = _OFF["sdfs"] + MAX_SDFS_SIZE
_OFF["lights"] = _OFF["materials"] + MAX_MATERIALS_SIZE
_OFF["lightIDs"] = _OFF["lights"] + MAX_LIGHTS_SIZE
_OFF["CIEXYZ1931"] = _OFF["lightIDs"] + MAX_LIGHTIDS_SIZE

SDF_NONE, SDF_BLOB, SDF_MANDELBULB, SDF_MENGER, SDF_TERRAIN, SDF_CUSTOM = range(6)
SDFMAT_DEFAULT, SDFMAT_CONSTANT = 0, 1


class PtoPush(ctypes.Structure):
    """The shader's push-constant block (src/shader.comp:31-52), 88 bytes."""

    _fields_ = [
        ("resolution", ctypes.c_int32 * 2),
        ("frame", ctypes.c_int32),
        ("currentSamples", ctypes.c_int32),
        ("samplesPerFrame", ctypes.c_int32),
        ("FPS", ctypes.c_float),
        ("persistence", ctypes.c_float),
        ("pathLength", ctypes.c_int32),
        ("cameraAngle", ctypes.c_float * 2),
        ("cameraPosX", ctypes.c_float),
        ("cameraPosY", ctypes.c_float),
        ("cameraPosZ", ctypes.c_float),
        ("ISO", ctypes.c_int32),
        ("cameraSize", ctypes.c_float),
        ("apertureSize", ctypes.c_float),
        ("apertureDist", ctypes.c_float),
        ("lensRadius", ctypes.c_float),
        ("lensFocalLength", ctypes.c_float),
        ("lensThickness", ctypes.c_float),
        ("lensDistance", ctypes.c_float),
        ("tonemap", ctypes.c_int32),
    ]


assert ctypes.sizeof(PtoPush) == 88


EXT_SKY, EXT_WAVELENGTHS, EXT_ANALYTIC_CMF, EXT_MARCH, EXT_MATERIALS = 1, 2, 4, 8, 16
BSDF_REFERENCE, BSDF_FLAT, BSDF_SMOOTH, BSDF_MIRROR, BSDF_CAUCHY, BSDF_SELLMEIER = range(6)
MAX_EXT_MATERIALS = 128


class PtoMaterialExt(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("p", ctypes.c_float * 6)]


class PtoSceneExt(ctypes.Structure):
    """A scene's full-form extensions as the oracle takes them (all zero: the
    reference's method): sky, wavelength range, analytic CMF, march limits,
    and surface models per material."""

    _fields_ = [
        ("flags", ctypes.c_int32),
        ("sky_temperature", ctypes.c_float),
        ("sky_luminosity", ctypes.c_float),
        ("lambda_min", ctypes.c_float),
        ("lambda_max", ctypes.c_float),
        ("march_max_steps", ctypes.c_int32),
        ("march_epsilon", ctypes.c_float),
        ("march_max_distance", ctypes.c_float),
        ("nmat", ctypes.c_int32),
        ("mat", PtoMaterialExt * MAX_EXT_MATERIALS),
    ]


_BSDF_KEYS = {
    "flat": (BSDF_FLAT, ("albedo",)),
    "smooth": (BSDF_SMOOTH, ("base", "amplitude", "center", "width")),
    "mirror": (BSDF_MIRROR, ("reflectance",)),
    "cauchy": (BSDF_CAUCHY, ("A", "B")),
}


def _bsdf(b) -> tuple[int, list]:
    """A material's "bsdf" object: (model, six parameters)."""
    if b is None:
        return BSDF_REFERENCE, [np.float32(0)] * 6
    t = b["type"]
    if t == "reference":
        return BSDF_REFERENCE, [np.float32(0)] * 6
    if t == "sellmeier":
        return BSDF_SELLMEIER, _vec(b["B"], 3) + _vec(b["C"], 3)
    if t not in _BSDF_KEYS:
        raise ValueError(f"material.bsdf.type: unknown {t!r}")
    kind, keys = _BSDF_KEYS[t]
    p = [_f(b[k]) for k in keys]
    return kind, p + [np.float32(0)] * (6 - len(p))


class PtoSdfPlugin(ctypes.Structure):
    """One SDF slot of the oracle: which shipped snippet, and the material
    constants the scene files vary in their copies of sdfmaterial."""

    _fields_ = [("kind", ctypes.c_int32), ("material_mode", ctypes.c_int32), ("material", ctypes.c_float * 3)]


def _f(v) -> np.float32:
    if isinstance(v, bool) or not isinstance(v, (int, float)):
        raise ValueError(f"expected a number, got {v!r}")
    return np.float32(v)


def _i(v) -> int:
    if isinstance(v, bool):
        return int(v)
    if isinstance(v, int):
        return v
    if isinstance(v, float):
        return int(v)  # truncation, as nlohmann's get<int>
    raise ValueError(f"expected an integer, got {v!r}")


def _b(v) -> bool:
    if isinstance(v, (bool, int, float)):
        return bool(v)
    raise ValueError(f"expected a boolean, got {v!r}")


def _vec(v, n):
    if not isinstance(v, list) or len(v) < n:
        raise ValueError(f"expected an array of {n}")
    return [_f(x) for x in v[:n]]


def _list(root, key):
    v = root.get(key)
    if v is None:
        return []
    if not isinstance(v, list):
        raise ValueError(f"{key}: expected an array")
    return v


class RefScene:
    """The reference host's in-memory scene (src/pathtracer.cpp:110-185)."""

    def __init__(self, root: dict):
        cam = root["camera"]
        n = _i(cam["numShots"])
        self.shots = [(_vec(cam["position"][i], 3), _vec(cam["angle"][i], 2)) for i in range(n)]
        self.ISO = _i(cam["ISO"])
        self.cam = {k: _f(cam[k]) for k in ("size", "apertureSize", "apertureDistance", "lensRadius",
                                            "lensFocalLength", "lensThickness", "lensDistance")}
        self.spheres = [dict(pos=_vec(o["position"], 3), radius=_f(o["radius"]), m=_i(o["materialID"]),
                             l=_i(o["lightID"])) for o in _list(root, "sphere")]
        self.planes = [dict(pos=_vec(o["position"], 3), m=_i(o["materialID"]), l=_i(o["lightID"]))
                       for o in _list(root, "plane")]
        self.boxes = [dict(pos=_vec(o["position"], 3), rot=_vec(o["rotation"], 3), size=_vec(o["size"], 3),
                           m=_i(o["materialID"]), l=_i(o["lightID"])) for o in _list(root, "box")]
        self.lenses = [dict(pos=_vec(o["position"], 3), rot=_vec(o["rotation"], 3), radius=_f(o["radius"]),
                            focal=_f(o["focalLength"]), thickness=_f(o["thickness"]),
                            conv=_b(o["isConverging"]), m=_i(o["materialID"]), l=_i(o["lightID"]))
                       for o in _list(root, "lens")]
        self.cyclides = [dict(pos=_vec(o["position"], 3), rot=_vec(o["rotation"], 3), scale=_vec(o["scale"], 3),
                              a=_f(o["a"]), b=_f(o["b"]), c=_f(o["c"]), d=_f(o["d"]),
                              brad=_f(o["boundingRadius"]), m=_i(o["materialID"]), l=_i(o["lightID"]))
                         for o in _list(root, "cyclide")]
        self.sdfs = []
        for o in _list(root, "sdf"):
            if isinstance(o.get("glsl"), str):
                src = o["glsl"]
            elif isinstance(o.get("builtin"), str):
                b = o["builtin"]
                src = b if b.startswith("builtin:") else "builtin:" + b
            else:
                raise ValueError('sdf: needs a "glsl" or "builtin" string')
            self.sdfs.append(dict(pos=_vec(o["position"], 3), size=_vec(o["boundingSize"], 3), src=src))
        self.materials = [[_f(o["reflection"]["peakWavelength"]), _f(o["reflection"]["sigma"]),
                           np.float32(1.0 if _b(o["reflection"]["isInvert"]) else 0.0)]
                          for o in _list(root, "material")]
        self.lights = [[_f(o["emission"]["temperature"]), _f(o["emission"]["luminosity"])]
                       for o in _list(root, "light")]
        # Full-form extensions: keys the reference's loader does not read.
        self.bsdfs = [_bsdf(o.get("bsdf")) for o in _list(root, "material")]
        self.environment = root.get("environment")
        self.spectral = root.get("spectral") or {}
        self.march = root.get("march")

    def sdf_sources(self) -> list[str]:
        return [d["src"] for d in self.sdfs]

    def pack_ubo(self, cie: np.ndarray | None) -> np.ndarray:
        """UpdateUniformBuffer: the 4097-float uniform buffer (CIE table from the caller)."""
        objects, lightIDs = [], []
        ns, npl, nb, nl = len(self.spheres), len(self.planes), len(self.boxes), len(self.lenses)
        for i, o in enumerate(self.spheres):
            objects += [*o["pos"], o["radius"], o["m"], o["l"]]
            if o["l"] > 0:
                lightIDs.append(i)
        for i, o in enumerate(self.planes):
            objects += [*o["pos"], o["m"], o["l"]]
            if o["l"] > 0:
                lightIDs.append(ns + i)
        for i, o in enumerate(self.boxes):
            objects += [*o["pos"], *o["rot"], *o["size"], o["m"], o["l"]]
            if o["l"] > 0:
                lightIDs.append(ns + npl + i)
        for i, o in enumerate(self.lenses):
            objects += [*o["pos"], *o["rot"], o["radius"], o["focal"], o["thickness"], 1.0 if o["conv"] else 0.0,
                        o["m"], o["l"]]
            if i < npl and self.planes[i]["l"] > 0:  # src/pathtracer.cpp:3704 tests the plane's lightID
                lightIDs.append(ns + npl + nb + i)
        for i, o in enumerate(self.cyclides):
            m = max(max(o["scale"][0], o["scale"][1]), o["scale"][2])
            objects += [*o["pos"], *o["rot"], *o["scale"], o["a"], o["b"], o["c"], o["d"],
                        (o["brad"] * o["brad"]) * (m * m), o["m"], o["l"]]
            if i < npl and self.planes[i]["l"] > 0:  # src/pathtracer.cpp:3728 likewise
                lightIDs.append(ns + npl + nb + nl + i)
        sdfs = [x for d in self.sdfs for x in (*d["pos"], *d["size"])]
        materials = [x for m in self.materials for x in m]
        lights = [x for l in self.lights for x in l]
        for arr, cap, name in ((objects, MAX_OBJECTS_SIZE, "objects"), (sdfs, MAX_SDFS_SIZE, "sdfs"),
                               (materials, MAX_MATERIALS_SIZE, "materials"), (lights, MAX_LIGHTS_SIZE, "lights"),
                               (lightIDs, MAX_LIGHTIDS_SIZE, "lightIDs")):
            if len(arr) > cap:
                raise ValueError(f"{name}: {len(arr)} floats exceed the uniform buffer's {cap}")
        ubo = np.zeros(UBO_FLOATS, np.float32)
        ubo[0:7] = [ns, npl, nb, nl, len(self.cyclides), len(self.sdfs), len(lightIDs)]
        for arr, name in ((objects, "objects"), (sdfs, "sdfs"), (materials, "materials"), (lights, "lights"),
                          (lightIDs, "lightIDs")):
            ubo[_OFF[name]:_OFF[name] + len(arr)] = np.array(arr, np.float32)
        if cie is not None:
            ubo[_OFF["CIEXYZ1931"]:] = np.asarray(cie, np.float32)
        return ubo

    def push_constants(self, width: int, height: int, frame: int, current_samples: int, spf: int,
                       path_length: int, shot: int = 1, fps=None, persistence: float = 0.0625,
                       tonemap: int = 3) -> PtoPush:
        """UpdatePushConstant for camera shot `shot` (1-based) and the given frame state."""
        if not 1 <= shot <= len(self.shots):
            raise ValueError(f"camera shot {shot} of {len(self.shots)}")
        pos, ang = self.shots[shot - 1]
        if fps is None:
            fps = np.float32(1.0) / np.float32(0.0166)  # 1.0f / frameTime, frameTime's initial value
        p = PtoPush()
        p.resolution[0], p.resolution[1] = width, height
        p.frame, p.currentSamples, p.samplesPerFrame = frame, current_samples, spf
        p.FPS, p.persistence, p.pathLength = float(fps), persistence, path_length
        p.cameraAngle[0], p.cameraAngle[1] = float(-ang[1]), float(ang[0])
        p.cameraPosX, p.cameraPosY, p.cameraPosZ = (float(v) for v in pos)
        p.ISO = self.ISO
        p.cameraSize = float(self.cam["size"])
        p.apertureSize = float(self.cam["apertureSize"])
        p.apertureDist = float(self.cam["apertureDistance"])
        p.lensRadius = float(self.cam["lensRadius"])
        p.lensFocalLength = float(self.cam["lensFocalLength"])
        p.lensThickness = float(self.cam["lensThickness"])
        p.lensDistance = float(self.cam["lensDistance"])
        p.tonemap = tonemap
        return p

    def pack_ext(self) -> PtoSceneExt:
        """The scene's extension block (flags 0 for a reference-method scene)."""
        x = PtoSceneExt()
        if self.environment is not None:
            x.flags |= EXT_SKY
            x.sky_temperature = float(_f(self.environment["temperature"]))
            x.sky_luminosity = float(_f(self.environment["luminosity"]))
        if self.spectral.get("range") is not None:
            lo, hi = _vec(self.spectral["range"], 2)
            x.flags |= EXT_WAVELENGTHS
            x.lambda_min, x.lambda_max = float(lo), float(hi)
        if self.spectral.get("cmf") is not None:
            if self.spectral["cmf"] not in ("analytic", "table"):
                raise ValueError('spectral.cmf: "analytic" or "table"')
            if self.spectral["cmf"] == "analytic":
                x.flags |= EXT_ANALYTIC_CMF
        if self.march is not None:
            x.flags |= EXT_MARCH
            x.march_max_steps = _i(self.march["maxSteps"])
            x.march_epsilon = float(_f(self.march["epsilon"]))
            x.march_max_distance = float(_f(self.march["maxDistance"]))
        last = max((i + 1 for i, (k, _) in enumerate(self.bsdfs) if k != BSDF_REFERENCE), default=0)
        if last > MAX_EXT_MATERIALS:
            raise ValueError(f"{last} materials with extension models exceed {MAX_EXT_MATERIALS}")
        if last:
            x.flags |= EXT_MATERIALS
            x.nmat = last
            for i in range(last):
                k, p = self.bsdfs[i]
                x.mat[i].type = k
                x.mat[i].p[:] = [float(v) for v in p]
        return x

    def plugins(self) -> list:
        """The oracle's plug-in per SDF slot (kind SDF_CUSTOM for text that is
        not a shipped snippet: the caller registers its C restatement)."""
        return [plugin_for(d["src"]) for d in self.sdfs]


def load_scene(path: str) -> RefScene:
    with open(path, "rb") as f:
        return RefScene(json.loads(f.read()))


def parse_scene(text: str) -> RefScene:
    return RefScene(json.loads(text))


def _lobe(x: float, mu: float, s1: float, s2: float) -> float:
    t = (x - mu) / (s1 if x < mu else s2)
    return math.exp(-0.5 * t * t)


def cie_analytic() -> np.ndarray:
    """x, y, z at 360..800 nm in 1 nm steps from the multi-lobe fit, in double, stored as float."""
    out = np.zeros(CIE_TABLE_SIZE, np.float32)
    for i in range(CIE_TABLE_SIZE // 3):
        l = 360.0 + i
        x = 1.056 * _lobe(l, 599.8, 37.9, 31.0) + 0.362 * _lobe(l, 442.0, 16.0, 26.7) - \
            0.065 * _lobe(l, 501.1, 20.4, 26.2)
        y = 0.821 * _lobe(l, 568.8, 46.9, 40.5) + 0.286 * _lobe(l, 530.9, 16.3, 31.1)
        z = 1.217 * _lobe(l, 437.0, 11.8, 36.0) + 0.681 * _lobe(l, 459.0, 26.0, 13.8)
        out[3 * i:3 * i + 3] = (x, y, z)
    return out


# Whitespace-normalised FNV-1a-64 hashes of the shipped snippets: the four
# files in sdfs/ and the copies in scenes/scene3..7.json (which differ only
# in sdfmaterial's constants), with the slot each selects.
_FINGERPRINTS = {
    0x6de57505fc723c7e: (SDF_BLOB, SDFMAT_DEFAULT, (4.0, 5.0, 6.0)),        # sdfs/blob.glsl
    0xdcc8f6bccda6d8d9: (SDF_MANDELBULB, SDFMAT_DEFAULT, (4.0, 3.0, 0.0)),  # sdfs/mandelbulb.glsl
    0x3c94eee4f8b59872: (SDF_MENGER, SDFMAT_CONSTANT, (0.0, 0.0, 0.0)),     # sdfs/menger.glsl
    0x742b6d88271746b9: (SDF_TERRAIN, SDFMAT_CONSTANT, (0.0, 0.0, 0.0)),    # sdfs/terrain.glsl
    0xe86f17a11e62fd66: (SDF_BLOB, SDFMAT_DEFAULT, (3.0, 4.0, 5.0)),        # scenes/scene3.json, scene5.json
    0x5e591c833348e2e0: (SDF_MANDELBULB, SDFMAT_CONSTANT, (3.0, 0.0, 0.0)), # scenes/scene4.json
    0x02cb7b03b6d3b701: (SDF_MANDELBULB, SDFMAT_DEFAULT, (3.0, 2.0, 0.0)),  # scenes/scene6.json
    0xc8ce1f6bb7bbc161: (SDF_MANDELBULB, SDFMAT_DEFAULT, (5.0, 4.0, 0.0)),  # scenes/scene7.json
}
_BUILTINS = {
    "blob": (SDF_BLOB, SDFMAT_DEFAULT, (4.0, 5.0, 6.0)),
    "mandelbulb": (SDF_MANDELBULB, SDFMAT_DEFAULT, (4.0, 3.0, 0.0)),
    "mandelbulb_const": (SDF_MANDELBULB, SDFMAT_CONSTANT, (3.0, 0.0, 0.0)),
    "menger": (SDF_MENGER, SDFMAT_CONSTANT, (0.0, 0.0, 0.0)),
    "terrain": (SDF_TERRAIN, SDFMAT_CONSTANT, (0.0, 0.0, 0.0)),
}


def fingerprint(text: str) -> int:
    """FNV-1a-64 of the text with every whitespace run collapsed to one space
    and leading/trailing whitespace dropped."""
    h = 0xcbf29ce484222325
    for tok_i, tok in enumerate(text.encode().split()):
        if tok_i:
            h = ((h ^ 0x20) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
        for c in tok:
            h = ((h ^ c) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return h


def plugin_for(src: str) -> PtoSdfPlugin:
    if src.startswith("builtin:"):
        name, _, params = src[len("builtin:"):].partition(":")
        if name not in _BUILTINS:
            raise ValueError(f"unknown built-in SDF {name!r}")
        kind, mode, mat = _BUILTINS[name]
        mat = list(mat)
        if params:
            vals = params.split(",")
            if len(vals) > 3:
                raise ValueError(f"bad built-in SDF parameters {params!r}")
            for i, v in enumerate(vals):
                mat[i] = float(np.float32(float(v)))
        return PtoSdfPlugin(kind, mode, (ctypes.c_float * 3)(*mat))
    hit = _FINGERPRINTS.get(fingerprint(src))
    if hit is None:
        return PtoSdfPlugin(SDF_CUSTOM, SDFMAT_DEFAULT, (ctypes.c_float * 3)(0.0, 0.0, 0.0))
    kind, mode, mat = hit
    return PtoSdfPlugin(kind, mode, (ctypes.c_float * 3)(*mat))
