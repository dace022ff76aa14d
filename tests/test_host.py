"""The headless host (libpt_host): scene JSON, uniform-buffer packing,
push constants, export tonemap and PPM — the parts of src/pathtracer.cpp (PT)
that sit above the compute dispatch."""
import glob
import json
import os

import numpy as np
import pytest

from conftest import REFERENCE, SCENES, reference_available


@pytest.fixture(scope="module")
def api(built):
    from pathtracer_gb300 import PathTracerError, Scene, cie_analytic, export_rgb8, native

    return {"Scene": Scene, "Err": PathTracerError, "cie": cie_analytic, "export": export_rgb8, "native": native}


def _off(name):
    from pathtracer_gb300.native import UBO_OFFSETS

    return UBO_OFFSETS[name][0]


MIN_SCENE = {
    "camera": {"numShots": 1, "position": [[1.0, 2.0, 3.0]], "angle": [[30.0, -10.0]], "ISO": 100, "size": 0.05,
               "apertureSize": 0.002, "apertureDistance": 0.04, "lensRadius": 0.01, "lensFocalLength": 0.03,
               "lensThickness": 0.0, "lensDistance": 0.05},
}


def test_missing_arrays_are_empty(api):
    s = api["Scene"].parse(json.dumps(MIN_SCENE))
    assert s.counts() == {"spheres": 0, "planes": 0, "boxes": 0, "lenses": 0, "cyclides": 0, "sdfs": 0,
                          "materials": 0, "lights": 0, "shots": 1}
    ubo = s.pack_ubo(None)
    assert np.all(ubo == 0.0)


@pytest.mark.parametrize("bad", ["{", "[]", '{"camera": {}}', "", '{"camera": 1}', "nul"])
def test_malformed_scene_is_an_error(api, bad):
    with pytest.raises(api["Err"]):
        api["Scene"].parse(bad)


def test_missing_object_field_is_an_error(api):
    sc = dict(MIN_SCENE, sphere=[{"position": [0, 0, 0], "radius": 1.0, "materialID": 1}])
    with pytest.raises(api["Err"]) as e:
        api["Scene"].parse(json.dumps(sc))
    assert "lightID" in str(e.value)


def test_pack_layout_and_light_list(api):
    """UpdateUniformBuffer (PT:3642-3811): strides 6/5/11/12/16, 1-based IDs
    stored as floats, the light list in scene order, and the lens/cyclide
    quirk that tests planes[i].lightID (PT:3704, PT:3728)."""
    sc = dict(MIN_SCENE)
    sc["sphere"] = [{"position": [1, 2, 3], "radius": 0.5, "materialID": 2, "lightID": 1},
                    {"position": [4, 5, 6], "radius": 1.5, "materialID": 1, "lightID": 0}]
    sc["plane"] = [{"position": [0, -1, 0], "materialID": 1, "lightID": 2}]
    sc["box"] = [{"position": [7, 8, 9], "rotation": [10, 20, 30], "size": [1, 2, 3], "materialID": 3,
                  "lightID": 1}]
    sc["lens"] = [{"position": [1, 1, 1], "rotation": [0, 0, 0], "radius": 0.5, "focalLength": 1.0,
                   "thickness": 0.1, "isConverging": False, "materialID": 1, "lightID": 0}]
    sc["cyclide"] = [{"position": [2, 2, 2], "rotation": [0, 0, 0], "scale": [0.5, 0.25, 0.75], "a": 1.0,
                      "b": 2.0, "c": 3.0, "d": 4.0, "boundingRadius": 2.0, "materialID": 1, "lightID": 0}]
    sc["sdf"] = [{"position": [0, 1, 0], "boundingSize": [2, 2, 2], "builtin": "menger"}]
    sc["material"] = [{"reflection": {"peakWavelength": 550.0, "sigma": 10.0, "isInvert": True}}]
    sc["light"] = [{"emission": {"temperature": 5000.0, "luminosity": 3.0}},
                   {"emission": {"temperature": 6000.0, "luminosity": 4.0}}]
    ubo = api["Scene"].parse(json.dumps(sc)).pack_ubo(np.arange(1323, dtype=np.float32))
    assert list(ubo[:7]) == [2, 1, 1, 1, 1, 1, 5]
    o = _off("objects")
    assert list(ubo[o:o + 6]) == [1, 2, 3, 0.5, 2, 1]
    assert list(ubo[o + 12:o + 17]) == [0, -1, 0, 1, 2]
    assert list(ubo[o + 17:o + 28]) == [7, 8, 9, 10, 20, 30, 1, 2, 3, 3, 1]
    assert list(ubo[o + 28:o + 40]) == [1, 1, 1, 0, 0, 0, 0.5, 1.0, 0.1, 0.0, 1, 0]
    cyc = ubo[o + 40:o + 56]
    assert cyc[13] == np.float32(2.0 * 2.0 * (0.75 * 0.75))  # brad^2 * max(scale)^2
    # light list: sphere 0, plane (index 2), box (index 3); the lens and the
    # cyclide are listed because planes[0].lightID > 0 (the quirk).
    li = _off("lightIDs")
    assert list(ubo[li:li + 6]) == [0, 2, 3, 4, 5, 0]
    assert list(ubo[_off("materials"):_off("materials") + 3]) == [550, 10, 1]
    assert list(ubo[_off("lights"):_off("lights") + 4]) == [5000, 3, 6000, 4]
    assert list(ubo[_off("sdfs"):_off("sdfs") + 6]) == [0, 1, 0, 2, 2, 2]
    assert ubo[_off("CIEXYZ1931") + 1322] == 1322.0


def test_pack_overflow_is_an_error(api):
    sc = dict(MIN_SCENE, sphere=[{"position": [0, 0, 0], "radius": 1.0, "materialID": 1, "lightID": 0}] * 171)
    with pytest.raises(api["Err"]):
        api["Scene"].parse(json.dumps(sc)).pack_ubo(None)  # 171 * 6 = 1026 > 1024 floats


def test_push_constants(api):
    """UpdatePushConstant (PT:3813-3834): cameraAngle = (-angle.y, angle.x)."""
    sc = dict(MIN_SCENE)
    sc["camera"] = dict(MIN_SCENE["camera"], numShots=2, position=[[1, 2, 3], [4, 5, 6]],
                        angle=[[30.0, -10.0], [45.0, 5.0]])
    s = api["Scene"].parse(json.dumps(sc))
    p = s.push_constants(640, 360, 24, 8, 8, 5, shot=2, tonemap=2)
    assert list(p.resolution) == [640, 360] and p.frame == 24 and p.currentSamples == 8
    assert p.samplesPerFrame == 8 and p.pathLength == 5 and p.tonemap == 2
    assert list(p.cameraAngle) == [-5.0, 45.0]
    assert (p.cameraPosX, p.cameraPosY, p.cameraPosZ) == (4.0, 5.0, 6.0)
    assert p.ISO == 100 and abs(p.apertureSize - 0.002) < 1e-9
    with pytest.raises(api["Err"]):
        s.push_constants(640, 360, 8, 8, 8, 5, shot=3)


def test_own_scenes_round_trip(api):
    # UpdateToJSON rounds every float to 1e-5 (RoundDecimal, PT:935-943), so
    # the first save may change values; from then on save/load is a fixed point.
    for f in glob.glob(os.path.join(SCENES, "*.json")):
        once = api["Scene"].parse(api["Scene"].load(f).to_json())
        twice = api["Scene"].parse(once.to_json())
        assert twice.to_json() == once.to_json()
        assert np.array_equal(once.pack_ubo(None), twice.pack_ubo(None))


@pytest.mark.skipif(not reference_available(), reason="reference tree not mounted")
def test_reference_scenes_round_trip_byte_for_byte(api):
    """UpdateFromJSON then UpdateToJSON + dump(4) reproduces every reference
    scene file byte for byte (line endings aside)."""
    for f in sorted(glob.glob(os.path.join(REFERENCE, "scenes", "*.json"))):
        text = open(f, "rb").read()
        s = api["Scene"].parse(text)
        assert s.to_json() == text.decode().replace("\r\n", "\n").rstrip("\n"), f


@pytest.mark.skipif(not reference_available(), reason="reference tree not mounted")
def test_reference_sdf_snippets_are_recognised(api):
    """Every SDF snippet of sdfs/ and of the scene files maps to its plug-in."""
    import ctypes

    lib = api["native"].cuda()
    want = {"blob": 1, "mandelbulb": 2, "menger": 3, "terrain": 4}
    for name, kind in want.items():
        p = api["native"].PtSdfPlugin()
        assert lib.pt_parse_sdf_source(open(os.path.join(REFERENCE, "sdfs", name + ".glsl"), "rb").read(),
                                       ctypes.byref(p)) == 0
        assert p.kind == kind
    for f in glob.glob(os.path.join(REFERENCE, "scenes", "*.json")):
        for sdf in api["Scene"].load(f).sdf_sources():
            p = api["native"].PtSdfPlugin()
            assert lib.pt_parse_sdf_source(sdf.encode(), ctypes.byref(p)) == 0, f


def test_builtin_specs_and_unknown_source(api):
    import ctypes

    lib = api["native"].cuda()
    p = api["native"].PtSdfPlugin()
    assert lib.pt_parse_sdf_source(b"builtin:blob:3,4,5", ctypes.byref(p)) == 0
    assert (p.kind, p.material_mode, list(p.material)) == (1, 0, [3.0, 4.0, 5.0])
    assert lib.pt_parse_sdf_source(b"builtin:mandelbulb_const:3", ctypes.byref(p)) == 0
    assert (p.kind, p.material_mode, p.material[0]) == (2, 1, 3.0)
    assert lib.pt_parse_sdf_source(b"builtin:torus", ctypes.byref(p)) == api["native"].PT_ERR_UNSUPPORTED
    assert lib.pt_parse_sdf_source(b"float sdf(in vec3 p) { return length(p) - 1.0; }",
                                   ctypes.byref(p)) == api["native"].PT_ERR_UNSUPPORTED
    # the fingerprint ignores whitespace layout
    fp = lib.pt_sdf_source_fingerprint
    assert fp(b"float  sdf(in vec3 p)\r\n{\treturn 1.0; }\n") == fp(b"float sdf(in vec3 p) { return 1.0; }")


def test_export_tonemap_chain(api):
    """SaveRender (PT:3491-3518): E->D65, XYZ->sRGB, max(0), tonemap, sRGB
    companding, byte truncation; checked against a float64 restatement."""
    rng = np.random.default_rng(5)
    acc = np.zeros((4, 8, 4), np.float32)
    acc[..., :3] = rng.uniform(0, 3, (4, 8, 3))
    acc[0, 0, :3] = 0.0
    m1 = np.array([[0.9531874, -0.0265906, 0.0238731], [-0.0382467, 1.0288406, 0.0094060],
                   [0.0026068, -0.0030332, 1.0892565]], np.float32)
    m2 = np.array([[3.2404542, -1.5371385, -0.4985314], [-0.9692660, 1.8760108, 0.0415560],
                   [0.0556434, -0.2040259, 1.0572252]], np.float32)
    for tm in (0, 1, 2, 3):
        got = api["export"](acc, tm).astype(int)
        c = acc[..., :3].astype(np.float64) @ m1.T.astype(np.float64) @ m2.T.astype(np.float64)
        c = np.maximum(c, 0)
        with np.errstate(divide="ignore"):
            if tm == 1:
                c = c / (1 + c)
            elif tm == 2:
                c = c * (2.51 * c + 0.03) / (c * (2.43 * c + 0.59) + 0.14)
            elif tm == 3:
                c = np.exp(-0.25 / c)
        c = np.clip(c, 0, 1)
        c = np.where(c <= 0.0031308, 12.92 * c, 1.055 * c ** (1 / 2.4) - 0.055)
        want = (c * 255.0).astype(int)
        assert np.abs(got - want).max() <= 1, tm


def test_save_ppm(api, tmp_path):
    rgb = np.arange(2 * 3 * 3, dtype=np.uint8).reshape(2, 3, 3)
    path = str(tmp_path / "x.ppm")
    assert api["native"].host().pt_save_ppm(path.encode(), rgb.ctypes.data, 3, 2) == 0
    data = open(path, "rb").read()
    assert data == b"P6\n3\n2\n255\n" + rgb.tobytes()


def test_cie_analytic_table(api):
    cie = api["cie"]().reshape(441, 3)
    # peaks of the fit: x-bar near 599 nm (~1.06), y-bar near 556 nm (~1.0), z-bar near 446 nm (~1.78)
    assert 595 <= 360 + int(np.argmax(cie[:, 0])) <= 602 and abs(cie[:, 0].max() - 1.06) < 0.02
    assert 550 <= 360 + int(np.argmax(cie[:, 1])) <= 562 and abs(cie[:, 1].max() - 1.0) < 0.02
    assert 440 <= 360 + int(np.argmax(cie[:, 2])) <= 452 and abs(cie[:, 2].max() - 1.78) < 0.05


@pytest.mark.skipif(not reference_available(), reason="reference tree not mounted")
def test_cie_fit_close_to_reference_table(api):
    """The analytic fit stays within a few percent of the tabulated CIE 1931
    functions (PT:396-842), read from the reference source."""
    src = open(os.path.join(REFERENCE, "src", "pathtracer.cpp")).read()
    body = src[src.index("const float CIEXYZ1931[1323] = {"):]
    body = body[body.index("{") + 1:body.index("};")]
    table = np.array([float(t.strip().rstrip("f")) for t in body.split(",") if t.strip()], np.float64)
    assert table.size == 1323
    fit = api["cie"]().astype(np.float64)
    assert np.abs(fit - table).max() < 0.05
