"""The oracle's restatement of the reference host's scene loading,
uniform-buffer packing and push constants (oracle/pack.py) against the
product's host library (libpt_host: pt_scene_parse, pt_scene_pack_ubo,
pt_scene_push_constants, pt_cie_analytic_table, pt_parse_sdf_source).

Both sides feed every parity test: the oracle gets what the packer made, so
an error shared by both would go unseen.  The restatement follows
UpdateFromJSON / UpdateUniformBuffer / UpdatePushConstant
(src/pathtracer.cpp:2576-2722, :3642-3811, :3813-3834) on its own; the two
must give the same bytes on the reference's 11 scene files, the repository's
scenes and generated jobs.
"""
import ctypes
import glob
import os

import numpy as np
import pytest

from conftest import REFERENCE, SCENES, reference_available


def _scene_files():
    files = sorted(glob.glob(os.path.join(SCENES, "*.json")))
    if reference_available():
        files += sorted(glob.glob(os.path.join(REFERENCE, "scenes", "*.json")))
    return files


def _check_same(text, product_scene, cie):
    from oracle import pack

    ref = pack.parse_scene(text)
    a = ref.pack_ubo(cie)
    b = product_scene.pack_ubo(cie)
    assert a.tobytes() == b.tobytes()
    assert ref.sdf_sources() == product_scene.sdf_sources()
    assert bytes(ref.pack_ext()) == bytes(product_scene.pack_ext())  # full-form extensions (zero when absent)
    for shot in range(1, len(ref.shots) + 1):
        for args in ((64, 48, 8, 8, 8, 6), (1024, 1024, 64, 16, 16, 12), (37, 23, 3, 3, 3, 0)):
            pa = ref.push_constants(*args, shot=shot)
            pb = product_scene.push_constants(*args, shot=shot)
            assert ctypes.sizeof(pa) == ctypes.sizeof(pb) == 88
            assert bytes(pa) == bytes(pb)


@pytest.mark.parametrize("path", _scene_files(), ids=lambda p: os.path.basename(os.path.dirname(os.path.dirname(p)))
                         + "/" + os.path.basename(p))
def test_pack_matches_product_host(built, path):
    from pathtracer_gb300 import Scene, cie_analytic

    with open(path) as f:
        text = f.read()
    _check_same(text, Scene.load(path), cie_analytic())


def test_pack_matches_on_generated_jobs(built):
    from pathtracer_gb300 import Scene, cie_analytic, native

    cie = cie_analytic()
    for kind in (native.PT_GEN_SPHERES, native.PT_GEN_SDF, native.PT_GEN_SDF_VARIED, native.PT_GEN_SPHERES_FULL):
        for seed in range(6):
            text = Scene.generate(kind, seed)[0].to_json()  # the JSON writer rounds to 1e-5, as the reference's
            _check_same(text, Scene.parse(text), cie)


def test_cie_table_matches(built):
    from oracle import pack
    from pathtracer_gb300 import cie_analytic

    assert pack.cie_analytic().tobytes() == cie_analytic().tobytes()


def test_plugins_match(built):
    """The shipped snippets (by fingerprint), builtin keys with and without
    material constants, and other text (a run-time compiled slot)."""
    from oracle import pack
    from pathtracer_gb300 import Scene, native

    texts = []
    for path in _scene_files():
        texts += Scene.load(path).sdf_sources()
    texts += ["builtin:menger", "builtin:blob:1,2,3", "builtin:mandelbulb_const:7", "builtin:terrain:2.5",
              "float sdf(in vec3 p) { return length(p) - 1.0; }\nfloat sdfmaterial(in vec3 p) { return 1.0; }"]
    if reference_available():
        for f in sorted(glob.glob(os.path.join(REFERENCE, "sdfs", "*.glsl"))):
            with open(f) as fh:
                texts.append(fh.read())
    kinds = set()
    for t in texts:
        mine = pack.plugin_for(t)
        p = native.PtSdfPlugin()
        rc = native.cuda().pt_parse_sdf_source(t.encode(), ctypes.byref(p))
        if rc == native.PT_OK:
            assert (mine.kind, mine.material_mode, list(mine.material)) == (p.kind, p.material_mode, list(p.material))
            assert pack.fingerprint(t) == native.cuda().pt_sdf_source_fingerprint(t.encode()) or t.startswith("builtin:")
        else:
            assert mine.kind == pack.SDF_CUSTOM
        kinds.add(mine.kind)
    assert {pack.SDF_MENGER, pack.SDF_BLOB, pack.SDF_CUSTOM} <= kinds


def test_pack_rejects_overflow():
    from oracle import pack

    root = {"camera": {"numShots": 1, "position": [[0, 0, 0]], "angle": [[0, 0]], "ISO": 100, "size": 0.036,
                       "apertureSize": 0.01, "apertureDistance": 0.1, "lensRadius": 0.1, "lensFocalLength": 1,
                       "lensThickness": 0.01, "lensDistance": 0.1},
            "sphere": [{"position": [0, 0, 0], "radius": 1, "materialID": 1, "lightID": 0}] * 200}
    with pytest.raises(ValueError):
        pack.RefScene(root).pack_ubo(None)
    root["sphere"] = root["sphere"][:3]
    ubo = pack.RefScene(root).pack_ubo(None)
    assert ubo.dtype == np.float32 and ubo.size == pack.UBO_FLOATS and ubo[0] == 3.0


def test_full_form_scenes_carry_their_extensions(built):
    """The full-form scene files set exactly the extensions their
    configurations name, and a reference-method scene sets none."""
    import os

    from oracle import pack

    x = pack.load_scene(os.path.join(SCENES, "cornell_box_full.json")).pack_ext()
    assert x.flags == pack.EXT_WAVELENGTHS | pack.EXT_ANALYTIC_CMF | pack.EXT_MATERIALS
    assert (x.lambda_min, x.lambda_max) == (380.0, 780.0)
    kinds = [x.mat[i].type for i in range(x.nmat)]
    assert kinds[-2:] == [pack.BSDF_FLAT, pack.BSDF_CAUCHY] and set(kinds[:-2]) == {pack.BSDF_REFERENCE}
    x = pack.load_scene(os.path.join(SCENES, "mandelbulb12_plane_full.json")).pack_ext()
    assert x.flags == (pack.EXT_SKY | pack.EXT_WAVELENGTHS | pack.EXT_ANALYTIC_CMF | pack.EXT_MARCH |
                       pack.EXT_MATERIALS)
    assert (x.march_max_steps, np.float32(x.march_epsilon), x.march_max_distance) == (256, np.float32(1e-4), 50.0)
    assert (x.sky_temperature, x.sky_luminosity) == (5800.0, 1.0)
    x = pack.load_scene(os.path.join(SCENES, "menger_terrain_full.json")).pack_ext()
    assert x.mat[x.nmat - 1].type == pack.BSDF_SELLMEIER
    assert [round(v, 4) for v in x.mat[x.nmat - 1].p] == [1.04, 0.23, 1.01, 0.006, 0.02, 103.6]
    assert pack.load_scene(os.path.join(SCENES, "cornell_box.json")).pack_ext().flags == 0


def test_extension_json_round_trip(built):
    """pt_scene_to_json writes the extension keys back; the written scene packs
    to the same extension block."""
    import os

    from pathtracer_gb300 import Scene, native

    for name in ("cornell_box_full", "mandelbulb12_plane_full", "menger_terrain_full"):
        a = Scene.load(os.path.join(SCENES, name + ".json"))
        b = Scene.parse(a.to_json())
        assert bytes(a.pack_ext()) == bytes(b.pack_ext()), name
    for seed in range(4):
        a, _ = Scene.generate(native.PT_GEN_SPHERES_FULL, seed)
        r, _ = Scene.generate(native.PT_GEN_SPHERES, seed)
        assert a.pack_ubo(None).tobytes() == r.pack_ubo(None).tobytes()  # same scene, same random stream
        x = a.pack_ext()
        assert x.flags == native.PT_EXT_MATERIALS
        kinds = {x.mat[i].type for i in range(x.nmat)}
        assert kinds <= {native.PT_BSDF_REFERENCE, native.PT_BSDF_MIRROR, native.PT_BSDF_CAUCHY}
