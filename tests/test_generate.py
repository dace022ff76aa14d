"""The seeded job generator (pt_scene_generate): deterministic per seed,
pinned by tests/golden/generated_jobs.json (tests/golden/make_generated.py),
within its documented distribution, and always packable into the reference's
uniform buffer."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.fixture(scope="module")
def gen(built):
    from pathtracer_gb300 import native, renderer

    return native, renderer


def _spec(native, spec):
    return {k: getattr(spec, k) for k, _ in native.PtJobSpec._fields_ if k != "pad"}


def test_generator_matches_golden(gen):
    native, renderer = gen
    with open(os.path.join(GOLDEN, "generated_jobs.json")) as f:
        golden = json.load(f)
    for item in golden["scenes"]:
        spec = item["spec"]
        scene, got = renderer.Scene.generate(spec["kind"], spec["seed"])
        assert _spec(native, got) == spec
        assert scene.to_json() == item["json"]
    for seed, spec in enumerate(golden["sphere_specs"]):
        assert _spec(native, renderer.Scene.generate(native.PT_GEN_SPHERES, seed)[1]) == spec
    for seed, spec in enumerate(golden["sdf_specs"]):
        assert _spec(native, renderer.Scene.generate(native.PT_GEN_SDF, seed)[1]) == spec


def test_generated_scene_round_trips_through_json(gen):
    """Saving rounds to 5 decimals, as the reference's UpdateToJSON does, so a
    reloaded scene matches to that precision."""
    native, renderer = gen
    cie = renderer.cie_analytic()
    for kind, seed in ((native.PT_GEN_SPHERES, 5), (native.PT_GEN_SDF, 9)):
        scene, _ = renderer.Scene.generate(kind, seed)
        again = renderer.Scene.parse(scene.to_json())
        a, b = again.pack_ubo(cie), scene.pack_ubo(cie)
        np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-5)
        assert again.counts() == scene.counts() and again.sdf_sources() == scene.sdf_sources()


def test_sphere_job_distribution(gen):
    native, renderer = gen
    cie = renderer.cie_analytic()
    res, spps, counts = set(), [], []
    for seed in range(400):
        scene, spec = renderer.Scene.generate(native.PT_GEN_SPHERES, seed)
        assert spec.width == spec.height and spec.pathLength == 8 and spec.sdf_kind == native.PT_SDF_NONE
        res.add(spec.width)
        spps.append(spec.spp)
        counts.append(spec.objects)
        c = scene.counts()
        assert c["spheres"] == spec.objects + 1 and c["planes"] == 1 and c["lights"] == 1 and c["sdfs"] == 0
        ubo = scene.pack_ubo(cie)
        assert ubo[6] == 1.0  # one light ID
        radii = ubo[7:7 + 6 * spec.objects].reshape(-1, 6)[:, 3]
        assert (radii >= 0.03).all() and (radii <= 1.0).all()
        centres = ubo[7:7 + 6 * spec.objects].reshape(-1, 6)[:, :3]
        assert (np.abs(centres) <= 2.0).all()
    assert res == {128, 256, 512, 1024}
    assert min(spps) >= 4 and max(spps) <= 256
    # log-uniform: about half the jobs below 32 spp (the geometric midpoint)
    assert 0.4 < np.mean(np.array(spps) < 32) < 0.6
    assert min(counts) >= 4 and max(counts) <= 64 and len(set(counts)) > 40


def test_sdf_job_distribution(gen):
    native, renderer = gen
    cie = renderer.cie_analytic()
    kinds, res = set(), set()
    for seed in range(60):
        scene, spec = renderer.Scene.generate(native.PT_GEN_SDF, seed)
        kinds.add(spec.sdf_kind)
        res.add(spec.width)
        plugins = scene.sdf_plugins()
        assert len(plugins) == 1 and plugins[0].kind == spec.sdf_kind
        scene.pack_ubo(cie)
    assert kinds == {native.PT_SDF_BLOB, native.PT_SDF_MANDELBULB, native.PT_SDF_MENGER}
    assert res == {256, 512, 1024}


def test_generate_rejects_unknown_kind(gen):
    native, renderer = gen
    with pytest.raises(renderer.PathTracerError):
        renderer.Scene.generate(7, 0)


def test_varied_sdf_jobs(gen):
    """PT_GEN_SDF_VARIED: the same scene for a seed, drawn mandelbulb powers
    in [4, 10] with 4-6 iterations and Menger levels in {3, 4, 5}, as GLSL
    the translator accepts; blobs stay the shipped plug-in."""
    import re

    from pathtracer_gb300 import Scene, glsl_translate, native

    kinds = set()
    for seed in range(3000, 3060):
        a, spec = Scene.generate(native.PT_GEN_SDF_VARIED, seed)
        b, _ = Scene.generate(native.PT_GEN_SDF_VARIED, seed)
        assert a.to_json() == b.to_json()
        src = a.sdf_sources()[0]
        m = re.match(r"// Mandelbulb of power ([0-9.]+), ([0-9]+) iterations", src)
        if m:
            assert 4.0 <= float(m.group(1)) <= 10.0 and 4 <= int(m.group(2)) <= 6
            assert spec.sdf_kind == native.PT_SDF_CUSTOM
            kinds.add("mandelbulb")
        elif src.startswith("// Menger sponge"):
            assert int(re.match(r"// Menger sponge, ([0-9]+) levels", src).group(1)) in (3, 4, 5)
            kinds.add("menger")
        else:
            assert src == "builtin:blob:0,1,2" and spec.sdf_kind == native.PT_SDF_BLOB
            kinds.add("blob")
        if spec.sdf_kind == native.PT_SDF_CUSTOM:
            glsl_translate(src)
    assert kinds == {"mandelbulb", "menger", "blob"}
