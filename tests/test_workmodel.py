"""The FP32 work model: its fixtures are the oracle's own counters (re-run
here on the fixture's rows) and give positive work in the stages that
perform it."""
import json
import os

from conftest import GOLDEN, SCENES


def test_mandelbulb_fixture_matches_the_oracle(built):
    from oracle import compare, oracle
    from pathtracer_gb300 import Scene, cie_analytic

    with open(os.path.join(GOLDEN, "work_mandelbulb_plane_1024x1024_64spp_depth6.json")) as f:
        fx = json.load(f)
    scene = Scene.load(os.path.join(SCENES, "mandelbulb_plane.json"))
    ubo = scene.pack_ubo(cie_analytic())
    push = scene.push_constants(1024, 1024, 64, 64, 64, 6)
    rows = fx["sample"]["rows"]
    tot = None
    for r in range(rows):
        y = (2 * r + 1) * 1024 // (2 * rows)
        c = oracle.count_work(ubo, push, compare.plugins_for(scene), rect=(0, y, 1024, y + 1))
        tot = c if tot is None else {k: tot[k] + c[k] for k in c}
    assert tot["samples"] == fx["sample"]["samples"]
    for k, v in tot.items():
        assert abs(v / tot["samples"] - fx["per_sample"][k]) < 1e-9, k


def test_work_per_stage():
    from pathtracer_gb300 import workmodel

    m = workmodel.fp32_ops_per_sample(workmodel.load("mandelbulb_plane_1024x1024_64spp_depth6")["per_sample"])
    assert m["march"] > 0.9 * m["total"] > 0
    b = workmodel.fp32_ops_per_sample(workmodel.load("batch64_spheres")["per_sample"])
    assert b["march"] == 0 and b["isect"] > b["shade"] > 0
    counts = workmodel.load("mandelbulb_plane_1024x1024_64spp_depth6")["per_sample"]
    assert 1.0 <= counts["mandelbulb_iters"] / counts["sdf_mandelbulb"] <= 4.0


def test_bulb12_fixture_matches_the_oracle(built):
    """The default bench workload's counts, including the iterations inside
    the C restatement of its run-time compiled SDF text."""
    from oracle import compare, oracle
    from pathtracer_gb300 import Scene, cie_analytic, workmodel

    name = "mandelbulb12_plane_1024x1024_64spp_depth6"
    fx = workmodel.load(name)
    scene = Scene.load(os.path.join(SCENES, "mandelbulb12_plane.json"))
    ubo = scene.pack_ubo(cie_analytic())
    push = scene.push_constants(1024, 1024, 64, 64, 64, 6)
    rows = fx["sample"]["rows"]
    y = (2 * 0 + 1) * 1024 // (2 * rows)
    c = oracle.count_work(ubo, push, compare.plugins_for(scene), rect=(0, y, 1024, y + 1))
    assert c["sdf_custom"] > 0 and c["bulb8_iters"] > 0
    per = fx["per_sample"]
    assert per["sdf_mandelbulb"] == 0 and 2.0 <= per["bulb8_iters"] / per["sdf_custom"] <= 12.0
    m = workmodel.fp32_ops_per_sample(per)
    assert m["march"] > 0.9 * m["total"] > 0
