"""The checked build of the wavefront kernels (pt_set_device_checks,
pt_batch_set_device_checks): the stand-in for a device memory checker on the
queue code.

With the checks on, every queue append, slot read from a queue or the free
list, pass index and sample index of the staged and persistent kernels is
checked before use; a failed check would skip its access and turn the
dispatch into PT_ERR_KERNEL.  These tests run the workloads at their own
sizes — where pool recycling, suspended marches and queue wrap-around happen
— with the checks on, and require that no check fails and that the results
are the unchecked kernels' bit for bit:
- the 12-iteration mandelbulb (run-time compiled march kernel, compiled
  again for the checked build), 1024x1024, 64 spp, depth 6;
- the shipped-snippet mandelbulb (the built-in warp-normal march kernel);
- menger + terrain at 1920x1080, 16 spp, depth 12;
- the Cornell box at 256x256, 16 spp, depth 8 (no SDF);
- sphere jobs of the 64-job batch on the persistent route and SDF jobs on
  the staged route.
No test makes a check fail: that needs an index out of range, i.e. a broken
kernel, which is not run on a GPU.
"""
import os

import numpy as np
import pytest

from conftest import SCENES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rt(built):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("no CUDA device: -m gpu tests need a GPU")
    from pathtracer_gb300 import Context, Scene, cie_analytic, native

    return {"Context": Context, "Scene": Scene, "cie": cie_analytic(), "native": native}


def _render(rt, scene, W, H, spf, depth, checks, passes=1):
    with rt["Context"](0) as ctx:
        ctx.set_engine(rt["native"].PT_ENGINE_WAVEFRONT)
        ctx.set_device_checks(checks)
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        for k in range(1, passes + 1):
            ctx.dispatch(scene.push_constants(W, H, k * spf, k * spf, spf, depth))
        ctx.wait()
        return ctx.read_accum()


@pytest.mark.parametrize("name,W,H,spf,depth,passes", [("mandelbulb12_plane", 1024, 1024, 64, 6, 1),
                                                       ("mandelbulb_plane", 512, 512, 16, 6, 2),
                                                       ("menger_terrain", 1920, 1080, 16, 12, 1),
                                                       ("cornell_box", 256, 256, 16, 8, 1)])
def test_checked_kernels_pass_and_match(rt, name, W, H, spf, depth, passes):
    scene = rt["Scene"].load(os.path.join(SCENES, name + ".json"))
    want = _render(rt, scene, W, H, spf, depth, False, passes)
    got = _render(rt, scene, W, H, spf, depth, True, passes)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("route", ["persistent", "staged"])
def test_checked_batch_passes_and_matches(rt, route):
    from pathtracer_gb300 import Batch

    native = rt["native"]
    kind = native.PT_GEN_SPHERES if route == "persistent" else native.PT_GEN_SDF
    jobs = [rt["Scene"].generate(kind, s) for s in (0, 2, 3, 8)]
    r = {"persistent": native.PT_BATCH_ROUTE_PERSISTENT, "staged": native.PT_BATCH_ROUTE_STAGED}[route]

    def run(checks):
        with Batch(0, pool_slots=1 << 19, max_passes=256) as b:
            b.set_route(r)
            b.set_device_checks(checks)
            tids = []
            for scene, spec in jobs:
                spp = spec.spp or 16  # SDF jobs are served in passes: 16 spp here
                sid = b.add_scene(scene.pack_ubo(rt["cie"]), scene.sdf_plugins())
                tid = b.add_target(spec.width, spec.height)
                b.add_pass(sid, tid, scene.push_constants(spec.width, spec.height, spp, spp, spp, spec.pathLength))
                tids.append(tid)
            b.run()
            return [b.read_target(t) for t in tids]

    want, got = run(False), run(True)
    for w, g in zip(want, got):
        assert np.array_equal(g.view(np.uint32), w.view(np.uint32))
