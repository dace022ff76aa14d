"""The iteration limits that stop device work which does not finish.

No kernel of this library waits on another block or another launch, so
nothing can spin forever; what can run long is the host loop that relaunches
the wavefront stages until every path has finished.  Both such loops have a
limit, after which the call returns PT_ERR_KERNEL with no result written and
the context or batch left usable:
- the dispatch drain of the wavefront engine (bound computed from the
  dispatch; pt_set_drain_limit lowers it for this test);
- pt_batch_run(max_iterations).
Each test makes the limit run out on a pass far larger than the limit
allows, checks the status, then finishes the work and checks the result
against a dispatch that never hit a limit, bit for bit.
"""
import os

import numpy as np
import pytest

from conftest import SCENES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("no CUDA device: -m gpu tests need a GPU")
    from pathtracer_gb300 import native, renderer

    return native, renderer, renderer.cie_analytic()


def _plain(renderer, cie, scene, W, H, spf, depth, engine):
    with renderer.Context(0) as ctx:
        ctx.set_engine(engine)
        ctx.bind(scene, cie)
        ctx.resize_accum(W, H)
        ctx.dispatch(scene.push_constants(W, H, spf, spf, spf, depth))
        ctx.wait()
        return ctx.read_accum()


@pytest.mark.parametrize("engines", [1, 2])
def test_dispatch_drain_limit(env, engines):
    """With two engines the dispatch is split (2^17-slot pools, 8 pools of
    samples): the limit stops both, and the next dispatch resets both."""
    native, renderer, cie = env
    scene = renderer.Scene.load(os.path.join(SCENES, "mandelbulb_plane.json"))
    W, H, spf, depth = 256, 256, 16, 6
    push = scene.push_constants(W, H, spf, spf, spf, depth)
    want = _plain(renderer, cie, scene, W, H, spf, depth, native.PT_ENGINE_WAVEFRONT)
    with renderer.Context(0) as ctx:
        ctx.set_engine(native.PT_ENGINE_WAVEFRONT)
        ctx.set_wavefront_engines(engines)
        if engines > 1:
            ctx.set_wavefront_pool(1 << 17)
        ctx.bind(scene, cie)
        ctx.resize_accum(W, H)
        ctx.set_drain_limit(2)  # 1 M samples of depth-6 paths need far more iterations
        with pytest.raises(renderer.PathTracerError) as e:
            ctx.dispatch(push)
        assert e.value.code == native.PT_ERR_KERNEL
        ctx.wait()
        assert not ctx.read_accum().any()  # nothing was resolved into the accumulator
        ctx.set_drain_limit(0)
        ctx.dispatch(push)
        ctx.wait()
        got = ctx.read_accum()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("route,kind,W,H,spf", [("staged", "sdf", 512, 512, 16), ("persistent", "spheres", 1024, 1024, 128)])
def test_batch_run_limit(env, route, kind, W, H, spf):
    native, renderer, cie = env
    if kind == "sdf":
        scene = renderer.Scene.load(os.path.join(SCENES, "mandelbulb_plane.json"))
        depth = 6
    else:
        scene, spec = renderer.Scene.generate(native.PT_GEN_SPHERES, 4)
        depth = spec.pathLength
    r = {"staged": native.PT_BATCH_ROUTE_STAGED, "persistent": native.PT_BATCH_ROUTE_PERSISTENT}[route]
    with renderer.Batch(0, pool_slots=1 << 19, max_passes=64) as b:
        b.set_route(r)
        sid = b.add_scene(scene.pack_ubo(cie), scene.sdf_plugins())
        tid = b.add_target(W, H)
        b.add_pass(sid, tid, scene.push_constants(W, H, spf, spf, spf, depth))
        with pytest.raises(renderer.PathTracerError) as e:
            b.run(max_iterations=1)
        assert e.value.code == native.PT_ERR_KERNEL
        assert b.pending() == 1
        b.run()  # the same batch finishes the pass
        assert b.pending() == 0 and b.target_samples(tid) == spf
        got = b.read_target(tid)
    want = _plain(renderer, cie, scene, W, H, spf, depth, native.PT_ENGINE_MEGAKERNEL)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
