"""A wavefront dispatch split between engines (pt_set_wavefront_engines).

With n engines, a dispatch of at least 2n pools' worth of samples is
rendered by n engines on n streams, each taking an equal share of the
samples in sample order; every sample's colour lands in the dispatch's
colour buffer and the resolve sums each pixel's samples in sample order.
So the accumulator must be the one-engine accumulator bit for bit, and the
megakernel's.  The tests use a 1024-slot pool so that small dispatches are
split (and recycle every slot many times), odd sample totals (uneven
shares), progressive passes, the run-time compiled march kernel and the
checked kernel build; one test runs the bench's full-size dispatch.
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
    from pathtracer_gb300 import Context, PathTracerError, Scene, cie_analytic, native

    return {"Context": Context, "Scene": Scene, "cie": cie_analytic(), "native": native, "Error": PathTracerError}


def _render(rt, scene, W, H, spf, depth, engine, engines=1, pool=1024, checks=False, passes=2):
    with rt["Context"](0) as ctx:
        ctx.set_engine(engine)
        ctx.set_wavefront_engines(engines)
        if pool:
            ctx.set_wavefront_pool(pool)
        ctx.set_device_checks(checks)
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        launches = []
        for k in range(1, passes + 1):
            ctx.dispatch(scene.push_constants(W, H, k * spf, k * spf, spf, depth))
            launches.append(ctx.last_kernel_launches())
        ctx.wait()
        return ctx.read_accum(), launches


@pytest.mark.parametrize("name,W,H,spf,depth", [("cornell_box", 64, 64, 4, 8),
                                                ("mandelbulb_plane", 64, 48, 8, 6),
                                                ("mandelbulb12_plane", 48, 40, 8, 6),
                                                ("menger_terrain", 64, 40, 4, 12),
                                                ("feature_mix", 51, 41, 5, 6)])
def test_split_engines_equal_one_and_megakernel(rt, name, W, H, spf, depth):
    scene = rt["Scene"].load(os.path.join(SCENES, name + ".json"))
    assert W * H * spf >= 8 * 1024  # split between up to four engines
    one, l1 = _render(rt, scene, W, H, spf, depth, 1, engines=1)
    two, l2 = _render(rt, scene, W, H, spf, depth, 1, engines=2)
    four, l4 = _render(rt, scene, W, H, spf, depth, 1, engines=4)
    mega, lm = _render(rt, scene, W, H, spf, depth, 0)
    assert np.array_equal(two.view(np.uint32), one.view(np.uint32))
    assert np.array_equal(four.view(np.uint32), one.view(np.uint32))
    assert np.array_equal(two.view(np.uint32), mega.view(np.uint32))
    assert lm == [1, 1]
    assert l4[1] >= 25 and (l4[1] - 9) % 4 == 0, l4
    # second pass (the engines exist): one engine launches init, job_add,
    # 4 kernels per iteration and the resolve; two add the second engine's
    # init, job_add and iterations
    assert l1[1] >= 7 and (l1[1] - 3) % 4 == 0, l1
    assert l2[1] >= 13 and (l2[1] - 5) % 4 == 0, l2


def test_two_engines_checked_build(rt):
    scene = rt["Scene"].load(os.path.join(SCENES, "mandelbulb12_plane.json"))
    want, _ = _render(rt, scene, 64, 48, 8, 6, 1, engines=1)
    got, _ = _render(rt, scene, 64, 48, 8, 6, 1, engines=2, checks=True)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_small_dispatch_runs_on_one_engine(rt):
    """Below four pools of samples a dispatch is not split."""
    scene = rt["Scene"].load(os.path.join(SCENES, "cornell_box.json"))
    one, l1 = _render(rt, scene, 32, 32, 3, 8, 1, engines=1)
    two, l2 = _render(rt, scene, 32, 32, 3, 8, 1, engines=2)
    assert np.array_equal(two.view(np.uint32), one.view(np.uint32))
    assert (l2[1] - 3) % 4 == 0, l2


def test_engines_knob(rt):
    with rt["Context"](0) as ctx:
        assert ctx.wavefront_engines() == 2
        for bad in (0, 5, -1):
            with pytest.raises(rt["Error"]):
                ctx.set_wavefront_engines(bad)
        ctx.set_wavefront_engines(1)
        assert ctx.wavefront_engines() == 1


@pytest.mark.parametrize("engines", [2, 3, 4])
def test_split_engines_full_size(rt, engines):
    """The bench's dispatch: 1024x1024, 64 spp, depth 6, default pool (2^22
    slots per engine, 16 pools of samples)."""
    scene = rt["Scene"].load(os.path.join(SCENES, "mandelbulb12_plane.json"))
    one, _ = _render(rt, scene, 1024, 1024, 64, 6, 1, engines=1, pool=0, passes=1)
    got, l = _render(rt, scene, 1024, 1024, 64, 6, 1, engines=engines, pool=0, passes=1)
    assert np.array_equal(got.view(np.uint32), one.view(np.uint32))
    assert l[0] > 4 * 100
