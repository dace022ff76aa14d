"""A wavefront dispatch split between engines (pt_set_wavefront_engines).

With n engines, a dispatch of at least 2n pools' worth of samples is
rendered by n engines on n streams, each taking an equal share of the
samples in sample order; every sample's colour lands in the dispatch's
colour buffer and the resolve sums each pixel's samples in sample order.
So the accumulator must be the one-engine accumulator bit for bit, and the
megakernel's.  The tests use a 1024-slot pool so that small dispatches are
split (and recycle every slot many times), odd sample totals (uneven
shares), progressive passes, the run-time compiled march kernel and the
checked kernel build; one test runs the bench's full-size dispatch.  A
batch splits its large staged passes the same way
(pt_batch_set_wavefront_engines): float and FP64 targets must be the
one-engine targets bit for bit, with passes of several jobs in flight
together or one job's passes after another.
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
    """Defaults, range, and lowering the count between dispatches (the
    engines past it are freed; the next dispatches render the same bits)."""
    scene = rt["Scene"].load(os.path.join(SCENES, "mandelbulb_plane.json"))
    W, H, spf, depth = 64, 48, 8, 6
    want, _ = _render(rt, scene, W, H, spf, depth, 1, engines=1, passes=3)
    with rt["Context"](0) as ctx:
        assert ctx.wavefront_engines() == 2
        for bad in (0, 5, -1):
            with pytest.raises(rt["Error"]):
                ctx.set_wavefront_engines(bad)
        ctx.set_wavefront_pool(1024)
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        for k, n in ((1, 4), (2, 1), (3, 3)):
            ctx.set_wavefront_engines(n)
            assert ctx.wavefront_engines() == n
            ctx.dispatch(scene.push_constants(W, H, k * spf, k * spf, spf, depth))
        ctx.wait()
        got = ctx.read_accum()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("engines", [2, 3, 4])
def test_split_engines_full_size(rt, engines):
    """The bench's dispatch: 1024x1024, 64 spp, depth 6, default pool (2^22
    slots per engine, 16 pools of samples)."""
    scene = rt["Scene"].load(os.path.join(SCENES, "mandelbulb12_plane.json"))
    one, _ = _render(rt, scene, 1024, 1024, 64, 6, 1, engines=1, pool=0, passes=1)
    got, l = _render(rt, scene, 1024, 1024, 64, 6, 1, engines=engines, pool=0, passes=1)
    assert np.array_equal(got.view(np.uint32), one.view(np.uint32))
    assert l[0] > 4 * 100


def _batch(rt, jobs, engines, kind=0, checks=False, interleave=True):
    """jobs: (scene, W, H, spf, depth, passes) on the staged route of a batch
    with 1024-slot pools; passes of all jobs in flight together."""
    from pathtracer_gb300 import Batch

    native = rt["native"]
    with Batch(0, pool_slots=1024, max_passes=64) as b:
        b.set_route(native.PT_BATCH_ROUTE_STAGED)
        b.set_wavefront_engines(engines)
        b.set_device_checks(checks)
        ids = []
        for scene, W, H, spf, depth, passes in jobs:
            sid = b.add_scene_sources(scene.pack_ubo(rt["cie"]), scene.sdf_sources())
            ids.append((sid, b.add_target(W, H, kind)))
        npass = max(j[5] for j in jobs)
        for k in range(1, npass + 1):
            for (sid, tid), (scene, W, H, spf, depth, passes) in zip(ids, jobs):
                if k <= passes:
                    b.add_pass(sid, tid, scene.push_constants(W, H, k * spf, k * spf, spf, depth))
            if not interleave:
                b.run()
        b.run()
        st = b.stats()
        assert st["samples_done"] == st["samples_added"]
        return [b.read_target(tid) for _, tid in ids]


def _batch_jobs(rt):
    S = rt["Scene"]
    # the first two jobs' passes are split (>= 4096 samples), the third's not
    return [(S.load(os.path.join(SCENES, "mandelbulb12_plane.json")), 48, 40, 8, 6, 2),
            (S.load(os.path.join(SCENES, "menger_terrain.json")), 51, 41, 3, 12, 3),
            (S.load(os.path.join(SCENES, "cornell_box.json")), 30, 20, 4, 8, 2)]


@pytest.mark.parametrize("interleave", [True, False])
def test_batch_split_passes_equal_one_engine(rt, interleave):
    jobs = _batch_jobs(rt)
    one = _batch(rt, jobs, 1, interleave=interleave)
    two = _batch(rt, jobs, 2, interleave=interleave)
    for a, b in zip(one, two):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    # and each equals its passes dispatched alone on one engine
    for got, (scene, W, H, spf, depth, passes) in zip(two, jobs):
        want, _ = _render(rt, scene, W, H, spf, depth, 1, engines=1, passes=passes)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_batch_split_passes_fp64_target_and_checks(rt):
    jobs = _batch_jobs(rt)[:2]
    native = rt["native"]
    one = _batch(rt, jobs, 1, kind=native.PT_TARGET_FP64)
    two = _batch(rt, jobs, 2, kind=native.PT_TARGET_FP64, checks=True)
    for a, b in zip(one, two):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_batch_engines_knob(rt):
    from pathtracer_gb300 import Batch

    with Batch(0, pool_slots=1024, max_passes=4) as b:
        for bad in (0, 3):
            with pytest.raises(rt["Error"]):
                b.set_wavefront_engines(bad)
        b.set_wavefront_engines(1)


def test_resize_to_the_same_size_zeroes_in_place(rt):
    """pt_resize_accum at the current size keeps the buffer and zeroes it in
    stream order, after the dispatch queued before it; a render after it
    equals a fresh context's render."""
    scene = rt["Scene"].load(os.path.join(SCENES, "cornell_box.json"))
    W, H, spf, depth = 64, 48, 8, 8
    want, _ = _render(rt, scene, W, H, spf, depth, 1, passes=1)
    with rt["Context"](0) as ctx:
        ctx.set_wavefront_pool(1024)
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        ptr = ctx.accum_device_ptr()
        ctx.dispatch(scene.push_constants(W, H, 7 * spf, 3 * spf, spf, depth))
        ctx.resize_accum(W, H)
        assert ctx.accum_device_ptr() == ptr
        assert not ctx.read_accum().any()
        ctx.dispatch(scene.push_constants(W, H, spf, spf, spf, depth))
        ctx.wait()
        got = ctx.read_accum()
        ctx.resize_accum(W + 1, H)
        assert not ctx.read_accum().any()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
