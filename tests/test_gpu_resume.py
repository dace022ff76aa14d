"""Checkpoint and resume of a progressive render.

The reference keeps no state between frames beyond its accumulator and the
frame / currentSamples counters (src/pathtracer.cpp:1164-1166), and every
sample's random stream is indexed by pixel and global sample index
(src/shader.comp:948-958).  So a render stopped after k passes can be
resumed elsewhere from the accumulator alone (pt_read_accum, then
pt_write_accum in a new context) with the counters continued, and must end
bit-identical to the render that never stopped: on both engines, with the
wavefront dispatch split between engines, and from a batch target.
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
    from pathtracer_gb300 import Batch, Context, Scene, cie_analytic, native

    return {"Context": Context, "Batch": Batch, "Scene": Scene, "cie": cie_analytic(), "native": native}


def _passes(rt, ctx, scene, W, H, spf, depth, ks):
    for k in ks:
        ctx.dispatch(scene.push_constants(W, H, k * spf, k * spf, spf, depth))
    ctx.wait()


def _ctx(rt, scene, W, H, engine, engines):
    ctx = rt["Context"](0)
    ctx.set_engine(engine)
    ctx.set_wavefront_engines(engines)
    ctx.set_wavefront_pool(1024)
    ctx.bind(scene, rt["cie"])
    ctx.resize_accum(W, H)
    return ctx


@pytest.mark.parametrize("engine,engines", [(0, 1), (1, 1), (1, 2)])
@pytest.mark.parametrize("name,W,H,spf,depth", [("mandelbulb12_plane", 64, 48, 8, 6), ("cornell_box", 64, 64, 4, 8)])
def test_resume_from_the_accumulator(rt, engine, engines, name, W, H, spf, depth):
    scene = rt["Scene"].load(os.path.join(SCENES, name + ".json"))
    with _ctx(rt, scene, W, H, engine, engines) as ctx:
        _passes(rt, ctx, scene, W, H, spf, depth, range(1, 5))
        want = ctx.read_accum()
    with _ctx(rt, scene, W, H, engine, engines) as ctx:
        _passes(rt, ctx, scene, W, H, spf, depth, range(1, 3))
        checkpoint = ctx.read_accum().copy()
    with _ctx(rt, scene, W, H, engine, engines) as ctx:
        ctx.write_accum(checkpoint)
        _passes(rt, ctx, scene, W, H, spf, depth, range(3, 5))
        got = ctx.read_accum()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_resume_a_batch_target_in_a_context(rt):
    """Two passes in a batch, the target read back, two more through
    pt_dispatch from that accumulator: the four-pass render's bits."""
    scene = rt["Scene"].load(os.path.join(SCENES, "menger_terrain.json"))
    W, H, spf, depth = 64, 40, 4, 12
    with _ctx(rt, scene, W, H, 1, 2) as ctx:
        _passes(rt, ctx, scene, W, H, spf, depth, range(1, 5))
        want = ctx.read_accum()
    with rt["Batch"](0, pool_slots=1024, max_passes=8) as b:
        sid = b.add_scene_sources(scene.pack_ubo(rt["cie"]), scene.sdf_sources())
        tid = b.add_target(W, H)
        for k in (1, 2):
            b.add_pass(sid, tid, scene.push_constants(W, H, k * spf, k * spf, spf, depth))
        b.run()
        checkpoint = b.read_target(tid)
    with _ctx(rt, scene, W, H, 1, 2) as ctx:
        ctx.write_accum(checkpoint)
        _passes(rt, ctx, scene, W, H, spf, depth, range(3, 5))
        got = ctx.read_accum()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
