"""Wavefront knobs and the autotuner (pt_*_wavefront_tuning,
pt_autotune_wavefront): every setting renders the same bits, the autotuner
leaves the accumulator as it found it and installs a valid setting."""
import os

import numpy as np
import pytest

from conftest import SCENES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from pathtracer_gb300 import Context, PathTracerError, Scene, cie_analytic, native

    return Context, PathTracerError, Scene, cie_analytic(), native


SETTINGS = [
    {},
    {"refill_min": 8, "drain_lanes": 0, "blocks_per_sm": 2, "march_inner": 1},
    {"pool_slots": 4096, "march_budget": 3, "refill_min": 32, "drain_lanes": 32, "blocks_per_sm": 1,
     "march_inner": 16},
    {"pool_slots": 1 << 16, "march_budget": 512, "refill_min": 2, "drain_lanes": 24, "blocks_per_sm": 8,
     "march_inner": 3},
]


def test_knobs_do_not_change_results(env):
    Context, _, Scene, cie, native = env
    scene = Scene.load(os.path.join(SCENES, "mandelbulb_plane.json"))
    W, H, spf = 96, 64, 6
    push = scene.push_constants(W, H, spf, spf, spf, 6)
    images = []
    for knobs in SETTINGS:
        with Context(0) as ctx:
            ctx.set_engine(native.PT_ENGINE_WAVEFRONT)
            if knobs:
                ctx.set_tuning(**knobs)
            ctx.bind(scene, cie)
            ctx.resize_accum(W, H)
            ctx.dispatch(push)
            ctx.wait()
            images.append(ctx.read_accum())
    for img in images[1:]:
        assert np.array_equal(img.view(np.uint32), images[0].view(np.uint32))


def test_autotune_keeps_the_accumulator_and_installs_a_setting(env):
    Context, PathTracerError, Scene, cie, native = env
    scene = Scene.load(os.path.join(SCENES, "menger_terrain.json"))
    W, H = 128, 96
    with Context(0) as ctx:
        ctx.bind(scene, cie)
        ctx.resize_accum(W, H)
        before = np.random.default_rng(3).random((H, W, 4), dtype=np.float32)
        ctx.write_accum(before)
        best, secs = ctx.autotune(scene.push_constants(W, H, 4, 4, 4, 12), rounds=1)
        assert np.array_equal(ctx.read_accum(), before)
        assert ctx.tuning() == best and secs > 0.0
        assert 1024 <= best["pool_slots"] and 1 <= best["refill_min"] <= 32 and 1 <= best["blocks_per_sm"] <= 8
        assert 1 <= best["march_inner"] <= 16
        for bad in ({"refill_min": 0}, {"march_inner": 0}, {"march_inner": 17}):
            with pytest.raises(PathTracerError) as e:
                ctx.set_tuning(**bad)
            assert e.value.code == native.PT_ERR_INVALID
        assert ctx.tuning() == best


def test_knobs_on_the_compiled_march_kernel(env):
    """The bench's default scene (SDF text compiled at run time into the march
    kernel): knob settings give the same bits there too."""
    Context, _, Scene, cie, native = env
    scene = Scene.load(os.path.join(SCENES, "mandelbulb12_plane.json"))
    W, H, spf = 128, 96, 4
    push = scene.push_constants(W, H, spf, spf, spf, 6)
    images = []
    for knobs in SETTINGS[:3]:
        with Context(0) as ctx:
            ctx.set_engine(native.PT_ENGINE_WAVEFRONT)
            if knobs:
                ctx.set_tuning(**knobs)
            ctx.bind(scene, cie)
            ctx.resize_accum(W, H)
            ctx.dispatch(push)
            ctx.wait()
            images.append(ctx.read_accum())
    for img in images[1:]:
        assert np.array_equal(img.view(np.uint32), images[0].view(np.uint32))
    assert images[0][..., :3].max() > 0
