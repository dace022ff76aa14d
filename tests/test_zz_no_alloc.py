"""pt_dispatch_noalloc: a dispatch that allocates no device memory.

It serves callers that cannot call cudaMalloc while they render — a plug-in
whose host application owns the GPU memory budget, a real-time loop that
cannot pay for an allocator — by keeping its working memory in a fixed array
inside the library.  Its output must be that of the regular entry point
(pt_dispatch with the wavefront engine) on two calls in a row: the second
call starts from the first call's accumulator and reuses the shared array,
so leftovers from the first call would show.  The device's free memory must
not change across a call after the first (the warm-up, which may commit the
array).  Called through the C ABI with a caller-owned device accumulator.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import SCENES

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4  # the parity tests' tolerance (the results are identical in practice)


def _plugins(scene, native):
    out = []
    for src in scene.sdf_sources():
        p = native.PtSdfPlugin()
        assert native.cuda().pt_parse_sdf_source(src.encode(), ctypes.byref(p)) == native.PT_OK
        out.append(p)
    return out


def test_noalloc_matches_dispatch_on_two_calls(built):
    import torch

    from pathtracer_gb300 import Context, Scene, cie_analytic, native

    assert torch.cuda.is_available(), "needs a GPU"
    scene = Scene.load(os.path.join(SCENES, "mandelbulb_plane.json"))
    cie = cie_analytic()
    ubo = scene.pack_ubo(cie)
    plugins = _plugins(scene, native)
    W, H, spf, depth = 96, 64, 8, 6
    pushes = [scene.push_constants(W, H, spf * (i + 1), spf * (i + 1), spf, depth) for i in range(2)]

    # The regular entry point: a context that allocates its own memory.
    want = []
    with Context(0) as ctx:
        ctx.set_engine(native.PT_ENGINE_WAVEFRONT)
        ctx.bind(scene, cie)
        ctx.resize_accum(W, H)
        for push in pushes:
            ctx.dispatch(push)
            ctx.wait()
            want.append(ctx.read_accum().copy())

    # The allocation-free entry point, twice in a row on a caller-owned accumulator.
    lib = native.cuda()
    arr = (native.PtSdfPlugin * max(1, len(plugins)))(*plugins)
    d_accum = torch.zeros(H * W * 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for i, (push, w) in enumerate(zip(pushes, want)):
        free_before = torch.cuda.mem_get_info()[0]
        rc = lib.pt_dispatch_noalloc(ubo.ctypes.data, arr, len(plugins), ctypes.byref(push), d_accum.data_ptr(), None)
        assert rc == native.PT_OK, rc
        free_after = torch.cuda.mem_get_info()[0]
        if i > 0:  # after the warm-up call nothing is allocated on the device
            assert free_after == free_before, (free_before, free_after)
        got = d_accum.cpu().numpy().reshape(H, W, 4)
        rel = np.abs(got - w) / np.maximum(np.maximum(np.abs(got), np.abs(w)), 1e-6)
        assert float(rel.max()) <= REL_TOL

    # A request larger than the fixed array is refused with its own status.
    big = scene.push_constants(1024, 1024, 2, 2, 2, depth)  # 2,097,152 samples > PT_NOALLOC_MAX_SAMPLES
    rc = lib.pt_dispatch_noalloc(ubo.ctypes.data, arr, len(plugins), ctypes.byref(big), d_accum.data_ptr(), None)
    assert rc == native.PT_ERR_TOO_LARGE


def test_noalloc_path_length_zero_matches_dispatch(built):
    """pathLength 0 traces no bounce: the call takes its megakernel branch."""
    import torch

    from pathtracer_gb300 import Context, Scene, cie_analytic, native

    assert torch.cuda.is_available(), "needs a GPU"
    scene = Scene.load(os.path.join(SCENES, "feature_mix.json"))
    cie = cie_analytic()
    ubo = scene.pack_ubo(cie)
    plugins = _plugins(scene, native)
    W, H, spf = 40, 24, 3
    push = scene.push_constants(W, H, spf, spf, spf, 0)
    with Context(0) as ctx:
        ctx.set_engine(native.PT_ENGINE_WAVEFRONT)
        ctx.bind(scene, cie)
        ctx.resize_accum(W, H)
        ctx.dispatch(push)
        ctx.wait()
        want = ctx.read_accum().copy()
    lib = native.cuda()
    arr = (native.PtSdfPlugin * max(1, len(plugins)))(*plugins)
    d_accum = torch.zeros(H * W * 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.pt_dispatch_noalloc(ubo.ctypes.data, arr, len(plugins), ctypes.byref(push), d_accum.data_ptr(), None)
    assert rc == native.PT_OK, rc
    got = d_accum.cpu().numpy().reshape(H, W, 4)
    rel = np.abs(got - want) / np.maximum(np.maximum(np.abs(got), np.abs(want)), 1e-6)
    assert float(rel.max()) <= REL_TOL
