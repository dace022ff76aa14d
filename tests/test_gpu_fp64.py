"""The FP64 reference renderer (pt_render_fp64) on the GPU.

It traces the dispatch's paths with the same method in double precision,
drawing the same random stream as the FP32 kernels.  Checked here:
- per path, against the FP32 megakernel on the same push constants: almost
  every path takes the identical branch sequence (the two precisions only
  part where a comparison sits within FP32 rounding of its threshold), and
  the colours of identical paths agree to FP32 accuracy — far closer than the
  paths' noise, so the FP64 image measures the FP32 arithmetic's error;
- the accumulated sums: exposed colour sums and sample counts over two
  calls, their mean equal to the FP32 accumulator's up to that error;
- what it refuses: scenes whose SDF text is compiled at run time.
Scenes: the full-form Cornell box (Cauchy dielectric, flat spectra, analytic
CMF), the shipped-snippet mandelbulb over a plane, and feature_mix (every
analytic primitive and plug-in).
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
    from pathtracer_gb300 import Context, Scene, cie_analytic

    return {"Context": Context, "Scene": Scene, "cie": cie_analytic()}


def _trace_buffers(n, depth):
    import torch

    ev = torch.zeros(n * depth, dtype=torch.int32, device="cuda")
    nev = torch.zeros(n, dtype=torch.int32, device="cuda")
    col = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    return ev, nev, col


def _host(tr, n, depth):
    ev, nev, col = tr
    return ev.cpu().numpy().view(np.uint32).reshape(n, depth), nev.cpu().numpy().view(np.uint32), \
        col.cpu().numpy().reshape(n, 3)


@pytest.mark.parametrize("name,W,H,spf,depth", [("cornell_box", 64, 64, 8, 8), ("cornell_box_full", 64, 64, 8, 8),
                                                ("mandelbulb_plane", 64, 48, 8, 6), ("feature_mix", 64, 48, 8, 6)])
def test_fp64_paths_follow_the_fp32_paths(rt, name, W, H, spf, depth):
    import torch

    from pathtracer_gb300 import native

    scene = rt["Scene"].load(os.path.join(SCENES, name + ".json"))
    push = scene.push_constants(W, H, spf, spf, spf, depth)
    n = W * H * spf
    with rt["Context"](0) as ctx:
        ctx.set_engine(0)
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        t32 = _trace_buffers(n, depth)
        ctx.set_trace(t32[0].data_ptr(), t32[1].data_ptr(), t32[2].data_ptr(), depth)
        ctx.dispatch(push)
        ctx.wait()
        acc32 = ctx.read_accum()
        t64 = _trace_buffers(n, depth)
        ctx.set_trace(t64[0].data_ptr(), t64[1].data_ptr(), t64[2].data_ptr(), depth)
        sums = torch.zeros(W * H * 4, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        ctx.render_fp64(push, sums.data_ptr())
        ctx.wait()
        ctx.set_trace(0, 0, 0, 0)
        s64 = sums.cpu().numpy().reshape(H, W, 4)
    ev32, nev32, col32 = _host(t32, n, depth)
    ev64, nev64, col64 = _host(t64, n, depth)
    cap = np.minimum(nev32, depth)
    mask = np.arange(depth)[None, :] < cap[:, None]
    same = np.all(np.where(mask, ev32 == ev64, True), axis=1) & (nev32 == nev64)
    frac = float(same.mean())
    a, b = col32[same], col64[same]
    floor = max(1e-6, float(np.abs(b).max()) * 1e-6)
    rel = (np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)).max(axis=1)
    # where the two precisions part: the first differing bounce and the event
    # fields that differ there (hit object, light pick, shadow outcome, RR)
    diff = ~same
    first = np.argmax(np.where(mask, ev32 != ev64, False), axis=1)
    x = (ev32[np.arange(n), first] ^ ev64[np.arange(n), first])[diff]
    fields = {"hit": int(np.count_nonzero(x & native.PT_EV_HIT_MASK)),
              "light_pick": int(np.count_nonzero(x & (0x7F << native.PT_EV_LIGHT_SHIFT))),
              "shadow": int(np.count_nonzero(x & (3 << native.PT_EV_SHADOW_SHIFT))),
              "rr": int(np.count_nonzero(x & native.PT_EV_RR_KILL)),
              "specular": int(np.count_nonzero(x & (native.PT_EV_SPECULAR | native.PT_EV_REFRACT))),
              "length_only": int(np.count_nonzero(x == 0))}
    print(name, {"paths": n, "identical_branches": frac, "median_rel": float(np.median(rel)),
                 "p99_rel": float(np.percentile(rel, 99)), "max_rel": float(rel.max()),
                 "first_differing_bounce": np.bincount(first[diff], minlength=depth).tolist(), "fields": fields})
    # FP32 rounding sends some paths another way at a comparison near its
    # threshold (a grazing hit, an SDF march converging one step apart, a light
    # sample at a shadow edge); from there the two paths are independent.
    assert frac >= 0.9
    # identical paths: FP32 accuracy, except the cone pdf's cancellation near
    # small lights (up to ~1e-2 relative, the error the FP64 reference exposes)
    assert np.median(rel) < 1e-5 and np.percentile(rel, 99) < 2e-2
    assert np.all(s64[..., 3] == spf)
    mean64 = s64[..., :3] / s64[..., 3:4]
    # the image's total: the parted paths' noise averages out over the frame
    bias = np.abs(mean64.sum(axis=(0, 1)) - acc32[..., :3].sum(axis=(0, 1))) / np.abs(mean64.sum(axis=(0, 1)))
    assert np.all(bias < 0.02), bias


def test_fp64_sums_accumulate_and_jit_text_is_refused(rt):
    import torch

    from pathtracer_gb300 import PathTracerError, native

    scene = rt["Scene"].load(os.path.join(SCENES, "cornell_box.json"))
    W, H, spf, depth = 32, 24, 4, 8
    with rt["Context"](0) as ctx:
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        sums = torch.zeros(W * H * 4, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for k in (1, 2):
            ctx.render_fp64(scene.push_constants(W, H, k * spf, k * spf, spf, depth), sums.data_ptr())
        ctx.wait()
        s = sums.cpu().numpy().reshape(H, W, 4)
        assert np.all(s[..., 3] == 2 * spf) and np.all(np.isfinite(s)) and s[..., :3].sum() > 0
    jit = rt["Scene"].load(os.path.join(SCENES, "mandelbulb12_plane.json"))
    with rt["Context"](0) as ctx:
        ctx.bind(jit, rt["cie"])
        with pytest.raises(PathTracerError) as e:
            ctx.render_fp64(jit.push_constants(W, H, spf, spf, spf, 6), sums.data_ptr())
        assert e.value.code == native.PT_ERR_UNSUPPORTED
