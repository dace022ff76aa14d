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
- scenes whose SDF text is compiled at run time (the 12-iteration
  mandelbulb, the fBm terrain), whose snippets are compiled once more with
  every GLSL float a double;
- the FP32 method's bias at high sample counts on the Cornell box and the
  12-iteration mandelbulb in their full forms: the mean of many samples
  against the FP64 mean of the same samples.
Scenes: the full-form Cornell box (Cauchy dielectric, flat spectra, analytic
CMF), the shipped-snippet mandelbulb over a plane, feature_mix (every
analytic primitive and plug-in), and the run-time compiled scenes.
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


# Fraction of paths with the FP32 kernels' branch sequence, at least: the
# escape-time fractal of 12 iterations parts more paths (its march converges
# a step earlier or later near the surface) than the analytic scenes do.
FRAC_MIN = {"mandelbulb12_plane": 0.85, "menger_terrain_full": 0.85}


@pytest.mark.parametrize("name,W,H,spf,depth", [("cornell_box", 64, 64, 8, 8), ("cornell_box_full", 64, 64, 8, 8),
                                                ("mandelbulb_plane", 64, 48, 8, 6), ("feature_mix", 64, 48, 8, 6),
                                                ("mandelbulb12_plane", 64, 48, 8, 6),
                                                ("menger_terrain_full", 48, 40, 4, 12)])
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
    assert frac >= FRAC_MIN.get(name, 0.9)
    # identical paths: FP32 accuracy, except the cone pdf's cancellation near
    # small lights (a few per cent at the 99th percentile behind the
    # mandelbulb scene's small sun: the error the FP64 reference exposes)
    assert np.median(rel) < 1e-5 and np.percentile(rel, 99) < 5e-2
    assert np.all(s64[..., 3] == spf)
    mean64 = s64[..., :3] / s64[..., 3:4]
    # the image's total: the parted paths' noise averages out over the frame
    bias = np.abs(mean64.sum(axis=(0, 1)) - acc32[..., :3].sum(axis=(0, 1))) / np.abs(mean64.sum(axis=(0, 1)))
    assert np.all(bias < 0.02), bias


def test_fp64_sums_accumulate(rt):
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
        with pytest.raises(PathTracerError) as e:
            ctx.render_fp64(scene.push_constants(W + 1, H, spf, spf, spf, 8), 0)
        assert e.value.code == native.PT_ERR_INVALID


@pytest.mark.parametrize("name,W,H,passes,spf,depth", [("cornell_box_full", 256, 256, 16, 16, 8),
                                                       ("mandelbulb12_plane_full", 256, 256, 8, 16, 6)])
def test_fp32_bias_at_high_spp(rt, name, W, H, passes, spf, depth):
    """The FP32 method's image after passes x spf samples per pixel against
    the FP64 renderer's mean of the same samples: the frame's total (the
    bias of the FP32 arithmetic, the parted paths' noise averaged over the
    frame) and the per-pixel relative RMSE (mostly the parted paths)."""
    import torch

    scene = rt["Scene"].load(os.path.join(SCENES, name + ".json"))
    with rt["Context"](0) as ctx:
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        sums = torch.zeros(W * H * 4, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for k in range(1, passes + 1):
            push = scene.push_constants(W, H, k * spf, k * spf, spf, depth)
            ctx.dispatch(push)
            ctx.render_fp64(push, sums.data_ptr())
        ctx.wait()
        acc = ctx.read_accum()[..., :3].astype(np.float64)
        s64 = sums.cpu().numpy().reshape(H, W, 4)
    assert np.all(s64[..., 3] == passes * spf)
    ref = s64[..., :3] / s64[..., 3:4]
    total = np.abs(acc.sum(axis=(0, 1)) - ref.sum(axis=(0, 1))) / np.abs(ref.sum(axis=(0, 1)))
    rmse = float(np.sqrt(((acc - ref) ** 2).sum() / (ref ** 2).sum()))
    print(f"{name} {W}x{H} {passes * spf} spp: frame total rel {total.tolist()}, per-pixel rel RMSE {rmse:.3e}")
    assert np.all(total < 5e-3), total
    assert rmse < 0.05


def _mean_f32(sums):
    """An FP64 target's read-back (pt_batch_read_target): sum * (1 / count), rounded to float."""
    inv = np.where(sums[..., 3:4] > 0, 1.0 / np.maximum(sums[..., 3:4], 1.0), 0.0)
    return (sums[..., :3] * inv).astype(np.float32)


def test_batch_fp64_pass_equals_the_context_renderer(rt):
    """pt_batch_render_fp64 on a resident scene (extensions included) adds
    the same sums as pt_render_fp64 on a context over two dispatches (the
    batch's read-back of them is the same bits); an FP32 pass into the same
    kind of target differs from it only by the FP32 arithmetic's error."""
    import torch

    from pathtracer_gb300 import Batch, PathTracerError, native

    scene = rt["Scene"].load(os.path.join(SCENES, "cornell_box_full.json"))
    W, H, spf, depth = 48, 40, 8, 8
    pushes = [scene.push_constants(W, H, k * spf, k * spf, spf, depth) for k in (1, 2)]
    with rt["Context"](0) as ctx:
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        sums = torch.zeros(W * H * 4, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for p in pushes:
            ctx.render_fp64(p, sums.data_ptr())
        ctx.wait()
        want = sums.cpu().numpy().reshape(H, W, 4)
    with Batch(0, pool_slots=1 << 14, max_passes=16) as b:
        sid = b.add_scene(scene.pack_ubo(rt["cie"]), scene.sdf_plugins())
        b.set_scene_ext(sid, scene.pack_ext())
        t64 = b.add_target(W, H, native.PT_TARGET_FP64)
        t32 = b.add_target(W, H, native.PT_TARGET_FP64)
        for p in pushes:
            b.render_fp64(sid, t64, p)
            b.add_pass(sid, t32, p)
        b.run()
        got = b.read_target(t64)
        f32 = b.read_target(t32)
        assert b.target_samples(t64) == 2 * spf
        with pytest.raises(PathTracerError) as e:
            b.render_fp64(sid, b.add_target(W, H), pushes[0])  # a float target
        assert e.value.code == native.PT_ERR_INVALID
    assert np.array_equal(got[..., :3].view(np.uint32), _mean_f32(want).view(np.uint32))
    tot64, tot32 = got[..., :3].sum(axis=(0, 1)), f32[..., :3].sum(axis=(0, 1))
    assert np.all(np.abs(tot64 - tot32) / np.abs(tot64) < 0.02), (tot64, tot32)


def test_server_references_with_fp64_paths(rt):
    """pt_server_opts.fp64_paths: references traced in double precision (for
    the scene compiled at run time too); each job reaches an RMSE against
    them close to its RMSE against the FP32-path reference (the two
    references differ by the FP32 error, far below the job's noise)."""
    from pathtracer_gb300 import Server, native

    cie = rt["cie"]
    W = H = 32
    sc, spec = rt["Scene"].generate(native.PT_GEN_SPHERES_FULL, 5)
    jit = rt["Scene"].load(os.path.join(SCENES, "mandelbulb12_plane.json"))
    rmse = {}
    for fp64 in (False, True):
        with Server(0, fp64_paths=fp64, keep_images=False, pool_slots=1 << 14, max_passes=64) as srv:
            srv.add_scene(0, sc.pack_ubo(cie), sc.sdf_plugins())
            srv.set_scene_ext(0, sc.pack_ext())
            srv.render_reference(0, sc.push_constants(W, H, 1, 1, 1, spec.pathLength), 256, 32)
            srv.add_scene_sources(1, jit.pack_ubo(cie), jit.sdf_sources())
            srv.render_reference(1, jit.push_constants(W, H, 1, 1, 1, 6), 32, 16)
            ids = [srv.submit(Server.job(0, sc.push_constants(W, H, 1, 1, 1, spec.pathLength), 32, 1e-9)),
                   srv.submit(Server.job(1, jit.push_constants(W, H, 1, 1, 1, 6), 8, 1e-9))]
            done = {r.job_id: r for r in srv.drain()}
            rmse[fp64] = [done[i].rmse for i in ids]
            assert all(done[i].status == native.PT_OK for i in ids)
    print("relative RMSE, FP32-path vs FP64-path references:", rmse)
    for a, b in zip(rmse[True], rmse[False]):
        assert 0 < a and abs(a - b) < 0.05 * b
