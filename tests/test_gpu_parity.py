"""Parity of both sm_103a engines (megakernel, wavefront) with the CPU
restatement of the shader.

Every test calls the library through its C ABI (ctypes), on the same scene,
UBO and push constants the oracle gets.  Criteria (oracle/compare.py):
>= 99.9% of paths follow the identical branch sequence; matching paths agree
in per-sample XYZ within 1e-4 relative; pixels whose paths all match agree in
the accumulated XYZ within 1e-4 relative; w == 1 everywhere.
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


ENGINES = [0, 1]  # PT_ENGINE_MEGAKERNEL, PT_ENGINE_WAVEFRONT


def _setup(rt, name, W, H, engine=1):
    from oracle import compare

    scene = rt["Scene"].load(os.path.join(SCENES, name + ".json"))
    ctx = rt["Context"](0)
    ctx.set_engine(engine)
    ctx.bind(scene, rt["cie"])
    ctx.resize_accum(W, H)
    ubo = scene.pack_ubo(rt["cie"])
    return scene, ctx, ubo, compare.plugins_for(scene)


def _check(report):
    from oracle import compare

    assert compare.passes(report), report


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize(
    "name,W,H,spf,depth",
    [
        ("cornell_box", 64, 64, 4, 8),
        ("mandelbulb_plane", 64, 48, 4, 6),
        ("feature_mix", 64, 48, 4, 6),
        ("menger_terrain", 48, 40, 4, 12),
    ],
)
def test_single_dispatch_matches_oracle(rt, name, W, H, spf, depth, engine):
    from oracle import compare

    scene, ctx, ubo, plugins = _setup(rt, name, W, H, engine)
    push = scene.push_constants(W, H, spf, spf, spf, depth)
    acc_o, tr_o = compare.run_oracle(ubo, push, plugins, trace_depth=depth)
    acc_g, tr_g = compare.run_gpu(ctx, push, trace_depth=depth)
    rep = compare.compare(acc_o, tr_o, acc_g, tr_g, spf)
    print(name, rep)
    _check(rep)
    ctx.close()


@pytest.mark.parametrize("engine", ENGINES)
def test_ragged_resolution_and_short_paths(rt, engine):
    """W, H not multiples of the 16x8 block; pathLength 1 and 0."""
    from oracle import compare

    W, H = 37, 23
    scene, ctx, ubo, plugins = _setup(rt, "feature_mix", W, H, engine)
    for depth in (1, 0):
        ctx.resize_accum(W, H)
        push = scene.push_constants(W, H, 3, 3, 3, depth)
        acc_o, tr_o = compare.run_oracle(ubo, push, plugins, trace_depth=max(depth, 1))
        acc_g, tr_g = compare.run_gpu(ctx, push, trace_depth=max(depth, 1))
        _check(compare.compare(acc_o, tr_o, acc_g, tr_g, 3))
    ctx.close()


@pytest.mark.parametrize("engine", ENGINES)
def test_progressive_running_mean_and_ema(rt, engine):
    """Several dispatches: running mean (SC:1504-1506), then a reset frame with
    frame > spf that takes the EMA branch (SC:1500-1502)."""
    from oracle import compare

    W, H, spf, depth = 40, 32, 2, 5
    scene, ctx, ubo, plugins = _setup(rt, "cornell_box", W, H, engine)
    acc_o = np.zeros((H, W, 4), np.float32)
    frame = cur = 0
    for it in range(4):
        frame += spf
        cur = spf if it == 3 else cur + spf  # the 4th dispatch is a reset with frame > spf
        push = scene.push_constants(W, H, frame, cur, spf, depth)
        acc_o, tr_o = compare.run_oracle(ubo, push, plugins, accum=acc_o, trace_depth=depth)
        acc_g, tr_g = compare.run_gpu(ctx, push, trace_depth=depth)
        _check(compare.compare(acc_o.copy(), tr_o, acc_g, tr_g, spf))
        ctx.write_accum(acc_o)  # continue both from the same state
    ctx.close()


def test_offscreen_loop_matches_oracle_loop(rt):
    """pt_render_offscreen (MainLoop offscreen) against the oracle driven the
    same way: frame and currentSamples += spf until numSamples."""
    from oracle import compare
    from pathtracer_gb300 import render_offscreen

    W, H, spf, n, depth = 48, 32, 3, 8, 6
    scene = rt["Scene"].load(os.path.join(SCENES, "mandelbulb_plane.json"))
    ubo = scene.pack_ubo(rt["cie"])
    plugins = compare.plugins_for(scene)
    with rt["Context"](0) as ctx:
        acc_g, secs = render_offscreen(ctx, scene, rt["cie"], W, H, n, spf, depth)
    acc_o = np.zeros((H, W, 4), np.float32)
    frame = cur = 0
    while True:
        frame += spf
        cur += spf
        compare.run_oracle(ubo, scene.push_constants(W, H, frame, cur, spf, depth), plugins, accum=acc_o)
        if cur >= n:
            break
    rel = np.abs(acc_o - acc_g) / np.maximum(np.maximum(np.abs(acc_o), np.abs(acc_g)), 1e-6)
    # No trace here: count pixels outside tolerance; path flips are rare.
    frac_bad = float(np.mean(rel[..., :3].max(axis=-1) > 1e-4))
    assert frac_bad < 0.02, frac_bad
    assert secs > 0


def test_error_paths(rt):
    from pathtracer_gb300 import PathTracerError, native

    ctx = rt["Context"](0)
    scene = rt["Scene"].load(os.path.join(SCENES, "cornell_box.json"))
    push = scene.push_constants(16, 16, 1, 1, 1, 4)
    with pytest.raises(PathTracerError) as e:
        ctx.dispatch(push)
    assert e.value.code == native.PT_ERR_NO_SCENE
    ctx.bind(scene, rt["cie"])
    ctx.resize_accum(8, 8)
    with pytest.raises(PathTracerError) as e:
        ctx.dispatch(push)  # resolution differs from the accumulator
    assert e.value.code == native.PT_ERR_INVALID
    bad = scene.pack_ubo(rt["cie"])
    bad[5] = 33.0  # 33 SDFs cannot be evaluated with a 32-bit set mask
    with pytest.raises(PathTracerError) as e:
        ctx.upload_scene(bad)
    assert e.value.code == native.PT_ERR_UNSUPPORTED
    with pytest.raises(PathTracerError):
        ctx.set_sdfs(["float sdf(in vec3 p) { return 1.0; }"])
    ctx.close()


def test_wait_deadline(rt):
    """pt_wait returns PT_ERR_TIMEOUT at its deadline instead of blocking, and
    the same context keeps working afterwards."""
    from pathtracer_gb300 import PathTracerError, native

    W = H = 512
    scene = rt["Scene"].load(os.path.join(SCENES, "mandelbulb_plane.json"))
    with rt["Context"](0) as ctx:
        ctx.set_engine(0)  # the megakernel's dispatch returns before the work is done
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        ctx.dispatch(scene.push_constants(W, H, 64, 64, 64, 6))
        try:
            ctx.wait(timeout_ns=1000)
            timed_out = False
        except PathTracerError as e:
            assert e.code == native.PT_ERR_TIMEOUT
            timed_out = True
        ctx.wait()
        acc = ctx.read_accum()
        assert np.isfinite(acc).all()
        assert timed_out


@pytest.mark.parametrize("name,W,H,spf,depth", [("mandelbulb_plane", 256, 256, 16, 6), ("feature_mix", 200, 150, 8, 8),
                                                ("menger_terrain", 160, 120, 8, 12)])
def test_wavefront_equals_megakernel_bitwise(rt, name, W, H, spf, depth):
    """The two engines schedule the same per-sample arithmetic differently;
    their accumulators are identical bit for bit."""
    scene = rt["Scene"].load(os.path.join(SCENES, name + ".json"))
    out = []
    for engine in ENGINES:
        with rt["Context"](0) as ctx:
            ctx.set_engine(engine)
            ctx.bind(scene, rt["cie"])
            ctx.resize_accum(W, H)
            for it in range(2):
                ctx.dispatch(scene.push_constants(W, H, spf * (it + 1), spf * (it + 1), spf, depth))
            ctx.wait()
            out.append(ctx.read_accum())
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


def test_wavefront_small_pool_recycles_slots(rt):
    """A pool far smaller than the sample count and a 3-step march budget:
    slots are freed and reused many times and marches are suspended and
    resumed across iterations; results stay identical to the oracle."""
    from oracle import compare

    W, H, spf, depth = 48, 40, 4, 6
    scene, ctx, ubo, plugins = _setup(rt, "feature_mix", W, H, 1)
    ctx.set_wavefront_pool(1024)
    ctx.set_march_budget(3)  # most marches are suspended and resumed several times
    push = scene.push_constants(W, H, spf, spf, spf, depth)
    acc_o, tr_o = compare.run_oracle(ubo, push, plugins, trace_depth=depth)
    acc_g, tr_g = compare.run_gpu(ctx, push, trace_depth=depth)
    _check(compare.compare(acc_o, tr_o, acc_g, tr_g, spf))
    assert ctx.last_iterations() > 10
    ctx.close()


@pytest.mark.parametrize("kind,seed", [(0, 4), (0, 9), (1, 2)])
def test_untraced_variants_match_oracle(rt, kind, seed):
    """Generated scenes through the specialised (untraced) kernel variants —
    the megakernel and the batch's persistent kernel — against the oracle:
    per-pixel XYZ identical."""
    from oracle import compare
    from pathtracer_gb300 import Batch, native

    scene, spec = rt["Scene"].generate(kind, seed)
    W, H, spf = 40, 32, 3
    push = scene.push_constants(W, H, spf, spf, spf, spec.pathLength)
    ubo = scene.pack_ubo(rt["cie"])
    acc_o, _ = compare.run_oracle(ubo, push, compare.plugins_for(scene))
    with rt["Context"](0) as ctx:
        ctx.set_engine(native.PT_ENGINE_MEGAKERNEL)
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        ctx.dispatch(push)
        ctx.wait()
        acc_m = ctx.read_accum()
    with Batch(0, pool_slots=1 << 12, max_passes=4) as b:
        b.set_route(native.PT_BATCH_ROUTE_PERSISTENT)
        sid = b.add_scene(ubo, scene.sdf_plugins())
        tid = b.add_target(W, H)
        b.add_pass(sid, tid, push)
        b.run()
        acc_p = b.read_target(tid)
    np.testing.assert_array_equal(acc_m[..., :3], acc_o[..., :3])
    np.testing.assert_array_equal(acc_p[..., :3], acc_o[..., :3])


def _capacity_scene(rt):
    """The uniform buffer filled to its limits: 160 spheres (960 of the 1024
    object floats) with 24 emitters, a plane, and 32 SDFs (every bit of the
    32-bit SDF set mask; 26 blobs, 4 mengers, 2 mandelbulbs)."""
    import json

    rng = np.random.default_rng(5)
    spheres = []
    for i in range(160):
        pos = [float(rng.uniform(-6, 6)), float(rng.uniform(0.2, 3)), float(rng.uniform(-9, 1))]
        spheres.append({"position": pos, "radius": float(rng.uniform(0.08, 0.3)),
                        "materialID": int(i % 4), "lightID": int(1 + i % 3) if i % 7 == 0 else 0})
    sdfs = []
    for i in range(32):
        x, z = -7.0 + 2.0 * (i % 8), -2.0 - 2.2 * (i // 8)
        kind = "mandelbulb" if i in (9, 22) else "menger" if i % 8 == 3 else "blob"
        scale = 0.45 if kind != "blob" else 0.35
        sdfs.append({"position": [x, 1.0, z], "boundingSize": [2.6 * scale * 2, 2.6 * scale * 2, 2.6 * scale * 2],
                     "builtin": kind})
    data = {
        "camera": {"numShots": 1, "position": [[0.0, 3.0, 6.0]], "angle": [[180.0, -12.0]], "ISO": 1600,
                   "size": 0.057, "apertureSize": 0.0025, "apertureDistance": 0.049, "lensRadius": 0.01,
                   "lensFocalLength": 0.03, "lensThickness": 0.0, "lensDistance": 0.05},
        "sphere": spheres,
        "plane": [{"position": [0.0, 0.0, 0.0], "materialID": 1, "lightID": 0}],
        "sdf": sdfs,
        "material": [{"reflection": {"peakWavelength": 450.0 + 40.0 * i, "sigma": 20.0 + 10.0 * i, "isInvert": i == 2}}
                     for i in range(7)],
        "light": [{"emission": {"temperature": 3000.0 + 1500.0 * i, "luminosity": 6.0}} for i in range(3)],
    }
    return rt["Scene"].parse(json.dumps(data))


@pytest.mark.parametrize("engine", ENGINES)
def test_capacity_scene_matches_oracle(rt, engine):
    from oracle import compare

    scene = _capacity_scene(rt)
    c = scene.counts()
    assert c["spheres"] == 160 and c["sdfs"] == 32
    W, H, spf, depth = 48, 32, 2, 4
    ctx = rt["Context"](0)
    ctx.set_engine(engine)
    ctx.bind(scene, rt["cie"])
    ctx.resize_accum(W, H)
    ubo = scene.pack_ubo(rt["cie"])
    assert ubo[5] == 32.0  # numObjects[5]: SDFs
    push = scene.push_constants(W, H, spf, spf, spf, depth)
    acc_o, tr_o = compare.run_oracle(ubo, push, compare.plugins_for(scene), trace_depth=depth)
    acc_g, tr_g = compare.run_gpu(ctx, push, trace_depth=depth)
    rep = compare.compare(acc_o, tr_o, acc_g, tr_g, spf)
    print(rep)
    _check(rep)
    ctx.close()


@pytest.mark.parametrize("engine", ENGINES)
def test_empty_scene_and_single_pixel(rt, engine):
    """A scene with no objects at all (every ray misses), and a 1x1 dispatch."""
    import json

    from oracle import compare

    with open(os.path.join(SCENES, "cornell_box.json")) as f:
        data = json.load(f)
    empty = {k: v for k, v in data.items() if k in ("camera", "material", "light")}
    for scene, (W, H) in ((rt["Scene"].parse(json.dumps(empty)), (24, 16)),
                          (rt["Scene"].load(os.path.join(SCENES, "feature_mix.json")), (1, 1))):
        ctx = rt["Context"](0)
        ctx.set_engine(engine)
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        push = scene.push_constants(W, H, 3, 3, 3, 5)
        acc_o, tr_o = compare.run_oracle(scene.pack_ubo(rt["cie"]), push, compare.plugins_for(scene), trace_depth=5)
        acc_g, tr_g = compare.run_gpu(ctx, push, trace_depth=5)
        _check(compare.compare(acc_o, tr_o, acc_g, tr_g, 3))
        ctx.close()


@pytest.mark.parametrize("which,name", [(0, "thritorius"), (1, "smooth_cuboid")])
def test_disabled_quartic_surfaces_match_oracle(rt, which, name):
    """The two quartic surfaces the reference's shader defines but never calls
    (Thritorius, SmoothCuboid; src/shader.comp:543-631) on the GPU against the
    oracle's restatement (itself pinned to the reference's own functions):
    hit flag and hit record bit for bit on rays aimed at and around them."""
    import ctypes

    import torch

    from oracle import oracle

    rng = np.random.default_rng(17 + which)
    n = 20000
    o = rng.uniform(-3.0, 3.0, (n, 3))
    d = rng.normal(size=(n, 3))
    aim = rng.uniform(size=n) < 0.5
    d[aim] = -o[aim] + rng.normal(0, 0.3, (int(aim.sum()), 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, d], axis=1).astype(np.float32)
    hits = np.zeros((n, 6), np.float32)
    hits[:, 0] = np.where(rng.uniform(size=n) < 0.7, 1e5, rng.uniform(0.5, 6.0, n)).astype(np.float32)
    hits[:, 5] = -1.0
    fn = getattr(oracle.lib(), f"pto_fn_{name}")
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    want = hits.copy()
    want_f = np.array([fn(rays[i].ctypes.data, None, want[i].ctypes.data) for i in range(n)], np.int32)
    with rt["Context"](0) as ctx:
        d_rays = torch.from_numpy(rays).cuda()
        d_hits = torch.from_numpy(hits).cuda()
        d_flags = torch.zeros(n, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        from pathtracer_gb300 import native

        assert native.cuda().pt_quartic_surface_eval(ctx.handle, which, d_rays.data_ptr(), d_hits.data_ptr(),
                                                     d_flags.data_ptr(), n) == native.PT_OK
        got, got_f = d_hits.cpu().numpy(), d_flags.cpu().numpy()
    assert np.array_equal(got_f, want_f)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert n // 50 < int(want_f.sum()) < n
