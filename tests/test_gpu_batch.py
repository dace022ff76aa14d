"""Batched rendering (pt_batch_*) on the GPU: every pass of a mixed batch —
different scenes, resolutions and sample counts sharing one path pool — ends
bit-identical to the same push constants dispatched alone through pt_dispatch,
whose parity with the oracle tests/test_gpu_parity.py establishes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from pathtracer_gb300 import native, renderer

    return native, renderer, renderer.cie_analytic()


def _jobs(renderer, native):
    """Three generated scenes at small sizes: two sphere jobs and an SDF job."""
    out = []
    for kind, seed, (w, h), spf in ((native.PT_GEN_SPHERES, 1, (48, 40), 3), (native.PT_GEN_SPHERES, 2, (33, 17), 5),
                                    (native.PT_GEN_SDF, 3, (40, 32), 2)):
        scene, spec = renderer.Scene.generate(kind, seed)
        out.append((scene, w, h, spf, spec.pathLength))
    return out


def _dispatch_alone(renderer, cie, scene, w, h, spf, depth, passes, engine):
    with renderer.Context(0) as ctx:
        ctx.set_engine(engine)
        ctx.bind(scene, cie)
        ctx.resize_accum(w, h)
        for k in range(1, passes + 1):
            ctx.dispatch(scene.push_constants(w, h, k * spf, k * spf, spf, depth))
        ctx.wait()
        return ctx.read_accum()


ROUTES = ("auto", "staged", "persistent")


def _route(native, name):
    return {"auto": native.PT_BATCH_ROUTE_AUTO, "staged": native.PT_BATCH_ROUTE_STAGED,
            "persistent": native.PT_BATCH_ROUTE_PERSISTENT}[name]


@pytest.mark.parametrize("route", ROUTES)
def test_mixed_batch_matches_single_dispatches(env, route):
    native, renderer, cie = env
    jobs = _jobs(renderer, native)
    passes = 2
    with renderer.Batch(0, pool_slots=1 << 14, max_passes=64) as b:
        b.set_route(_route(native, route))
        ids = []
        for scene, w, h, spf, depth in jobs:
            sid = b.add_scene(scene.pack_ubo(cie), scene.sdf_plugins())
            ids.append((sid, b.add_target(w, h)))
        # interleave the passes of all jobs in one pool
        for k in range(1, passes + 1):
            for (sid, tid), (scene, w, h, spf, depth) in zip(ids, jobs):
                b.add_pass(sid, tid, scene.push_constants(w, h, k * spf, k * spf, spf, depth))
        b.run()
        assert b.pending() == 0
        got = [b.read_target(tid) for _, tid in ids]
        for (_, tid), (scene, w, h, spf, depth) in zip(ids, jobs):
            assert b.target_samples(tid) == passes * spf
        st = b.stats()
        assert st["samples_done"] == st["samples_added"] == sum(w * h * spf * passes for _, w, h, spf, _ in jobs)
        staged = {"auto": 2, "staged": 6, "persistent": 0}[route]  # the SDF job's two passes under auto
        assert (st["passes_staged"], st["passes_persistent"]) == (staged, 6 - staged)
    for g, (scene, w, h, spf, depth) in zip(got, jobs):
        want = _dispatch_alone(renderer, cie, scene, w, h, spf, depth, passes, native.PT_ENGINE_MEGAKERNEL)
        assert np.array_equal(g.view(np.uint32), want.view(np.uint32))
        assert np.isfinite(g).all() and g[..., :3].sum() > 0


@pytest.mark.parametrize("route", ("staged", "persistent"))
def test_pass_ring_wraps_and_keeps_target_order(env, route):
    """Eight progressive passes of one job through a ring of three pass slots:
    passes complete in order and the result equals eight dispatches."""
    native, renderer, cie = env
    scene, _ = renderer.Scene.generate(native.PT_GEN_SPHERES, 7)
    w, h, spf, depth, passes = 24, 20, 2, 8, 8
    with renderer.Batch(0, pool_slots=1024, max_passes=3) as b:
        b.set_route(_route(native, route))
        sid = b.add_scene(scene.pack_ubo(cie), scene.sdf_plugins())
        tid = b.add_target(w, h)
        added, done = 0, []
        while len(done) < passes:
            while added < passes:
                try:
                    b.add_pass(sid, tid, scene.push_constants(w, h, (added + 1) * spf, (added + 1) * spf, spf, depth))
                except renderer.PathTracerError as e:
                    assert e.code == native.PT_ERR_BUSY
                    break
                added += 1
            done += b.step(4)
        assert done == sorted(done) == list(range(passes))
        got = b.read_target(tid)
    want = _dispatch_alone(renderer, cie, scene, w, h, spf, depth, passes, native.PT_ENGINE_WAVEFRONT)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_fp64_target_and_rmse(env):
    """An FP64 target holds the mean of the exposed sample colours: one pass
    into it equals one pass into a float target to float rounding, and the
    device RMSE reduction agrees with numpy."""
    native, renderer, cie = env
    scene, _ = renderer.Scene.generate(native.PT_GEN_SPHERES, 11)
    w, h, spf, depth = 32, 24, 4, 8
    push = scene.push_constants(w, h, spf, spf, spf, depth)
    with renderer.Batch(0, pool_slots=1 << 12, max_passes=8) as b:
        sid = b.add_scene(scene.pack_ubo(cie), scene.sdf_plugins())
        tf = b.add_target(w, h)
        td = b.add_target(w, h, native.PT_TARGET_FP64)
        tf2 = b.add_target(w, h)
        b.add_pass(sid, tf, push)
        b.add_pass(sid, td, push)
        b.add_pass(sid, tf2, scene.push_constants(w, h, spf, spf, spf, 3))  # shorter paths: another image
        b.run()
        a, d, a2 = b.read_target(tf), b.read_target(td), b.read_target(tf2)
        assert b.target_samples(td) == spf
        np.testing.assert_allclose(d[..., :3], a[..., :3], rtol=2e-6, atol=1e-12)
        assert b.rmse(tf, tf) == 0.0
        assert b.rmse(tf, td) < 1e-6
        r = b.rmse(tf2, tf)
        want = np.sqrt(((a2[..., :3].astype(np.float64) - a[..., :3]) ** 2).sum() / (a[..., :3].astype(np.float64) ** 2).sum())
        assert r == pytest.approx(want, rel=1e-9)
        assert r > 0.0


def test_persistent_launch_budget_splits_a_pass(env):
    """A pass larger than one persistent launch (2^23 samples) spans several
    launches and still matches the megakernel bit for bit."""
    native, renderer, cie = env
    scene, _ = renderer.Scene.generate(native.PT_GEN_SPHERES, 21)
    w, h, spf, depth = 1024, 1024, 9, 8  # 9.4 M samples: two launches
    push = scene.push_constants(w, h, spf, spf, spf, depth)
    with renderer.Batch(0, pool_slots=1 << 16, max_passes=4) as b:
        b.set_route(native.PT_BATCH_ROUTE_PERSISTENT)
        sid = b.add_scene(scene.pack_ubo(cie), scene.sdf_plugins())
        tid = b.add_target(w, h)
        b.add_pass(sid, tid, push)
        b.run()
        got = b.read_target(tid)
        assert b.stats()["iterations"] >= 2
    want = _dispatch_alone(renderer, cie, scene, w, h, spf, depth, 1, native.PT_ENGINE_MEGAKERNEL)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_batch_errors(env):
    native, renderer, cie = env
    scene, _ = renderer.Scene.generate(native.PT_GEN_SPHERES, 3)
    with renderer.Batch(0, pool_slots=1024, max_passes=4) as b:
        sid = b.add_scene(scene.pack_ubo(cie), scene.sdf_plugins())
        tid = b.add_target(16, 16)
        with pytest.raises(renderer.PathTracerError) as e:
            b.add_pass(sid, tid, scene.push_constants(16, 8, 1, 1, 1, 8))  # wrong resolution
        assert e.value.code == native.PT_ERR_INVALID
        with pytest.raises(renderer.PathTracerError) as e:
            b.add_pass(sid + 5, tid, scene.push_constants(16, 16, 1, 1, 1, 8))
        assert e.value.code == native.PT_ERR_INVALID
        b.add_pass(sid, tid, scene.push_constants(16, 16, 1, 1, 1, 8))
        for release in (b.release_target, lambda _: b.release_scene(sid)):
            with pytest.raises(renderer.PathTracerError) as e:
                release(tid)
            assert e.value.code == native.PT_ERR_BUSY
        b.run()
        b.release_target(tid)
        b.release_scene(sid)
        with pytest.raises(renderer.PathTracerError) as e:
            b.read_target(tid)
        assert e.value.code == native.PT_ERR_INVALID
        bad = scene.pack_ubo(cie)
        bad[0] = 1.5  # non-integral sphere count
        with pytest.raises(renderer.PathTracerError) as e:
            b.add_scene(bad, [])
        assert e.value.code == native.PT_ERR_INVALID


@pytest.mark.parametrize("seeds", [(0, 2, 5), (2, 5, 7)], ids=["with_mandelbulb", "even_cost_sdfs"])
def test_sdf_scenes_share_march_warps(env, seeds):
    """Three SDF scenes of different plug-ins in one staged pool: a march warp
    holds rays of several scenes.  With a mandelbulb in the batch (seeds 0, 2,
    5: mandelbulb, blob, menger) the normals of converged rays are probed
    across the warp's lanes with each ray's own scene; without one (blob,
    menger, menger) each ray probes on its own lane.  Each image equals the
    plain megakernel's bit for bit."""
    native, renderer, cie = env
    jobs = []
    for seed, (w, h), spf in zip(seeds, ((40, 36), (36, 30), (44, 28)), (3, 2, 2)):
        scene, spec = renderer.Scene.generate(native.PT_GEN_SDF, seed)
        jobs.append((scene, w, h, spf, spec.pathLength))
    with renderer.Batch(0, pool_slots=1 << 13, max_passes=16) as b:
        b.set_route(native.PT_BATCH_ROUTE_STAGED)
        ids = [(b.add_scene(s.pack_ubo(cie), s.sdf_plugins()), b.add_target(w, h)) for s, w, h, _, _ in jobs]
        for k in (1, 2):
            for (sid, tid), (scene, w, h, spf, depth) in zip(ids, jobs):
                b.add_pass(sid, tid, scene.push_constants(w, h, k * spf, k * spf, spf, depth))
        b.run()
        got = [b.read_target(tid) for _, tid in ids]
    for g, (scene, w, h, spf, depth) in zip(got, jobs):
        want = _dispatch_alone(renderer, cie, scene, w, h, spf, depth, 2, native.PT_ENGINE_MEGAKERNEL)
        assert np.array_equal(g.view(np.uint32), want.view(np.uint32))
        assert g[..., :3].sum() > 0
