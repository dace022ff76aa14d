"""Render serving (pt_server_*) on the GPU: a job's result is the same bits
alone, in a mix of concurrent jobs, and through the plain serial megakernel;
admission keeps admitted jobs within the memory budget; arrival traces
replay with every job finishing after it arrived; cancelled jobs stop at a
pass boundary."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 48, 40


@pytest.fixture(scope="module")
def env(built):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from pathtracer_gb300 import native, renderer

    cie = renderer.cie_analytic()
    scenes = {}
    for key, (kind, seed) in enumerate(((native.PT_GEN_SPHERES, 31), (native.PT_GEN_SPHERES, 32),
                                        (native.PT_GEN_SDF, 33))):
        sc, spec = renderer.Scene.generate(kind, seed)
        scenes[key] = (sc, sc.pack_ubo(cie), sc.sdf_plugins(), sc.push_constants(W, H, 1, 1, 1, spec.pathLength))
    return native, renderer, scenes


def _server(renderer, native, scenes, mode, ref_spp=64, **kw):
    s = renderer.Server(0, mode=mode, keep_images=True, pool_slots=1 << 14, max_passes=256, **kw)
    for key, (_, ubo, plugins, push) in scenes.items():
        s.add_scene(key, ubo, plugins)
        s.render_reference(key, push, ref_spp, 32)
    return s


def _run(s, requests):
    ids = [s.submit(r) for r in requests]
    done = {r.job_id: r for r in s.drain()}
    assert set(done) == set(ids)
    return [(done[i], s.read_image(i)) for i in ids]


def test_job_is_the_same_alone_in_a_mix_and_plain(env):
    native, renderer, scenes = env
    target = 0.25  # reachable in a few 8-spp passes at this size

    def req(key, max_spp=96):
        return renderer.Server.job(key, scenes[key][3], max_spp, target)

    mix = [req(0), req(1), req(2), req(0, 32), req(1), req(2, 16)]
    with _server(renderer, native, scenes, native.PT_SERVE_BATCHED) as s:
        in_mix = _run(s, mix)
    for k, r in enumerate(mix):
        with _server(renderer, native, scenes, native.PT_SERVE_BATCHED) as s:
            (alone_r, alone_img), = _run(s, [r])
        mix_r, mix_img = in_mix[k]
        assert np.array_equal(alone_img.view(np.uint32), mix_img.view(np.uint32)), k
        assert (alone_r.spp, alone_r.rmse) == (mix_r.spp, mix_r.rmse)
        assert mix_r.spp <= r.max_spp and mix_r.spp % 8 == 0
        assert mix_r.rmse <= target or mix_r.spp == r.max_spp
    # the plain path gives the same bits, pass count and error
    with _server(renderer, native, scenes, native.PT_SERVE_PLAIN) as s:
        for k, r in enumerate(mix):
            (plain_r, plain_img), = _run(s, [r])
            mix_r, mix_img = in_mix[k]
            assert np.array_equal(plain_img.view(np.uint32), mix_img.view(np.uint32)), k
            assert (plain_r.spp, plain_r.rmse) == (mix_r.spp, mix_r.rmse)


def test_admission_respects_the_memory_budget(env):
    native, renderer, scenes = env
    per_job = W * H * 16 * (1 + 8)  # accumulator + one 8-spp pass of colours
    with _server(renderer, native, scenes, native.PT_SERVE_BATCHED, hbm_budget=2 * per_job + 100) as s:
        reqs = [renderer.Server.job(k % 3, scenes[k % 3][3], 24) for k in range(7)]
        out = _run(s, reqs)
        st = s.stats()
        assert st["completed"] == 7 and st["queued"] == 0 and st["active"] == 0
        assert 0 < st["bytes_peak"] <= 2 * per_job
        assert st["bytes_in_use"] == 0
        assert all(r.spp == 24 for r, _ in out)


def test_trace_replay(env):
    native, renderer, scenes = env
    with _server(renderer, native, scenes, native.PT_SERVE_BATCHED) as s:
        reqs = [renderer.Server.job(k % 3, scenes[k % 3][3], 64, 0.3) for k in range(12)]
        arrivals = [0.005 * k for k in range(12)]
        res = s.run_trace(reqs, arrivals)
    for r, a in zip(res, arrivals):
        assert r.t_submit == pytest.approx(a, abs=1e-9)
        assert r.t_done >= r.t_admit >= r.t_submit - 1e-6
        assert r.samples == W * H * r.spp > 0


def test_server_errors(env):
    native, renderer, scenes = env
    with _server(renderer, native, scenes, native.PT_SERVE_BATCHED, hbm_budget=1 << 20) as s:
        with pytest.raises(renderer.PathTracerError) as e:
            s.submit(renderer.Server.job(9, scenes[0][3], 8))  # unknown scene
        assert e.value.code == native.PT_ERR_INVALID
        big = renderer.Server.job(0, scenes[0][3], 8, 0.1)
        big.push.resolution[0], big.push.resolution[1] = 64, 64  # no reference at this size
        with pytest.raises(renderer.PathTracerError) as e:
            s.submit(big)
        assert e.value.code == native.PT_ERR_INVALID
        huge = renderer.Server.job(0, scenes[0][3], 8)
        huge.push.resolution[0], huge.push.resolution[1] = 1024, 1024  # 144 MiB > 1 MiB budget
        with pytest.raises(renderer.PathTracerError) as e:
            s.submit(huge)
        assert e.value.code == native.PT_ERR_TOO_LARGE


def test_cancel_queued_admitted_and_plain(env):
    """A queued job is dropped at once; an admitted one stops after its pass
    in flight; the plain path stops between passes.  Cancelled jobs come back
    with PT_ERR_CANCELLED and the samples they rendered; the others finish."""
    native, renderer, scenes = env
    per_job = W * H * 16 * (1 + 8)
    with _server(renderer, native, scenes, native.PT_SERVE_BATCHED, hbm_budget=per_job + 100) as s:
        ids = [s.submit(renderer.Server.job(k, scenes[k][3], 512 if k == 0 else 24)) for k in range(3)]
        s.cancel(ids[2])  # still queued
        first = s.poll()  # admits job 0 (budget: one job), queues its first pass, returns the cancelled one
        assert [r.job_id for r in first] == [ids[2]]
        assert first[0].status == native.PT_ERR_CANCELLED and first[0].spp == 0 and first[0].t_admit < 0
        assert s.stats()["active"] == 1
        s.cancel(ids[0])  # admitted, pass in flight
        done = {r.job_id: r for r in s.drain()}
        assert set(done) == {ids[0], ids[1]}
        assert done[ids[0]].status == native.PT_ERR_CANCELLED and 8 <= done[ids[0]].spp < 512
        assert done[ids[1]].status == native.PT_OK and done[ids[1]].spp == 24
        assert s.stats()["bytes_in_use"] == 0
        with pytest.raises(renderer.PathTracerError) as e:
            s.cancel(ids[1])  # finished
        assert e.value.code == native.PT_ERR_INVALID
    with _server(renderer, native, scenes, native.PT_SERVE_PLAIN) as s:
        a = s.submit(renderer.Server.job(0, scenes[0][3], 512))
        b = s.submit(renderer.Server.job(1, scenes[1][3], 16))
        assert s.poll() == []  # one pass of job a
        s.cancel(a)
        done = {r.job_id: r for r in s.drain()}
        assert done[a].status == native.PT_ERR_CANCELLED and done[a].spp == 8
        assert done[b].status == native.PT_OK and done[b].spp == 16
