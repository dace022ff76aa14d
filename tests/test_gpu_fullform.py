"""The full-form extensions on the GPU against the oracle (pt_scene_ext:
environment sky, wavelength range, analytic CMF, march limits, flat and
smooth Lambertian spectra, conductor mirror, Cauchy and Sellmeier
dielectrics).

The GPU side binds the product's scene (libpt_host packs the extensions);
the oracle side packs the same JSON with the oracle's own restatement
(oracle/pack.py), so the packer is not checked against itself.  Every engine
runs the scenes of the workloads in their full form:
- cornell_box_full (flat 0.75 sphere, Cauchy A 1.5, B 0.0042 um^2 sphere,
  380-780 nm, analytic CMF): small and at 256x256, 16 spp, depth 8;
- mandelbulb12_plane_full (smooth bulb spectrum, flat 0.5 plane, 5800 K sky,
  256-step march capped at distance 50): small and at 1024x1024, 64 spp,
  depth 6 (16 rows);
- menger_terrain_full (Menger sponge on an fBm terrain compiled at run time,
  Sellmeier BK7-like glass sphere): small and at 1920x1080, 16 spp, depth 12;
- seeded sphere jobs with mirrors and Cauchy dielectrics through the batch
  (persistent and staged routes) and the server.
Criteria as in test_gpu_parity.py: >= 99.9 % of paths identical, matching
paths within 1e-4 relative in XYZ, pixels whose paths all match within 1e-4.
"""
import os

import numpy as np
import pytest

from conftest import SCENES

pytestmark = pytest.mark.gpu

ENGINES = [0, 1]
FULL = ["cornell_box_full", "mandelbulb12_plane_full", "menger_terrain_full"]


@pytest.fixture(scope="module")
def rt(built):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("no CUDA device: -m gpu tests need a GPU")
    from pathtracer_gb300 import Context, Scene, cie_analytic

    return {"Context": Context, "Scene": Scene, "cie": cie_analytic()}


def _oracle_side(name):
    """ubo, ext and plug-ins of a scene file from the oracle's restatement."""
    from oracle import oracle, pack

    sc = pack.load_scene(os.path.join(SCENES, name + ".json"))
    return sc, sc.pack_ubo(pack.cie_analytic()), sc.pack_ext(), oracle.plugins_for_sources(sc.sdf_sources())


def _ctx(rt, name, W, H, engine):
    scene = rt["Scene"].load(os.path.join(SCENES, name + ".json"))
    ctx = rt["Context"](0)
    ctx.set_engine(engine)
    ctx.bind(scene, rt["cie"])
    ctx.resize_accum(W, H)
    return scene, ctx


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("name,W,H,spf,depth", [("cornell_box_full", 64, 64, 4, 8),
                                                ("mandelbulb12_plane_full", 64, 48, 4, 6),
                                                ("menger_terrain_full", 48, 40, 4, 12)])
def test_full_form_scene_matches_oracle(rt, name, W, H, spf, depth, engine):
    from oracle import compare

    osc, ubo, ext, plugins = _oracle_side(name)
    assert ext.flags
    scene, ctx = _ctx(rt, name, W, H, engine)
    push = scene.push_constants(W, H, spf, spf, spf, depth)
    acc_o, tr_o = compare.run_oracle(ubo, osc.push_constants(W, H, spf, spf, spf, depth), plugins,
                                     trace_depth=depth, ext=ext)
    acc_g, tr_g = compare.run_gpu(ctx, push, trace_depth=depth)
    rep = compare.compare(acc_o, tr_o, acc_g, tr_g, spf)
    print(name, "engine", engine, rep)
    assert compare.passes(rep), rep
    ctx.close()


def _rows(H, n):
    return sorted({int(round(i * (H - 1) / (n - 1))) for i in range(n)})


def _traced_rows(ctx, push, ys, depth):
    import torch

    W, H, spf = push.resolution[0], push.resolution[1], push.samplesPerFrame
    n = W * H * spf
    ev = torch.zeros(n * depth, dtype=torch.int32, device="cuda")
    nev = torch.zeros(n, dtype=torch.int32, device="cuda")
    col = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.set_trace(ev.data_ptr(), nev.data_ptr(), col.data_ptr(), depth)
    ctx.dispatch(push)
    ctx.wait()
    ctx.set_trace(0, 0, 0, 0)
    idx = torch.tensor(ys, device="cuda")
    return ctx.read_accum(), (
        ev.view(H, W, spf, depth).index_select(0, idx).reshape(-1, depth).cpu().numpy().view(np.uint32),
        nev.view(H, W, spf).index_select(0, idx).reshape(-1).cpu().numpy().view(np.uint32),
        col.view(H, W, spf, 3).index_select(0, idx).reshape(-1, 3).cpu().numpy())


_CACHE = {}


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("name,W,H,spf,depth,nrows", [("cornell_box_full", 256, 256, 16, 8, 256),
                                                      ("mandelbulb12_plane_full", 1024, 1024, 64, 6, 16),
                                                      ("menger_terrain_full", 1920, 1080, 16, 12, 4)])
def test_full_form_at_workload_size(rt, name, W, H, spf, depth, nrows, engine):
    """Each full-form workload at its own size (every row of the Cornell box,
    stratified rows of the others), per path."""
    from oracle import compare

    osc, ubo, ext, plugins = _oracle_side(name)
    ys = list(range(H)) if nrows >= H else _rows(H, nrows)
    key = name
    if key not in _CACHE:
        acc_o = np.zeros((H, W, 4), np.float32)
        opush = osc.push_constants(W, H, spf, spf, spf, depth)
        parts = [compare.run_oracle(ubo, opush, plugins, accum=acc_o, rect=(0, y, W, y + 1), trace_depth=depth,
                                    ext=ext)[1] for y in ys]
        _CACHE[key] = (acc_o[ys].copy(), tuple(np.concatenate([p[i] for p in parts]) for i in range(3)))
    acc_rows, tr_o = _CACHE[key]
    scene, ctx = _ctx(rt, name, W, H, engine)
    acc_g, tr_g = _traced_rows(ctx, scene.push_constants(W, H, spf, spf, spf, depth), ys, depth)
    rep = compare.compare(acc_rows, tr_o, acc_g[ys], tr_g, spf)
    print(f"{name} {W}x{H}x{spf} engine {engine}", rep)
    assert compare.passes(rep), rep
    ctx.close()


def _pixel_report(want, got):
    a, b = want[..., :3].reshape(-1, 3), got[..., :3].reshape(-1, 3)
    floor = max(1e-6, float(np.abs(a).max()) * 1e-6)
    rel = (np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)).max(axis=1)
    return {"pixels": int(rel.size), "within_tol": float(np.mean(rel <= 1e-4)), "max_rel": float(rel.max()),
            "bit_identical": float(np.mean(np.all(want.view(np.uint32) == got.view(np.uint32), axis=-1)))}


@pytest.mark.parametrize("route", ["persistent", "staged"])
def test_full_form_sphere_jobs_in_a_batch(rt, route):
    """Seeded sphere jobs with mirrors and Cauchy dielectrics
    (PT_GEN_SPHERES_FULL) at their own sizes in one batch, against the oracle
    on two rows of each job."""
    from oracle import compare
    from pathtracer_gb300 import Batch, native

    cie = rt["cie"]
    jobs = []
    for seed in (0, 2, 3, 8):  # 512^2x248, 128^2x137, 1024^2x9, 256^2x182
        scene, spec = rt["Scene"].generate(native.PT_GEN_SPHERES_FULL, seed)
        jobs.append((seed, scene, spec.width, spec.height, spec.spp, spec.pathLength))
    r = {"persistent": native.PT_BATCH_ROUTE_PERSISTENT, "staged": native.PT_BATCH_ROUTE_STAGED}[route]
    with Batch(0, pool_slots=1 << 19, max_passes=256) as b:
        b.set_route(r)
        tids = []
        for seed, scene, W, H, spp, depth in jobs:
            sid = b.add_scene(scene.pack_ubo(cie), scene.sdf_plugins())
            b.set_scene_ext(sid, scene.pack_ext())
            tid = b.add_target(W, H)
            b.add_pass(sid, tid, scene.push_constants(W, H, spp, spp, spp, depth))
            tids.append(tid)
        b.run()
        got = [b.read_target(t) for t in tids]
    for (seed, scene, W, H, spp, depth), g in zip(jobs, got):
        ys = _rows(H, 2)
        acc_o = np.zeros((H, W, 4), np.float32)
        for y in ys:
            compare.run_oracle(scene.pack_ubo(cie), scene.push_constants(W, H, spp, spp, spp, depth), [],
                               accum=acc_o, rect=(0, y, W, y + 1), ext=_o_ext(scene))
        rep = _pixel_report(acc_o[ys], g[ys])
        print(f"full-form job seed {seed} {W}x{H}x{spp} route {route}", rep)
        assert rep["within_tol"] >= 0.999, (seed, rep)


def _o_ext(scene):
    """A generated job's extension block in the oracle's struct (same layout;
    the oracle-side packer is pinned to the product's in test_oracle_pack.py)."""
    from oracle import pack

    return pack.PtoSceneExt.from_buffer_copy(bytes(scene.pack_ext()))


def test_full_form_served_job_alone_in_a_mix_and_plain(rt):
    """A served full-form job (mirrors and dielectrics) ends with the same
    image, pass count and error batched alone, batched among other jobs, and
    on the plain path."""
    from pathtracer_gb300 import Server, native

    cie = rt["cie"]
    W = H = 48
    scenes = [rt["Scene"].generate(native.PT_GEN_SPHERES_FULL, s) for s in (20, 21, 22)]

    def server(mode):
        srv = Server(0, mode=mode, keep_images=True, pool_slots=1 << 14, max_passes=256)
        for k, (sc, spec) in enumerate(scenes):
            srv.add_scene(k, sc.pack_ubo(cie), sc.sdf_plugins())
            srv.set_scene_ext(k, sc.pack_ext())
            srv.render_reference(k, sc.push_constants(W, H, 1, 1, 1, spec.pathLength), 64, 32)
        return srv

    def req(k):
        sc, spec = scenes[k]
        return Server.job(k, sc.push_constants(W, H, 1, 1, 1, spec.pathLength), 32, 0.25)

    def run(srv, reqs):
        ids = [srv.submit(r) for r in reqs]
        done = {r.job_id: r for r in srv.drain()}
        return [(done[i], srv.read_image(i)) for i in ids]

    with server(native.PT_SERVE_BATCHED) as srv:
        (ar, alone), = run(srv, [req(0)])
    with server(native.PT_SERVE_BATCHED) as srv:
        mr, mixed = run(srv, [req(1), req(0), req(2)])[1]
    with server(native.PT_SERVE_PLAIN) as srv:
        (pr, plain), = run(srv, [req(0)])
    assert np.array_equal(alone.view(np.uint32), mixed.view(np.uint32))
    assert np.array_equal(alone.view(np.uint32), plain.view(np.uint32))
    assert (ar.spp, ar.rmse) == (mr.spp, mr.rmse) == (pr.spp, pr.rmse)
    assert alone[..., :3].sum() > 0
