"""Parity with the oracle at the workloads' own sizes, on the routes that
serve them.

The small-image parity tests (test_gpu_parity.py) cannot show what only
appears at full size: a path pool recycled many times, marches
suspended and resumed over many iterations, queue indices wrapping around
the path pool, grids of thousands of blocks.  Here each workload runs
at its stated size through the same entry point and settings as bench.py,
and the oracle (oracle/pt_oracle.c) renders a stratified set of rows of the
same frame (all of it where that is cheap) for comparison:
- the Cornell box, 256x256, 16 spp, depth 8: the whole frame, per path,
  both engines;
- the 12-iteration power-8 mandelbulb over a plane, 1024x1024, 64 spp,
  depth 6: 16 rows, per path (traced dispatch) and per pixel (the untraced
  dispatch the bench times), both engines;
- menger sponge + terrain, 1920x1080, depth 12, two progressive 16-spp
  passes: 4 rows, per path, both engines;
- five seeded sphere jobs of the 64-job batch (128^2 to 1024^2, 9 to 248
  spp, depth 8) in one batch on the persistent route: 2 rows each, per
  pixel.

Criteria (oracle/compare.py): >= 99.9 % of paths take the identical branch
sequence, matching paths agree in XYZ within 1e-4 relative, pixels whose
paths all match agree in the accumulator within 1e-4 relative.  Untraced
pixels: >= 99.9 % of pixels within 1e-4 relative.  Each test prints the
path-match fraction and the largest relative error it saw.
"""
import os

import numpy as np
import pytest

from conftest import SCENES

pytestmark = pytest.mark.gpu

ENGINES = [0, 1]  # PT_ENGINE_MEGAKERNEL, PT_ENGINE_WAVEFRONT
REL_TOL = 1e-4
PIXEL_MATCH_MIN = 0.999


@pytest.fixture(scope="module")
def rt(built):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("no CUDA device: -m gpu tests need a GPU")
    from pathtracer_gb300 import Context, Scene, cie_analytic

    return {"Context": Context, "Scene": Scene, "cie": cie_analytic()}


def _rows(H, n):
    """n rows spread over the frame, first and last included."""
    return sorted({int(round(i * (H - 1) / (n - 1))) for i in range(n)}) if n > 1 else [H // 2]


class _Trace:
    """A per-path trace of one whole dispatch in device memory; rows are
    copied out as the compare module expects them."""

    def __init__(self, W, H, spf, depth):
        import torch

        n = W * H * spf
        self.shape = (H, W, spf, depth)
        self.ev = torch.zeros(n * depth, dtype=torch.int32, device="cuda")
        self.nev = torch.zeros(n, dtype=torch.int32, device="cuda")
        self.col = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()

    def attach(self, ctx):
        ctx.set_trace(self.ev.data_ptr(), self.nev.data_ptr(), self.col.data_ptr(), self.shape[3])

    def rows(self, ys):
        H, W, spf, depth = self.shape
        idx = __import__("torch").tensor(ys, device="cuda")
        ev = self.ev.view(H, W, spf, depth).index_select(0, idx).reshape(-1, depth).cpu().numpy().view(np.uint32)
        nev = self.nev.view(H, W, spf).index_select(0, idx).reshape(-1).cpu().numpy().view(np.uint32)
        col = self.col.view(H, W, spf, 3).index_select(0, idx).reshape(-1, 3).cpu().numpy()
        return ev, nev, col


_ORACLE_CACHE = {}


def _oracle_rows(ubo, push, plugins, acc, ys, depth, key=None):
    """The oracle over rows ys (updating acc in place), traces concatenated in
    row order.  With a key the result is kept for the other engine's test."""
    from oracle import compare

    if key is not None and key in _ORACLE_CACHE:
        rows, tr = _ORACLE_CACHE[key]
        acc[ys] = rows
        return tr
    W = push.resolution[0]
    parts = [compare.run_oracle(ubo, push, plugins, accum=acc, rect=(0, y, W, y + 1), trace_depth=depth)[1]
             for y in ys]
    tr = tuple(np.concatenate([p[i] for p in parts]) for i in range(3))
    if key is not None:
        _ORACLE_CACHE[key] = (acc[ys].copy(), tr)
    return tr


def _pixel_report(want, got):
    """Per-pixel agreement of two accumulator row sets (untraced runs)."""
    a, b = want[..., :3].reshape(-1, 3), got[..., :3].reshape(-1, 3)
    floor = max(1e-6, float(np.abs(a).max()) * 1e-6)
    rel = (np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)).max(axis=1)
    return {"pixels": int(rel.size), "within_tol": float(np.mean(rel <= REL_TOL)),
            "bit_identical": float(np.mean(np.all(want.view(np.uint32) == got.view(np.uint32), axis=-1).reshape(-1))),
            "max_rel": float(rel.max()), "w_ok": bool(np.all(got[..., 3] == 1.0))}


def _pixel_ok(rep):
    return rep["within_tol"] >= PIXEL_MATCH_MIN and rep["w_ok"]


def _setup(rt, name, W, H, engine):
    from oracle import compare

    scene = rt["Scene"].load(os.path.join(SCENES, name + ".json"))
    ctx = rt["Context"](0)
    ctx.set_engine(engine)
    ctx.bind(scene, rt["cie"])
    ctx.resize_accum(W, H)
    return scene, ctx, scene.pack_ubo(rt["cie"]), compare.plugins_for(scene)


@pytest.mark.parametrize("engine", ENGINES)
def test_cornell_box_256_16spp_depth8_whole_frame(rt, engine):
    from oracle import compare

    W, H, spf, depth = 256, 256, 16, 8
    scene, ctx, ubo, plugins = _setup(rt, "cornell_box", W, H, engine)
    push = scene.push_constants(W, H, spf, spf, spf, depth)
    acc_o, tr_o = compare.run_oracle(ubo, push, plugins, trace_depth=depth)
    acc_g, tr_g = compare.run_gpu(ctx, push, trace_depth=depth)
    rep = compare.compare(acc_o, tr_o, acc_g, tr_g, spf)
    print("cornell_box 256x256x16 engine", engine, rep)
    assert compare.passes(rep), rep
    ctx.close()


@pytest.mark.parametrize("engine", ENGINES)
def test_mandelbulb12_1024_64spp_depth6_rows(rt, engine):
    """The bench's workload and dispatch (one dispatch of 64 spp; the
    wavefront engine with its default pool and knobs)."""
    from oracle import compare

    W, H, spf, depth = 1024, 1024, 64, 6
    ys = _rows(H, 16)
    scene, ctx, ubo, plugins = _setup(rt, "mandelbulb12_plane", W, H, engine)
    push = scene.push_constants(W, H, spf, spf, spf, depth)
    acc_o = np.zeros((H, W, 4), np.float32)
    tr_o = _oracle_rows(ubo, push, plugins, acc_o, ys, depth, key="mandelbulb12")
    # traced dispatch: per path
    tr = _Trace(W, H, spf, depth)
    tr.attach(ctx)
    ctx.dispatch(push)
    ctx.wait()
    ctx.set_trace(0, 0, 0, 0)
    acc_t = ctx.read_accum()
    rep = compare.compare(acc_o[ys], tr_o, acc_t[ys], tr.rows(ys), spf)
    print("mandelbulb12 1024x1024x64 traced engine", engine, rep)
    assert compare.passes(rep), rep
    del tr
    # the untraced dispatch the bench times: per pixel
    ctx.resize_accum(W, H)
    ctx.dispatch(push)
    ctx.wait()
    prep = _pixel_report(acc_o[ys], ctx.read_accum()[ys])
    print("mandelbulb12 1024x1024x64 untraced engine", engine, prep)
    assert _pixel_ok(prep), prep
    ctx.close()


@pytest.mark.parametrize("engine", ENGINES)
def test_menger_terrain_1080p_progressive_16spp_passes(rt, engine):
    from oracle import compare

    W, H, spf, depth = 1920, 1080, 16, 12
    ys = _rows(H, 4)
    scene, ctx, ubo, plugins = _setup(rt, "menger_terrain", W, H, engine)
    acc_o = np.zeros((H, W, 4), np.float32)
    tr = _Trace(W, H, spf, depth)
    for k in (1, 2):
        push = scene.push_constants(W, H, k * spf, k * spf, spf, depth)
        tr_o = _oracle_rows(ubo, push, plugins, acc_o, ys, depth, key=("menger_terrain", k))
        tr.attach(ctx)
        ctx.dispatch(push)
        ctx.wait()
        ctx.set_trace(0, 0, 0, 0)
        acc_g = ctx.read_accum()
        rep = compare.compare(acc_o[ys], tr_o, acc_g[ys], tr.rows(ys), spf)
        print("menger_terrain 1920x1080 pass", k, "engine", engine, rep)
        assert compare.passes(rep), rep
        # continue both from the same accumulator (rows outside ys are the GPU's own)
        acc_g[ys] = acc_o[ys]
        ctx.write_accum(acc_g)
    ctx.close()


def test_batch64_jobs_persistent_route_rows(rt):
    """Seeded jobs of the 64-job batch at their own sizes, all in one batch
    on the persistent route (the route the bench's batch takes), against the
    oracle on two rows of each job."""
    from oracle import compare
    from pathtracer_gb300 import Batch, native

    cie = rt["cie"]
    jobs = []
    for seed in (0, 2, 3, 7, 8):  # 512^2x248, 128^2x137, 1024^2x9, 1024^2x207, 256^2x182
        scene, spec = rt["Scene"].generate(native.PT_GEN_SPHERES, seed)
        jobs.append((seed, scene, spec.width, spec.height, spec.spp, spec.pathLength))
    with Batch(0, pool_slots=1 << 19, max_passes=4096) as b:
        b.set_route(native.PT_BATCH_ROUTE_PERSISTENT)
        tids = []
        for seed, scene, W, H, spp, depth in jobs:
            sid = b.add_scene(scene.pack_ubo(cie), scene.sdf_plugins())
            tid = b.add_target(W, H)
            b.add_pass(sid, tid, scene.push_constants(W, H, spp, spp, spp, depth))
            tids.append(tid)
        b.run()
        assert b.pending() == 0
        st = b.stats()
        assert st["passes_persistent"] == len(jobs) and st["passes_staged"] == 0
        got = [b.read_target(t) for t in tids]
    for (seed, scene, W, H, spp, depth), g in zip(jobs, got):
        ys = _rows(H, 2)
        push = scene.push_constants(W, H, spp, spp, spp, depth)
        acc_o = np.zeros((H, W, 4), np.float32)
        for y in ys:
            compare.run_oracle(scene.pack_ubo(cie), push, compare.plugins_for(scene), accum=acc_o,
                               rect=(0, y, W, y + 1))
        rep = _pixel_report(acc_o[ys], g[ys])
        print(f"batch job seed {seed} {W}x{H}x{spp}", rep)
        assert _pixel_ok(rep), (seed, rep)
