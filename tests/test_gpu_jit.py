"""Scenes whose SDF text is not one of the reference's four snippets: the
text is translated (pt_glsl_translate), compiled with NVRTC into the
megakernel or the wavefront engine's march kernel on the first dispatch of
that engine, and cached.  Parity is against the oracle with a
hand restatement of each snippet in C (oracle/user_sdfs.c) registered for its
slot; criteria as in test_gpu_parity (oracle/compare.py)."""
import json
import os
import time

import numpy as np
import pytest

from conftest import SCENES
from user_snippets import LATTICE, SNIPPETS, SPIRAL, TORUS

pytestmark = pytest.mark.gpu

CUSTOM = {g: (s, m) for g, s, m in SNIPPETS.values()}


@pytest.fixture(scope="module")
def rt(built):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("no CUDA device: -m gpu tests need a GPU")
    from pathtracer_gb300 import Context, Scene, cie_analytic

    return {"Context": Context, "Scene": Scene, "cie": cie_analytic()}


def _scene(rt, sdfs):
    with open(os.path.join(SCENES, "mandelbulb_plane.json")) as f:
        data = json.load(f)
    data["sdf"] = sdfs
    return rt["Scene"].parse(json.dumps(data))


TORUS_SDF = {"position": [-1.3, 0.6, 0.0], "boundingSize": [2.4, 2.4, 2.4], "glsl": TORUS}
LATTICE_SDF = {"position": [1.3, 1.0, 0.0], "boundingSize": [2.0, 2.0, 2.0], "glsl": LATTICE}
BULB_SDF = {"position": [0.0, 1.15, -2.0], "boundingSize": [2.5, 2.5, 2.5], "builtin": "mandelbulb"}
SPIRAL_SDF = {"position": [0.0, 0.45, 1.2], "boundingSize": [2.2, 1.2, 2.2], "glsl": SPIRAL}


@pytest.mark.parametrize("engine", [0, 1])
def test_user_snippets_match_oracle(rt, engine):
    """Three user snippets and a shipped one in one scene, traced per path,
    through the compiled megakernel (engine 0) and the wavefront engine with
    the compiled march kernel (engine 1)."""
    from oracle import compare

    W, H, spf, depth = 64, 48, 4, 6
    scene = _scene(rt, [TORUS_SDF, LATTICE_SDF, BULB_SDF, SPIRAL_SDF])
    ubo = scene.pack_ubo(rt["cie"])
    plugins = compare.plugins_for(scene, custom=CUSTOM)
    with rt["Context"](0) as ctx:
        ctx.set_engine(engine)
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        push = scene.push_constants(W, H, spf, spf, spf, depth)
        acc_o, tr_o = compare.run_oracle(ubo, push, plugins, trace_depth=depth)
        acc_g, tr_g = compare.run_gpu(ctx, push, trace_depth=depth)
        rep = compare.compare(acc_o, tr_o, acc_g, tr_g, spf)
        print(rep)
        assert compare.passes(rep), rep
        # the sdf hits are there: some paths end on each user snippet's materials
        assert np.isfinite(acc_g).all() and acc_g[..., :3].max() > 0


def test_untraced_progressive_matches_oracle(rt):
    """The wavefront engine (the default) with the compiled march kernel over
    three progressive dispatches (running mean), the snippets in other
    slots."""
    from oracle import compare

    W, H, spf, depth = 48, 40, 2, 8
    scene = _scene(rt, [BULB_SDF, LATTICE_SDF, TORUS_SDF])
    ubo = scene.pack_ubo(rt["cie"])
    plugins = compare.plugins_for(scene, custom=CUSTOM)
    acc_o = np.zeros((H, W, 4), np.float32)
    with rt["Context"](0) as ctx:
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        for it in range(3):
            push = scene.push_constants(W, H, spf * (it + 1), spf * (it + 1), spf, depth)
            compare.run_oracle(ubo, push, plugins, accum=acc_o)
            ctx.dispatch(push)
        ctx.wait()
        acc_g = ctx.read_accum()
    rel = np.abs(acc_o - acc_g) / np.maximum(np.maximum(np.abs(acc_o), np.abs(acc_g)), 1e-6)
    frac_bad = float(np.mean(rel[..., :3].max(axis=-1) > 1e-4))
    assert frac_bad < 0.02, frac_bad


def test_engines_agree_bitwise_on_user_snippets(rt):
    """A larger render with several wavefront iterations (rays suspended and
    resumed by the compiled march kernel): both engines give the same bits."""
    W, H, spf, depth = 192, 128, 8, 6
    scene = _scene(rt, [TORUS_SDF, LATTICE_SDF, BULB_SDF])
    out = []
    for engine in (0, 1):
        with rt["Context"](0) as ctx:
            ctx.set_engine(engine)
            ctx.set_march_budget(8)
            ctx.bind(scene, rt["cie"])
            ctx.resize_accum(W, H)
            for it in range(2):
                ctx.dispatch(scene.push_constants(W, H, spf * (it + 1), spf * (it + 1), spf, depth))
            ctx.wait()
            out.append(ctx.read_accum())
            if engine == 1:
                assert ctx.last_iterations() > 8
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


def test_module_is_cached_across_scene_changes(rt):
    """The first dispatch compiles; later ones, also after a scene with only
    shipped snippets was bound in between, reuse the module."""
    W, H = 32, 32
    custom = _scene(rt, [TORUS_SDF])
    plain = rt["Scene"].load(os.path.join(SCENES, "mandelbulb_plane.json"))
    with rt["Context"](0) as ctx:
        ctx.resize_accum(W, H)
        times = []
        for scene in (custom, plain, custom):
            ctx.bind(scene, rt["cie"])
            t0 = time.perf_counter()
            ctx.dispatch(scene.push_constants(W, H, 1, 1, 1, 4))
            ctx.wait()
            times.append(time.perf_counter() - t0)
        print("dispatch seconds (compile, shipped, cached):", times)
        assert times[2] < 0.5 * times[0]
        assert np.isfinite(ctx.read_accum()).all()


def test_compile_error_is_reported_and_context_recovers(rt):
    from pathtracer_gb300 import PathTracerError, native

    W, H = 16, 16
    bad = dict(TORUS_SDF, glsl="float sdf(vec3 p){ return wobble(p); }\nfloat sdfmaterial(vec3 p){ return 1.0; }")
    with rt["Context"](0) as ctx:
        ctx.resize_accum(W, H)
        scene = _scene(rt, [bad])
        ctx.bind(scene, rt["cie"])
        with pytest.raises(PathTracerError) as e:
            ctx.dispatch(scene.push_constants(W, H, 1, 1, 1, 4))
        assert e.value.code == native.PT_ERR_UNSUPPORTED and "wobble" in str(e.value)
        good = rt["Scene"].load(os.path.join(SCENES, "cornell_box.json"))
        ctx.bind(good, rt["cie"])
        ctx.dispatch(good.push_constants(W, H, 1, 1, 1, 4))
        ctx.wait()
        assert np.isfinite(ctx.read_accum()).all()


def test_batch_rejects_run_time_snippets(rt):
    from pathtracer_gb300 import Batch, PathTracerError, native

    scene = _scene(rt, [TORUS_SDF])
    with Batch(0) as b:
        with pytest.raises(PathTracerError) as e:
            b.add_scene(scene.pack_ubo(rt["cie"]), [native.plugin(native.PT_SDF_CUSTOM)])
        assert e.value.code == native.PT_ERR_UNSUPPORTED
    with rt["Context"](0) as ctx:
        with pytest.raises(PathTracerError) as e:
            ctx.set_sdf_plugins([native.plugin(native.PT_SDF_CUSTOM)])
        assert e.value.code == native.PT_ERR_INVALID


def _dispatch_passes(rt, scene, W, H, spf, depth, npass):
    with rt["Context"](0) as ctx:
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        for k in range(npass):
            ctx.dispatch(scene.push_constants(W, H, spf * (k + 1), spf * (k + 1), spf, depth))
        ctx.wait()
        return ctx.read_accum()


def test_batch_renders_user_snippets_like_dispatch(rt):
    """Two scenes with different user snippets in one batch (their slots
    numbered across the batch, one compiled march kernel for all), two
    progressive passes each: the same bits as pt_dispatch."""
    from pathtracer_gb300 import Batch

    W, H, spf, depth = 96, 64, 4, 6
    scenes = [_scene(rt, [TORUS_SDF, LATTICE_SDF, BULB_SDF]), _scene(rt, [SPIRAL_SDF, TORUS_SDF])]
    with Batch(0, pool_slots=1 << 15, max_passes=64) as b:
        ids = [b.add_scene_sources(sc.pack_ubo(rt["cie"]), sc.sdf_sources()) for sc in scenes]
        tgts = [b.add_target(W, H) for _ in scenes]
        for k in range(2):
            for sid, tid, sc in zip(ids, tgts, scenes):
                b.add_pass(sid, tid, sc.push_constants(W, H, spf * (k + 1), spf * (k + 1), spf, depth))
        b.run()
        assert b.stats()["passes_staged"] == 4
        got = [b.read_target(t) for t in tgts]
    for sc, img in zip(scenes, got):
        ref = _dispatch_passes(rt, sc, W, H, spf, depth, 2)
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
        assert img[..., :3].max() > 0


def test_batch_user_snippets_need_the_staged_engine(rt):
    from pathtracer_gb300 import Batch, PathTracerError, native

    W, H = 32, 32
    sc = _scene(rt, [TORUS_SDF])
    with Batch(0, pool_slots=1 << 12, max_passes=16) as b:
        sid = b.add_scene_sources(sc.pack_ubo(rt["cie"]), sc.sdf_sources())
        tid = b.add_target(W, H)
        b.set_route(native.PT_BATCH_ROUTE_PERSISTENT)
        with pytest.raises(PathTracerError) as e:
            b.add_pass(sid, tid, sc.push_constants(W, H, 1, 1, 1, 4))
        assert e.value.code == native.PT_ERR_UNSUPPORTED
        with pytest.raises(PathTracerError) as e:
            b.add_scene_sources(sc.pack_ubo(rt["cie"]), ["struct S { float a; }; float sdf(vec3 p){return 0.0;}"])
        assert e.value.code == native.PT_ERR_UNSUPPORTED


def test_server_serves_user_snippets_batched_and_plain(rt):
    """A resident scene with user snippets: a job's image is the same bits
    through the batched server and the plain path (which sets the texts with
    pt_set_sdfs and compiles its own megakernel)."""
    from pathtracer_gb300 import Server, native

    W, H = 48, 40
    sc = _scene(rt, [TORUS_SDF, SPIRAL_SDF, BULB_SDF])
    push = sc.push_constants(W, H, 1, 1, 1, 6)
    out = []
    for mode in (native.PT_SERVE_BATCHED, native.PT_SERVE_PLAIN):
        with Server(0, mode=mode, keep_images=True, pool_slots=1 << 14, max_passes=64) as s:
            s.add_scene_sources(0, sc.pack_ubo(rt["cie"]), sc.sdf_sources())
            jid = s.submit(Server.job(0, push, 24))
            done = s.drain()
            assert [r.job_id for r in done] == [jid] and done[0].spp == 24
            out.append(s.read_image(jid))
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


@pytest.mark.parametrize("kind", ["mandelbulb", "menger"])
def test_generated_varied_scene_matches_oracle(rt, kind):
    """A PT_GEN_SDF_VARIED job (its SDF as generated GLSL: a mandelbulb of a
    drawn power, or a Menger sponge of drawn levels) through the wavefront
    engine with the compiled march kernel, against the oracle with the C
    restatement of that text."""
    from oracle import compare
    from pathtracer_gb300 import native
    from user_snippets import generated_params, set_generated

    for seed in range(2000, 2100):
        sc, spec = rt["Scene"].generate(native.PT_GEN_SDF_VARIED, seed)
        src = sc.sdf_sources()[0]
        if generated_params(src) and generated_params(src)[0] == kind:
            break
    W, H, spf, depth = 48, 40, 2, 6
    plugins = compare.plugins_for(sc, custom={src: set_generated(src)})
    ubo = sc.pack_ubo(rt["cie"])
    with rt["Context"](0) as ctx:
        ctx.bind(sc, rt["cie"])
        ctx.resize_accum(W, H)
        push = sc.push_constants(W, H, spf, spf, spf, depth)
        acc_o, tr_o = compare.run_oracle(ubo, push, plugins, trace_depth=depth)
        acc_g, tr_g = compare.run_gpu(ctx, push, trace_depth=depth)
    rep = compare.compare(acc_o, tr_o, acc_g, tr_g, spf)
    print(kind, generated_params(src), rep)
    assert compare.passes(rep), rep


@pytest.mark.parametrize("engine", [0, 1])
def test_headline_bulb_scene_matches_oracle(rt, engine):
    """The bench's default scene (scenes/mandelbulb12_plane.json: a power-8
    mandelbulb of 12 iterations, bailout 2, as scene GLSL) at 96x96, 4 spp,
    depth 6, traced per path, through the compiled megakernel (engine 0) and
    the wavefront engine's compiled march kernel (engine 1), against the
    oracle with the C restatement of that text."""
    from oracle import compare

    W, H, spf, depth = 96, 96, 4, 6
    scene = rt["Scene"].load(os.path.join(SCENES, "mandelbulb12_plane.json"))
    ubo = scene.pack_ubo(rt["cie"])
    plugins = compare.plugins_for(scene)
    with rt["Context"](0) as ctx:
        ctx.set_engine(engine)
        ctx.bind(scene, rt["cie"])
        ctx.resize_accum(W, H)
        push = scene.push_constants(W, H, spf, spf, spf, depth)
        acc_o, tr_o = compare.run_oracle(ubo, push, plugins, trace_depth=depth)
        acc_g, tr_g = compare.run_gpu(ctx, push, trace_depth=depth)
    rep = compare.compare(acc_o, tr_o, acc_g, tr_g, spf)
    print(rep)
    assert compare.passes(rep), rep
    assert np.isfinite(acc_g).all() and acc_g[..., :3].max() > 0
