#!/usr/bin/env python3
"""Benchmark: path samples/s on the SDF-fractal scene: a power-8 mandelbulb
(12 iterations, bailout 2; scene GLSL compiled at run time) over a ground
plane under a 5800 K sky dome, 1024x1024, 64 spp, max depth 6
(pathtracer_gb300/scenes/mandelbulb12_plane.json).  --workload mandelbulb
renders the same scene with the shipped mandelbulb snippet (4 iterations,
bailout 16) instead.

One step = one full render of the workload: 1024*1024*64 = 67.1 M camera
paths (4 hero wavelengths each) in ceil(64/spf) dispatches, inputs resident on
the device.  `e2e` repeats the step through the reference-facing C ABI
(pt_render_offscreen) from host buffers: scene packing and upload, the
dispatches, and the read-back of the 16 MiB accumulator each step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
  python bench.py --workload batch64 [--steps K] [--warmup W]
  python bench.py --workload serve [--rate R] [--duration T]
  python bench.py --workload progressive [--spp N] [--ref-spp M]

--workload batch64 is the mixed-job batch: 64 seeded sphere-scene jobs
(pt_scene_generate, seeds 0-63: 128^2-1024^2, 4-256 spp, depth 8; 1.80 G
path samples) rendered as one batch through pt_batch (one pass per job, all
in one wavefront pool), against the same 64 jobs dispatched one after
another through the plain megakernel on one stream.  Both render the same
samples, so the images are bit-identical (checked) and the RMSE is equal.

--workload serve replays a Poisson request stream (70% sphere jobs, 30% SDF
jobs, from a pool of resident scenes with FP64 references) through
pt_server: each job is refined in 8-spp passes until its relative RMSE is at
most the target (or the sample cap), batched (continuous batching under an
HBM budget) and then plain (one job at a time through the megakernel), on
the same trace.  Both arms render the same passes of every job, so each
job's error is identical between them.

--workload progressive is the mixed-SDF config in its reference-expressible
form: menger sponge + sine terrain + a sphere under a sphere light
(pathtracer_gb300/scenes/menger_terrain.json), 1920x1080, rendered in 16-spp
passes to --spp samples per pixel at depth 12, by the staged wavefront engine
and by the plain megakernel, with each pass's relative RMSE against an FP64
reference (--ref-spp samples per pixel, FP32 paths, FP64 sums).

Under torchrun each rank renders its own replica (distinct sample indices,
no exchange): weak scaling.  --impl reference times the reference's own
compute shader on the host cores (all threads): its GLSL built for the CPU
through the repository's translator by oracle/ref_shader.py (made by
__graft_entry__.build() for the default scene; the reference program itself
is Vulkan-only), or the CPU restatement of it (oracle/) where that build is
absent.  The same figure is the `cpu_baseline` of the GPU arm's line.
"""
from __future__ import annotations

import argparse
import faulthandler
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# The single-scene workloads: scene file and workload name (at the default
# 1024x1024, 64 spp, depth 6).
RENDER_WORKLOADS = {
    # power-8 mandelbulb, 12 iterations, bailout 2, as scene GLSL compiled at run time
    "mandelbulb12": ("mandelbulb12_plane.json", "mandelbulb12_plane_1024x1024_64spp_depth6"),
    # the shipped mandelbulb snippet (power 8, 4 iterations, bailout 16)
    "mandelbulb": ("mandelbulb_plane.json", "mandelbulb_plane_1024x1024_64spp_depth6"),
    # the SDF-fractal configuration in its full form: the same fractal with a smooth bulb spectrum, a flat
    # 0.5 plane, a 5800 K environment sky, a 256-step march capped at distance 50, 380-780 nm and the
    # analytic CIE fit (scene extensions the reference's shader does not have)
    "mandelbulb12_full": ("mandelbulb12_plane_full.json", "mandelbulb12_plane_full_1024x1024_64spp_depth6"),
}


def scene_path(workload):
    return os.path.join(ROOT, "pathtracer_gb300", "scenes", RENDER_WORKLOADS[workload][0])


def workload_name(args):
    name = RENDER_WORKLOADS[args.workload][1]
    if (args.res, args.spp, args.depth) != (1024, 64, 6):
        name = name.replace("1024x1024_64spp_depth6", f"{args.res}x{args.res}_{args.spp}spp_depth{args.depth}")
    return name

METRIC = "path_samples_per_s"
UNIT = "path samples/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--res", type=int, default=1024)
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--spf", type=int, default=64, help="samples per dispatch")
    ap.add_argument("--depth", type=int, default=6)
    ap.add_argument("--cpu-rows", type=int, default=384, help="rows in the CPU baseline sample (about 10 s on 16 cores)")
    ap.add_argument("--engine", default="wavefront", choices=["wavefront", "megakernel"])
    ap.add_argument("--compare-engines", type=int, default=1, help="also time the other engine (1 step)")
    ap.add_argument("--pool", type=int, default=0, help="wavefront path slots (0: library default)")
    ap.add_argument("--wf-engines", type=int, default=0,
                    help="wavefront engines a large dispatch is split between (1..4; 0: library default)")
    ap.add_argument("--budget", type=int, default=0, help="wavefront march steps per launch (0: default)")
    ap.add_argument("--refill", type=int, default=0, help="wavefront march refill threshold (0: default)")
    ap.add_argument("--drain", type=int, default=-1, help="wavefront march drain lanes (-1: default)")
    ap.add_argument("--blocks", type=int, default=0, help="wavefront stage blocks per SM (0: default)")
    ap.add_argument("--inner", type=int, default=0, help="wavefront SDF evaluations per march lane between refills (0: default)")
    ap.add_argument("--fp-contract", type=int, default=0,
                    help="FMA contraction in run-time compiled kernels (1: faster, not bit-exact; 0: the shader's rounding)")
    ap.add_argument("--autotune", type=int, default=1,
                    help="rounds of pt_autotune_wavefront on a 1024x1024x16spp dispatch before timing (0: off)")
    ap.add_argument("--workload", default="mandelbulb12",
                    choices=["mandelbulb12", "mandelbulb", "mandelbulb12_full", "batch64", "serve", "progressive"])
    ap.add_argument("--pass-spp", type=int, default=16, help="progressive: samples per pixel per pass")
    ap.add_argument("--form", default="reference", choices=["reference", "full"],
                    help="progressive: the scene in the reference's method, or in its full form (fBm terrain "
                         "compiled at run time, a dispersive glass sphere, sky; menger_terrain_full.json)")
    ap.add_argument("--rate", type=float, default=2.0, help="serve: Poisson arrivals per second")
    ap.add_argument("--duration", type=float, default=30.0, help="serve: seconds of arrivals")
    ap.add_argument("--target-rmse", type=float, default=0.02, help="serve: relative RMSE target per job")
    ap.add_argument("--max-spp", type=int, default=512, help="serve: sample cap per job")
    ap.add_argument("--ref-spp", type=int, default=1024, help="serve: FP64 reference samples per pixel")
    ap.add_argument("--pool-scenes", type=int, default=16, help="serve: scenes in the request pool")
    ap.add_argument("--iters-per-poll", type=int, default=4, help="serve: engine iterations per server poll")
    ap.add_argument("--passes-in-flight", type=int, default=1, help="serve: passes in flight per job")
    ap.add_argument("--serve-spheres", default="full", choices=["full", "reference"],
                    help="serve: sphere jobs with real conductor mirrors and Cauchy dielectrics (PT_GEN_SPHERES_FULL, "
                         "the configuration's materials) or mapped to the reference's Lambertian spectra")
    ap.add_argument("--ref-paths", default="fp32", choices=["fp32", "fp64"],
                    help="serve: references of FP32 paths summed in double, or traced in double (slow)")
    ap.add_argument("--sdf-scenes", default="varied", choices=["varied", "shipped"],
                    help="serve: SDF scenes with drawn powers/levels (GLSL compiled at run time) or the shipped snippets")
    ap.add_argument("--burst", type=int, default=0,
                    help="serve: N requests all arriving at t=0 instead of the Poisson stream (saturates both arms)")
    ap.add_argument("--jobs", type=int, default=64, help="batch64: jobs per batch")
    ap.add_argument("--serve-jobs", type=int, default=16,
                    help="render workloads: jobs of the saturated serve burst reported in the line's `serve` object "
                         "(batched-served vs plain at equal per-job RMSE; 0: off; N=1 only)")
    ap.add_argument("--route", default="auto", choices=["auto", "staged", "persistent"],
                    help="batch64: engine route of the passes")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def fp32_peak_tflops(peaks):
    """Nominal FP32 FMA rate at the measured maximum SM clock: SMs x 128 lanes x 2."""
    import torch

    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    return sms * 128 * 2 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12


# DRAM bytes per launch of each stage kernel (dram__bytes_read.sum +
# dram__bytes_write.sum) in the steady state of the workload's scene, keyed
# by workload and path-pool size; the other knobs were the library defaults
# (one engine).  Each comes from one small-case ncu capture of two launches
# per stage with the pool full
# (profiles/wf_stages_mandelbulb12_1024x1024_16spp_pool2e22.md):
# per launch a stage moves the state of the rays in its queues, which a full
# pool of the same size bounds the same way at the full image size (the last
# iterations of a dispatch, with the pool draining, move less).  At 2^22
# slots gen had nothing to start in the captured launches: no figure.
# Other settings report null.
STAGE_TRAFFIC_BYTES = {
    ("mandelbulb12_plane_1024x1024_64spp_depth6", 1 << 20): {"march": 297.99e6, "shade": 351.92e6, "gen": 36.48e6},
    ("mandelbulb12_plane_1024x1024_64spp_depth6", 1 << 21): {"march": 809.99e6, "shade": 949.24e6, "gen": 78.17e6},
    ("mandelbulb12_plane_1024x1024_64spp_depth6", 1 << 22): {"march": 1183.41e6, "shade": 1504.67e6},
}
# The library's default wavefront knobs.
DEFAULT_TUNING = {"pool_slots": 1 << 22, "march_budget": 64, "refill_min": 2, "drain_lanes": 24, "blocks_per_sm": 4,
                  "march_inner": 6}


def traffic_key(workload, spf, tuning):
    """The STAGE_TRAFFIC_BYTES key of a run, or None when its knobs differ
    from every capture's in a way that changes what one launch moves.  The
    march budget only sets how many steps a ray takes per launch (each
    queued ray's state is read and written once per launch either way), so
    it is not part of the key; pool size, thresholds and blocks are."""
    skip = ("pool_slots", "march_budget")
    rest = {k: v for k, v in tuning.items() if k not in skip}
    if spf != 64 or rest != {k: v for k, v in DEFAULT_TUNING.items() if k not in skip}:
        return None
    return (workload, tuning["pool_slots"])


def stage_roofline(ctx, run_step, samples, workload, peaks, peak_kind, tkey=None):
    """One extra step with per-stage CUDA events: each stage kernel's device
    time and, from the committed work model, its achieved FP32 rate, and for
    a captured configuration its DRAM rate (captured bytes per launch over
    the live time per launch) against the measured HBM bandwidth; the
    roofline object is the march kernel's (the dominant one)."""
    from pathtracer_gb300 import workmodel

    ctx.set_stage_timing(True)
    run_step()
    ctx.wait()
    ms, iters = ctx.stage_times()
    ctx.set_stage_timing(False)
    ops = workmodel.fp32_ops_per_sample(workmodel.load(workload)["per_sample"])
    total_ms = sum(ms.values())
    peak = fp32_peak_tflops(peaks)
    traffic = STAGE_TRAFFIC_BYTES.get(tkey, {})
    hbm = peaks.get("hbm_gbs")
    stages = {}
    for st in ("isect", "march", "shade", "gen", "book"):
        secs = ms[st] / 1000.0
        work = ops.get(st, 0.0) * samples
        per_launch = ms[st] / iters if iters else None
        gbs = traffic[st] / (per_launch / 1000.0) / 1e9 if st in traffic and per_launch else None
        stages[st] = {"ms": ms[st], "share": ms[st] / total_ms if total_ms else None,
                      "ms_per_launch": per_launch,
                      "fp32_tflops": (work / secs / 1e12) if secs and work else None,
                      "dram_bytes_per_launch": traffic.get(st), "dram_gbs": gbs,
                      "dram_frac": (gbs / hbm) if gbs and hbm else None}
    march = stages["march"]
    roof = {"bound": "fp32", "kernel": "wf_march", "achieved": march["fp32_tflops"], "peak": peak,
            "unit": "TFLOP/s", "frac": (march["fp32_tflops"] or 0.0) / peak,
            "traffic": traffic.get("march"),
            "work_per_sample": ops["march"], "launches": iters,
            "note": f"peak: nominal FP32 FMA rate (SMs x 128 x 2) at the measured max SM clock ({peak_kind} peaks "
                    "hold no FP32 figure); achieved: hand-counted FP32 operations of the march stage's events "
                    "(pathtracer_gb300/workmodel.py, counts per sample from tests/golden/work_*.json) over the "
                    "summed device time of its launches in one step timed with per-stage CUDA events (one engine, "
                    "its kernels one at a time); traffic: "
                    "DRAM bytes per launch from one small-case ncu capture of this scene with the pool full (profiles/)"}
    return roof, stages, ops


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def reference_cpu(scene):
    """The reference's own shader built for the CPU for this scene's SDF texts
    (oracle/_ref, made by __graft_entry__.build()), or None where it was not
    built (then the oracle port stands in)."""
    import ctypes

    from oracle import ref_shader

    texts = scene.sdf_sources()
    if any(t.startswith("builtin:") for t in texts):
        return None  # a shipped plug-in named by key: no snippet text to splice
    try:
        lib = ctypes.CDLL(ref_shader.build_scene(None, texts))
    except (FileNotFoundError, OSError, subprocess.CalledProcessError):
        return None
    lib.refsc_bind.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.refsc_render_rows.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    return lib


def cpu_baseline(args, W, H, spf_total, nthreads):
    """Path samples/s on the host cores over a stratified sample of rows: the
    reference's own shader built for the CPU where it was built ("reference":
    OpenMP over the rows' pixels), else the oracle (the CPU restatement,
    "port": one row per call, rows spread over `nthreads` host threads).
    The scene is read, packed and given its CIE table by the oracle's own
    restatement of the reference host (oracle/pack.py): no library of the
    product is loaded on this path."""
    import ctypes

    from oracle import oracle as _o
    from oracle import pack

    scene = pack.load_scene(scene_path(args.workload))
    ubo = scene.pack_ubo(pack.cie_analytic())
    ext = scene.pack_ext()
    push = scene.push_constants(W, H, spf_total, spf_total, spf_total, args.depth)
    rows = max(1, min(args.cpu_rows, H))
    stride = H // rows
    # the reference's own shader has none of the full-form extensions: such scenes run on the oracle port
    ref = reference_cpu(scene) if not ext.flags else None
    kind = "reference" if ref is not None else "port"
    plugins = None if ref is not None else _o.plugins_for_sources(scene.sdf_sources())
    ys = np.array([r * stride + stride // 2 for r in range(rows)], np.int32)
    acc = np.zeros((H, W, 4), np.float32)
    out = np.zeros((rows, W, 3), np.float32)
    t0 = time.perf_counter()
    if ref is not None:
        ref.refsc_bind(ubo.ctypes.data, ctypes.addressof(push))
        ref.refsc_render_rows(ys.ctypes.data, rows, out.ctypes.data, nthreads)
    else:
        from concurrent.futures import ThreadPoolExecutor

        def one_row(y):  # ctypes releases the GIL: rows run in parallel
            _o.dispatch(ubo, push, plugins, acc, rect=(0, int(y), W, int(y) + 1), nthreads=1, ext=ext)

        with ThreadPoolExecutor(max_workers=nthreads) as ex:
            list(ex.map(one_row, ys))
    dt = time.perf_counter() - t0
    samples = rows * W * spf_total
    return samples / dt, samples, dt, rows, kind


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from oracle import oracle as _o

    _o.build()
    W = H = args.res
    nthreads = os.cpu_count() or 1
    vals = []
    for i in range(args.warmup + args.steps):
        v, samples, dt, rows, kind = cpu_baseline(args, W, H, args.spp, nthreads)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.mean(vals)
    sample = f"{rows} evenly spaced rows of {W}x{H} at {args.spp} spp ({samples} paths per step)"
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * samples / value, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": workload_name(args), "resolution": [W, H], "spp": args.spp, "max_depth": args.depth},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0

BATCH_WORKLOAD = "batch64_spheres_seeds0-63_res128-1024_spp4-256_depth8"


def make_jobs(n, first_seed, kind=None):
    """n seeded jobs: (scene, spec, packed ubo, plug-ins)."""
    from pathtracer_gb300 import Scene, cie_analytic, native

    cie = cie_analytic()
    out = []
    for seed in range(first_seed, first_seed + n):
        scene, spec = Scene.generate(native.PT_GEN_SPHERES if kind is None else kind, seed)
        out.append((scene, spec, scene.pack_ubo(cie), scene.sdf_plugins()))
    return out, cie


def pctl(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = min(len(xs) - 1, max(0, int(np.ceil(q / 100.0 * len(xs))) - 1))
    return xs[k]


def batch_cpu_baseline(jobs, nthreads, rows_per_job=2, njobs=16):
    """Rows of the first jobs on the host cores: the reference's own shader
    built for the CPU (the jobs have no SDFs; kind "reference", OpenMP over
    each job's rows' pixels) where it was built, else the oracle (one row per
    call, the rows spread over `nthreads` host threads; kind "port")."""
    import ctypes
    from concurrent.futures import ThreadPoolExecutor

    from oracle import compare

    ref = reference_cpu(jobs[0][0]) if jobs and not jobs[0][0].sdf_sources() else None
    work = []
    for scene, spec, ubo, plugins in jobs[:njobs]:
        W, H = spec.width, spec.height
        push = scene.push_constants(W, H, spec.spp, spec.spp, spec.spp, spec.pathLength)
        ys = np.array([(2 * r + 1) * H // (2 * rows_per_job) for r in range(rows_per_job)], np.int32)
        work.append((scene, ubo, push, W, H, ys, rows_per_job * W * spec.spp))

    def one_row(w, y):  # ctypes releases the GIL: rows run in parallel
        scene, ubo, push, W, H, _, _ = w
        acc = np.zeros((H, W, 4), np.float32)
        compare.run_oracle(ubo, push, compare.plugins_for(scene), accum=acc, rect=(0, int(y), W, int(y) + 1),
                           nthreads=1)

    t0 = time.perf_counter()
    if ref is not None:
        for scene, ubo, push, W, H, ys, _ in work:
            out = np.zeros((len(ys), W, 3), np.float32)
            ref.refsc_bind(ubo.ctypes.data, ctypes.addressof(push))
            ref.refsc_render_rows(ys.ctypes.data, len(ys), out.ctypes.data, nthreads)
    else:
        with ThreadPoolExecutor(max_workers=nthreads) as ex:
            list(ex.map(lambda a: one_row(*a), [(w, y) for w in work for y in w[5]]))
    dt = time.perf_counter() - t0
    samples = sum(w[6] for w in work)
    return samples / dt, samples, dt, ("reference" if ref is not None else "port")


def batch_roofline(samples, secs, peaks, peak_kind):
    """FP32 roofline of the persistent path kernel over a batched step (it is
    nearly all of the step's device time)."""
    from pathtracer_gb300 import workmodel

    ops = workmodel.fp32_ops_per_sample(workmodel.load("batch64_spheres")["per_sample"])
    peak = fp32_peak_tflops(peaks)
    ach = ops["total"] * samples / secs / 1e12
    return {"bound": "fp32", "kernel": "wf_persist", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
            "frac": ach / peak, "traffic": None, "work_per_sample": ops["total"],
            "note": f"peak: nominal FP32 FMA rate at the measured max SM clock ({peak_kind}); achieved: work-model "
                    "FP32 operations of the whole step over the step's device time"}


def run_batch(args, rank, world):
    """The mixed-job batch: batched wavefront vs the plain megakernel, serial."""
    import torch

    from pathtracer_gb300 import Batch, Context, build, native

    build.build()
    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", "0")))
    local = torch.cuda.current_device()
    from pathtracer_gb300 import replicas

    jobs, cie = make_jobs(args.jobs, replicas.job_seeds(rank, args.jobs).start)
    pushes = [sc.push_constants(sp.width, sp.height, sp.spp, sp.spp, sp.spp, sp.pathLength) for sc, sp, _, _ in jobs]
    samples = sum(sp.width * sp.height * sp.spp for _, sp, _, _ in jobs)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    b = Batch(local, pool_slots=args.pool or (1 << 19), max_passes=4096)
    b.set_route({"auto": native.PT_BATCH_ROUTE_AUTO, "staged": native.PT_BATCH_ROUTE_STAGED,
                 "persistent": native.PT_BATCH_ROUTE_PERSISTENT}[args.route])
    if args.budget:
        b.set_march_budget(args.budget)
    sids = [b.add_scene(ubo, plugins) for _, _, ubo, plugins in jobs]
    tids = [b.add_target(sp.width, sp.height) for _, sp, _, _ in jobs]
    bstream = torch.cuda.ExternalStream(b.stream())

    def batched_step():
        with torch.cuda.stream(bstream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(bstream)
        st0 = b.stats()
        it0, k0 = st0["iterations"], st0["kernel_launches"]
        for sid, tid, push in zip(sids, tids, pushes):
            b.add_pass(sid, tid, push)
        lat = {}
        chunk = 16
        while b.pending():
            for pid in b.step(chunk):
                lat[pid] = time.perf_counter() - t0
        e1.record(bstream)
        e1.synchronize()
        st1 = b.stats()
        return (e0.elapsed_time(e1) / 1000.0, list(lat.values()), st1["iterations"] - it0,
                st1["kernel_launches"] - k0)

    for _ in range(args.warmup):
        batched_step()
    bt, blat, biters, blaunch = [], [], [], []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            secs, lat, iters, launches = batched_step()
            bt.append(secs)
            blat += lat
            biters.append(iters)
            blaunch.append(launches)
    b_secs = statistics.mean(bt)
    batched_images = [b.read_target(t) for t in tids[:8]]

    # The plain megakernel: one context per job (scene bound, accumulator
    # resident), every dispatch on one stream, one after another.
    ctxs = []
    for scene, spec, _, _ in jobs:
        c = Context(local)
        c.set_engine(native.PT_ENGINE_MEGAKERNEL)
        c.bind(scene, cie)
        c.resize_accum(spec.width, spec.height)
        ctxs.append(c)
    shared = ctxs[0].stream()
    for c in ctxs:
        c.set_stream(shared)
    pstream = torch.cuda.ExternalStream(shared)

    def plain_step():
        with torch.cuda.stream(pstream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e0.record(pstream)
        evs = []
        for c, push in zip(ctxs, pushes):
            c.dispatch(push)
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(pstream)
            evs.append(ev)
        evs[-1].synchronize()
        return e0.elapsed_time(evs[-1]) / 1000.0, [e0.elapsed_time(ev) / 1000.0 for ev in evs]

    plain_steps = max(1, min(args.steps, 2))
    plain_step()
    pt_, plat = [], []
    for _ in range(plain_steps):
        secs, lat = plain_step()
        pt_.append(secs)
        plat += lat
    p_secs = statistics.mean(pt_)
    identical = all(np.array_equal(img.view(np.uint32), c.read_accum().view(np.uint32))
                    for img, c in zip(batched_images, ctxs))
    # The shared stream belongs to ctxs[0]: hand every context its own stream
    # back before any is destroyed.
    for c in ctxs:
        c.set_stream(None)
    for c in ctxs:
        c.close()

    # End to end through the C ABI from host buffers: scene upload, targets,
    # passes, run, read-back of every image, release.
    e2e = []
    h2d = d2h = 0
    for _ in range(max(1, min(args.steps, 2))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = [b.add_scene(ubo, plugins) for _, _, ubo, plugins in jobs]
        t2 = [b.add_target(sp.width, sp.height) for _, sp, _, _ in jobs]
        for sid, tid, push in zip(s2, t2, pushes):
            b.add_pass(sid, tid, push)
        b.run()
        imgs = [b.read_target(t) for t in t2]
        e2e.append(time.perf_counter() - t0)
        h2d = native.UBO_FLOATS * 4 * len(jobs)
        d2h = sum(im.nbytes for im in imgs)
        for sid, tid in zip(s2, t2):
            b.release_target(tid)
            b.release_scene(sid)
    e2e_secs = statistics.median(e2e)
    st = b.stats()
    b.close()

    b_secs, e2e_secs = replicas.max_over_ranks([b_secs, e2e_secs])
    value = samples * world / b_secs
    peaks, peak_kind = measured_peaks()
    iters = statistics.mean(biters)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * b_secs, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
        "config": {"workload": BATCH_WORKLOAD, "jobs": len(jobs), "samples_per_step": samples,
                   "passes_per_job": 1, "route": args.route, "passes_staged": st["passes_staged"],
                   "passes_persistent": st["passes_persistent"], "l2": "flushed between timed steps (256 MiB write)",
                   "parallelism": f"replicas x{world}", "wavefront_pool": st["pool_slots"],
                   "march_budget": args.budget or None},
        "e2e": {"value": samples * world / e2e_secs, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "batched": {"value": samples / b_secs, "ms_per_step": 1000.0 * b_secs,
                    "job_latency_s": {"p50": pctl(blat, 50), "p99": pctl(blat, 99)},
                    "iterations_per_step": iters},
        "plain_megakernel_serial": {"value": samples / p_secs, "ms_per_step": 1000.0 * p_secs,
                                    "job_latency_s": {"p50": pctl(plat, 50), "p99": pctl(plat, 99)}},
        "speedup_vs_plain": p_secs / b_secs,
        "results_identical_to_plain": identical,
        "gpu_launches": int(sum(blaunch)),  # the library's count (pt_batch_info.kernel_launches)
        "roofline": batch_roofline(samples, b_secs, peaks, peak_kind),
        "clocks": clk.summary(),
    }
    if rank == 0:
        nthreads = os.cpu_count() or 1
        v, n, dt, kind = batch_cpu_baseline(jobs, nthreads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": nthreads, "kind": kind,
                                "sample": f"2 rows of each of the first 16 jobs at their spp ({n} paths, {dt:.1f} s)"}
        print(json.dumps(line), flush=True)
    return 0


SERVE_WORKLOAD = "serve_poisson_70pct_spheres_30pct_sdf_rmse2pct_8spp_passes"


def serve_measure(opts, local, rank):
    """A request stream through pt_server, batched then plain on the same
    trace: pool of opts.pool_scenes generated scenes (70 % sphere jobs, 30 %
    SDF jobs) with FP64 references, jobs refined in 8-spp passes until their
    relative RMSE is at most opts.target_rmse (or opts.max_spp).  Returns the
    per-arm figures and the comparison."""
    from pathtracer_gb300 import Scene, Server, cie_analytic, native

    cie = cie_analytic()
    n_sdf = max(1, round(0.3 * opts.pool_scenes))
    n_sph = opts.pool_scenes - n_sdf
    pool = []
    sdf_kind = native.PT_GEN_SDF_VARIED if opts.sdf_scenes == "varied" else native.PT_GEN_SDF
    sph_kind = native.PT_GEN_SPHERES_FULL if opts.serve_spheres == "full" else native.PT_GEN_SPHERES
    for k in range(opts.pool_scenes):
        kind, seed = (sph_kind, 1000 + k) if k < n_sph else (sdf_kind, 2000 + k)
        sc, spec = Scene.generate(kind, seed + 100000 * rank)
        push = sc.push_constants(spec.width, spec.height, 1, 1, 1, spec.pathLength)
        pool.append((kind, sc, spec, push))
    srv = Server(local, mode=native.PT_SERVE_BATCHED, spp_per_pass=8, hbm_budget=64 << 30,
                 pool_slots=opts.pool or (1 << 21), iterations_per_poll=opts.iters_per_poll,
                 passes_in_flight=opts.passes_in_flight, fp64_paths=opts.ref_paths == "fp64")
    t0 = time.perf_counter()
    for key, (kind, sc, spec, push) in enumerate(pool):
        # SDFs as text: generated snippets are compiled at run time (the
        # batch's march kernel, before its first step: here)
        srv.add_scene_sources(key, sc.pack_ubo(cie), sc.sdf_sources())
        srv.set_scene_ext(key, sc.pack_ext())  # mirrors and dielectrics of the full-form sphere jobs
        srv.render_reference(key, push, opts.ref_spp, 32)
    ref_secs = time.perf_counter() - t0

    rng = np.random.default_rng(7 + rank)
    arrivals, reqs = [], []
    t = 0.0 if opts.burst else rng.exponential(1.0 / opts.rate)
    while (len(reqs) < opts.burst) if opts.burst else (t < opts.duration):
        key = int(rng.integers(0, n_sph)) if rng.random() < 0.7 else n_sph + int(rng.integers(0, n_sdf))
        reqs.append(Server.job(key, pool[key][3], opts.max_spp, opts.target_rmse))
        arrivals.append(float(t))
        if not opts.burst:
            t += rng.exponential(1.0 / opts.rate)

    kinds = [pool[r.scene_key][0] for r in reqs]

    def by_kind(res, serial):
        """Jobs and samples per scene kind; on the serial plain path also the
        seconds spent on each kind (admission to completion)."""
        out = {}
        for name, kv in (("spheres", sph_kind), ("sdf", sdf_kind)):
            sel = [r for r, k in zip(res, kinds) if k == kv]
            out[name] = {"jobs": len(sel), "samples": sum(r.samples for r in sel)}
            if serial:
                secs = sum(r.t_done - r.t_admit for r in sel)
                out[name].update({"seconds": secs, "path_samples_per_s": out[name]["samples"] / secs if secs else None})
        return out

    def arm(mode):
        srv.set_mode(mode)
        with ClockSampler(local) as clk:
            res = srv.run_trace(reqs, arrivals)
        lat = [r.t_done - r.t_submit for r in res]
        samples = sum(r.samples for r in res)
        makespan = max(r.t_done for r in res) - min(arrivals)
        return res, {"jobs": len(res), "samples": samples, "makespan_s": makespan,
                     "by_kind": by_kind(res, mode == native.PT_SERVE_PLAIN),
                     "path_samples_per_s": samples / makespan,
                     "time_to_target_s": {"p50": pctl(lat, 50), "p99": pctl(lat, 99), "mean": statistics.mean(lat)},
                     "queue_wait_s": {"p50": pctl([r.t_admit - r.t_submit for r in res], 50),
                                      "p99": pctl([r.t_admit - r.t_submit for r in res], 99)},
                     "clocks": clk.summary()}

    res_b, batched = arm(native.PT_SERVE_BATCHED)
    st = srv.stats()
    # The plain path compiles its megakernel for each scene's snippets on the
    # scene's first job: one short untimed job per scene first.
    srv.set_mode(native.PT_SERVE_PLAIN)
    srv.run_trace([Server.job(k, pool[k][3], 8) for k in range(len(pool))], [0.0] * len(pool))
    res_p, plain = arm(native.PT_SERVE_PLAIN)
    identical = all((a.spp, a.rmse) == (b.spp, b.rmse) for a, b in zip(res_b, res_p))
    reached = sum(1 for r in res_b if r.rmse <= opts.target_rmse) / max(1, len(res_b))
    per_job = [r.samples for r in res_b]
    srv.close()
    span = opts.duration if not opts.burst else None
    mean_job = sum(per_job) / max(1, len(per_job))
    return {"batched": batched, "plain_megakernel_serial": plain,
            "throughput_speedup_vs_plain": batched["path_samples_per_s"] / plain["path_samples_per_s"],
            "p50_speedup_vs_plain": plain["time_to_target_s"]["p50"] / batched["time_to_target_s"]["p50"],
            "p99_speedup_vs_plain": plain["time_to_target_s"]["p99"] / batched["time_to_target_s"]["p99"],
            "rmse_identical_per_job": identical, "reached_target_fraction": reached,
            "final_rmse_per_job": [r.rmse for r in res_b], "spp_per_job": [r.spp for r in res_b],
            "offered_samples_per_s": sum(per_job) / span if span else None, "mean_samples_per_job": mean_job,
            "offered_at_200_jobs_per_s": mean_job * 200.0,
            "saturates_at_200_jobs_per_s": mean_job * 200.0 > batched["path_samples_per_s"],
            "reference_render_s": ref_secs, "hbm_peak_bytes": st["bytes_peak"],
            "resident_bytes": st["resident_bytes"]}


def serve_config(opts):
    return {"workload": SERVE_WORKLOAD + ("_full_spheres" if opts.serve_spheres == "full" else "")
            + ("_varied_sdf" if opts.sdf_scenes == "varied" else "")
            + ("_burst" if opts.burst else ""), "sdf_scenes": opts.sdf_scenes,
            "rate_jobs_per_s": None if opts.burst else opts.rate,
            "duration_s": None if opts.burst else opts.duration, "burst_jobs": opts.burst or None,
            "target_rmse": opts.target_rmse, "max_spp": opts.max_spp, "spp_per_pass": 8,
            "reference_spp": opts.ref_spp,
            "reference": "FP64 paths" if opts.ref_paths == "fp64" else "FP32 paths summed in FP64",
            "sphere_jobs": ("full form: Lambertian spectra, conductor mirrors, Cauchy dielectrics"
                            if opts.serve_spheres == "full" else "materials mapped to Lambertian spectra"),
            "pool_scenes": opts.pool_scenes, "hbm_budget_gib": 64,
            "iterations_per_poll": opts.iters_per_poll, "passes_in_flight": opts.passes_in_flight}


def run_serve(args, rank, world):
    """Poisson request stream through pt_server, batched vs plain."""
    import torch

    from pathtracer_gb300 import build, replicas

    build.build()
    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", "0")))
    local = torch.cuda.current_device()
    serve = serve_measure(args, local, rank)
    batched = serve["batched"]
    makespan = replicas.max_over_ranks([batched["makespan_s"]])[0]
    value = replicas.whole_job_rate(batched["samples"], world, makespan)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": 1, "warmup": 0,
        "ms_per_step": 1000.0 * makespan, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, Poisson arrivals)",
        "config": {**serve_config(args), "parallelism": f"replicas x{world}"},
        "serve": serve,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "note": "requests carry no host buffers; scenes are resident"},
        "gpu_launches": None,
        "roofline": None,
        "clocks": batched["clocks"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


PROGRESSIVE_WORKLOAD = "menger_terrain_1920x1080_16spp_passes_depth12"
PROGRESSIVE_SCENES = {"reference": "menger_terrain.json", "full": "menger_terrain_full.json"}


def run_progressive(args, rank, world):
    """Progressive rendering in 16-spp passes, wavefront vs plain, error per pass."""
    import torch

    from pathtracer_gb300 import Batch, Context, Scene, build, cie_analytic, native, replicas

    build.build()
    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", "0")))
    local = torch.cuda.current_device()
    W, H, depth, spf = 1920, 1080, 12, args.pass_spp
    npass = max(1, args.spp // spf)
    scene = Scene.load(os.path.join(ROOT, "pathtracer_gb300", "scenes", PROGRESSIVE_SCENES[args.form]))
    cie = cie_analytic()
    ubo = scene.pack_ubo(cie)
    base = replicas.frame_base(rank, 1, 1, args.spp)  # distinct samples per replica

    b = Batch(local, pool_slots=args.pool or (1 << 22), max_passes=4096)
    b.set_route(native.PT_BATCH_ROUTE_STAGED)
    if args.wf_engines:
        b.set_wavefront_engines(min(args.wf_engines, 2))
    # the scene's SDFs as text: shipped snippets select plug-ins, the full
    # form's fBm terrain is compiled at run time
    sid = b.add_scene_sources(ubo, scene.sdf_sources())
    b.set_scene_ext(sid, scene.pack_ext())
    ref = b.add_target(W, H, native.PT_TARGET_FP64)
    t0 = time.perf_counter()
    for k in range(max(1, args.ref_spp // 64)):
        b.add_pass(sid, ref, scene.push_constants(W, H, (1 << 30) + (k + 1) * 64, 64, 64, depth))
        if b.pending() >= 64:
            b.run()
    b.run()
    ref_secs = time.perf_counter() - t0

    def push_k(k):
        # frame = currentSamples = k*spf: the reference's offscreen loop
        return scene.push_constants(W, H, k * spf, k * spf, spf, depth)

    # Wavefront: every pass through the batch, error checked after each.
    stream = torch.cuda.ExternalStream(b.stream())
    tgt = b.add_target(W, H)
    wf_err, wf_secs = [], 0.0
    with ClockSampler(local) as clk:
        for k in range(1, npass + 1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            b.add_pass(sid, tgt, push_k(k))
            b.run()
            e1.record(stream)
            e1.synchronize()
            wf_secs += e0.elapsed_time(e1) / 1000.0
            wf_err.append(b.rmse(tgt, ref))
    wf_img = b.read_target(tgt)

    # Plain megakernel: the same passes through pt_dispatch.
    ctx = Context(local)
    ctx.set_engine(native.PT_ENGINE_MEGAKERNEL)
    ctx.bind(scene, cie)
    ctx.resize_accum(W, H)
    # SDF text compiled at run time: the megakernel is compiled on its first
    # dispatch, here, outside the timed passes (the batch compiled its march
    # kernel for the reference render above)
    ctx.dispatch(scene.push_constants(W, H, 1, 1, 1, depth))
    ctx.wait()
    ctx.resize_accum(W, H)
    cstream = torch.cuda.ExternalStream(ctx.stream())
    pl_err, pl_secs = [], 0.0
    for k in range(1, npass + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(cstream)
        ctx.dispatch(push_k(k))
        e1.record(cstream)
        e1.synchronize()
        pl_secs += e0.elapsed_time(e1) / 1000.0
        pl_err.append(b.rmse_image(ctx.accum_device_ptr(), W, H, ref))
    identical = bool(np.array_equal(ctx.read_accum().view(np.uint32), wf_img.view(np.uint32)))
    ctx.close()
    b.close()

    samples = W * H * spf * npass
    wf_secs, pl_secs = replicas.max_over_ranks([wf_secs, pl_secs])
    value = replicas.whole_job_rate(samples, world, wf_secs)
    peaks, peak_kind = measured_peaks()
    every = max(1, npass // 8)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": npass, "warmup": 0,
        "ms_per_step": 1000.0 * wf_secs / npass, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": PROGRESSIVE_WORKLOAD + ("_full" if args.form == "full" else ""), "resolution": [W, H],
                   "spp": spf * npass, "pass_spp": spf,
                   "max_depth": depth, "reference_spp": args.ref_spp, "parallelism": f"replicas x{world}"},
        "progressive": {"wavefront": {"value": samples / wf_secs, "seconds": wf_secs},
                        "plain_megakernel": {"value": samples / pl_secs, "seconds": pl_secs},
                        "speedup_vs_plain": pl_secs / wf_secs, "results_identical": identical,
                        "rmse_per_pass": {str((k + 1) * spf): wf_err[k] for k in range(every - 1, npass, every)},
                        "rmse_identical_per_pass": wf_err == pl_err, "final_rmse": wf_err[-1],
                        "reference_render_s": ref_secs},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "note": "passes on a resident scene; each pass's error is reduced on the device"},
        "gpu_launches": None, "roofline": None, "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    faulthandler.enable()
    args = parse_args()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            import torch

            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    if args.workload in ("batch64", "serve", "progressive"):
        rc = {"batch64": run_batch, "serve": run_serve, "progressive": run_progressive}[args.workload](args, rank, world)
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()
        return rc
    if args.impl == "reference":
        rc = run_reference(args, rank, world)
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()
        return rc

    import torch

    from pathtracer_gb300 import Context, Scene, build, cie_analytic, native, render_offscreen

    build.build()
    torch.cuda.set_device(local)
    W = H = args.res
    spf = min(args.spf, args.spp)
    ndisp = (args.spp + spf - 1) // spf
    samples_per_step = W * H * spf * ndisp
    scene = Scene.load(scene_path(args.workload))
    workload = workload_name(args)
    work_fixture = RENDER_WORKLOADS[args.workload][1]  # counts per sample, measured at the default size
    cie = cie_analytic()
    ctx = Context(local)
    engine_id = native.PT_ENGINE_WAVEFRONT if args.engine == "wavefront" else native.PT_ENGINE_MEGAKERNEL
    ctx.set_engine(engine_id)
    if args.pool:
        ctx.set_wavefront_pool(args.pool)
    if args.wf_engines:
        ctx.set_wavefront_engines(args.wf_engines)
    if args.fp_contract:
        ctx.set_fp_contract(True)
    if args.budget:
        ctx.set_march_budget(args.budget)
    knobs = {k: v for k, v in (("refill_min", args.refill), ("blocks_per_sm", args.blocks),
                               ("march_inner", args.inner)) if v}
    if args.drain >= 0:
        knobs["drain_lanes"] = args.drain
    if knobs:
        ctx.set_tuning(**knobs)
    ctx.bind(scene, cie)
    ctx.resize_accum(W, H)
    tuned, tune_secs = None, 0.0
    if args.autotune and args.engine == "wavefront":
        t0 = time.perf_counter()
        tuned, _ = ctx.autotune(scene.push_constants(W, H, 16, 16, 16, args.depth), rounds=args.autotune)
        tune_secs = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(ctx.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > 129 MB L2

    # Distinct sample indices per rank and per step (replicas, no exchange).
    from pathtracer_gb300 import replicas

    base = replicas.frame_base(rank, args.warmup + args.steps, ndisp, spf)

    launches = [0]  # the library's count of the kernels each dispatch launched

    def one_step(step_idx):
        frame = base + step_idx * ndisp * spf
        cur = 0
        for _ in range(ndisp):
            frame += spf
            cur += spf
            ctx.dispatch(scene.push_constants(W, H, frame, cur, spf, args.depth))
            launches[0] += ctx.last_kernel_launches()

    for i in range(args.warmup):
        one_step(i)
    ctx.wait()
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    torch.cuda.synchronize()

    times = []
    launches[0] = 0
    with ClockSampler(local) as clk:
        t_wall0 = time.perf_counter()
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            one_step(args.warmup + i)
            e1.record(stream)
            times.append((e0, e1))
        ctx.wait()
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    timed_launches = launches[0]
    ms = [a.elapsed_time(b) for a, b in times]
    ms_step = sum(ms) / len(ms)
    iters = ctx.last_iterations()

    # The other engine on the same workload (one warm-up, one timed step).
    other = {}
    if args.compare_engines:
        ctx.set_engine(1 - engine_id)
        one_step(args.warmup + args.steps)
        ctx.wait()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            flush.zero_()
            o0 = torch.cuda.Event(enable_timing=True)
            o1 = torch.cuda.Event(enable_timing=True)
            o0.record(stream)
        one_step(args.warmup + args.steps + 1)
        o1.record(stream)
        ctx.wait()
        torch.cuda.synchronize()
        oms = o0.elapsed_time(o1)
        other = {("megakernel" if engine_id == native.PT_ENGINE_WAVEFRONT else "wavefront"):
                 {"value": samples_per_step / (oms / 1000.0), "ms_per_step": oms}}
        ctx.set_engine(engine_id)
    ms_step = replicas.max_over_ranks([ms_step])[0]
    value = replicas.whole_job_rate(samples_per_step, world, ms_step / 1000.0)

    # End to end through the C ABI with host buffers.
    e2e_secs = []
    for i in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        acc, _ = render_offscreen(ctx, scene, cie, W, H, args.spp, spf, args.depth,
                                  frame_offset=base + (args.warmup + args.steps + 2 + i) * ndisp * spf)
        e2e_secs.append(time.perf_counter() - t0)
    e2e_step = statistics.median(e2e_secs)
    e2e_step = replicas.max_over_ranks([e2e_step])[0]
    e2e_value = replicas.whole_job_rate(samples_per_step, world, e2e_step)
    h2d = native.UBO_FLOATS * 4
    d2h = W * H * 16 + 9 * 4 * sum(list(scene.counts().values())[:5])

    peaks, peak_kind = measured_peaks()
    if args.engine == "wavefront":
        roofline, stages, ops = stage_roofline(ctx, lambda: one_step(args.warmup + args.steps + 5), samples_per_step,
                                               work_fixture, peaks, peak_kind,
                                               traffic_key(workload, spf, ctx.tuning()))
    else:
        from pathtracer_gb300 import workmodel

        ops = workmodel.fp32_ops_per_sample(workmodel.load(work_fixture)["per_sample"])
        peak = fp32_peak_tflops(peaks)
        ach = ops["total"] * samples_per_step / (ms_step / 1000.0) / 1e12
        roofline = {"bound": "fp32", "kernel": "megakernel", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                    "frac": ach / peak, "traffic": None, "work_per_sample": ops["total"]}
        stages = None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload, "resolution": [W, H], "spp": args.spp, "max_depth": args.depth,
                   "samples_per_dispatch": spf, "dispatches_per_step": ndisp,
                   "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"replicas x{world}",
                   "wavefront_tuning": ctx.tuning() if args.engine == "wavefront" else None,
                   "wavefront_engines": ctx.wavefront_engines() if args.engine == "wavefront" else None,
                   "autotuned": bool(tuned), "autotune_s": tune_secs,
                   "fp_contract": bool(args.fp_contract)},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "engine": args.engine,
        "engines": {args.engine: {"value": value / world, "ms_per_step": ms_step}, **other},
        "wavefront_iterations_per_dispatch": iters if args.engine == "wavefront" else None,
        # the library's count per dispatch (pt_last_kernel_launches): per
        # wavefront engine init, job_add and 4 kernels per iteration (graph
        # replays counted per kernel), then the resolve
        "gpu_launches": timed_launches,
        "wall_s_timed_region": t_wall,
        "roofline": roofline,
        "stages": stages,
        "fp32_ops_per_sample": ops,
        "clocks": clk.summary(),
    }
    if args.serve_jobs and world == 1:
        # The spec comparison on the serving workload: a saturated burst
        # of jobs drawn from the serving distribution (70 % sphere jobs, 30 %
        # SDF jobs with drawn mandelbulb powers / Menger levels), each refined
        # to 2 % relative RMSE against its FP64-summed reference, batched and
        # served vs one after another through the plain megakernel.
        sopts = argparse.Namespace(pool_scenes=8, burst=args.serve_jobs, rate=args.rate, duration=args.duration,
                                   ref_spp=1024, max_spp=512, target_rmse=0.02, sdf_scenes="varied",
                                   iters_per_poll=4, passes_in_flight=1, pool=0, serve_spheres=args.serve_spheres,
                                   ref_paths=args.ref_paths)
        t0 = time.perf_counter()
        serve = serve_measure(sopts, local, rank)
        line["serve"] = {"config": serve_config(sopts), **serve, "wall_s": time.perf_counter() - t0,
                         "note": "a saturated burst of jobs from the serving configuration's job distribution; its "
                                 "200 jobs/s x 60 s stream offers far more work than one GPU serves "
                                 "(saturates_at_200_jobs_per_s)"}
    if rank == 0:
        nthreads = os.cpu_count() or 1
        v, samples, dt, rows, kind = cpu_baseline(args, W, H, args.spp, nthreads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": nthreads, "kind": kind,
                                "sample": f"{rows} evenly spaced rows of {W}x{H} at {args.spp} spp "
                                          f"({samples} paths, {dt:.1f} s)"}
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
