"""Writes work_<workload>.json: event counts per path sample of the bench
workloads, from the CPU restatement's work counters (oracle.count_work) on
evenly spaced rows.  pathtracer_gb300/workmodel.py turns them into FP32
operations per stage for the roofline.

    python tests/golden/make_workmodel.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import compare, oracle  # noqa: E402
from pathtracer_gb300 import Scene, cie_analytic, native  # noqa: E402

ROWS = 4


def per_sample(scene, W, H, spp, depth, rows=ROWS):
    ubo = scene.pack_ubo(cie_analytic())
    push = scene.push_constants(W, H, spp, spp, spp, depth)
    tot = None
    for r in range(rows):
        y = (2 * r + 1) * H // (2 * rows)
        c = oracle.count_work(ubo, push, compare.plugins_for(scene), rect=(0, y, W, y + 1), ext=scene.ext_or_none())
        tot = c if tot is None else {k: tot[k] + c[k] for k in c}
    n = tot["samples"]
    return {k: v / n for k, v in tot.items()}, {"rows": rows, "samples": n}


def main():
    oracle.build()
    out = {}
    scene = Scene.load(os.path.join(ROOT, "pathtracer_gb300", "scenes", "mandelbulb_plane.json"))
    out["mandelbulb_plane_1024x1024_64spp_depth6"] = per_sample(scene, 1024, 1024, 64, 6)
    scene = Scene.load(os.path.join(ROOT, "pathtracer_gb300", "scenes", "mandelbulb12_plane.json"))
    out["mandelbulb12_plane_1024x1024_64spp_depth6"] = per_sample(scene, 1024, 1024, 64, 6)
    # the same fractal in the SDF-fractal configuration's full form (sky, spectra, march limits)
    scene = Scene.load(os.path.join(ROOT, "pathtracer_gb300", "scenes", "mandelbulb12_plane_full.json"))
    out["mandelbulb12_plane_full_1024x1024_64spp_depth6"] = per_sample(scene, 1024, 1024, 64, 6)
    # The mixed-job batch: the first 8 generated sphere jobs, 1 row each, weighted by their samples.
    tot, n = {}, 0
    for seed in range(8):
        sc, spec = Scene.generate(native.PT_GEN_SPHERES, seed)
        c, meta = per_sample(sc, spec.width, spec.height, spec.spp, spec.pathLength, rows=1)
        for k, v in c.items():
            tot[k] = tot.get(k, 0.0) + v * meta["samples"]
        n += meta["samples"]
    out["batch64_spheres"] = ({k: v / n for k, v in tot.items()}, {"jobs": 8, "rows_per_job": 1, "samples": n})
    for name, (counts, meta) in out.items():
        with open(os.path.join(HERE, f"work_{name}.json"), "w") as f:
            json.dump({"workload": name, "per_sample": counts, "sample": meta}, f, indent=1, sort_keys=True)
            f.write("\n")


if __name__ == "__main__":
    main()
