"""Algorithmic FP32 work of the path tracer, per stage, from event counts.

An event is one call of a reference function on the hot path (one sphere
test, one SDF evaluation, one mandelbulb iteration, ...); the counts per
path sample of a workload come from the CPU restatement's instrumented run
and are committed as fixtures (tests/golden/work_*.json, written by
tests/golden/make_workmodel.py).  OPS gives the FP32 operations of one event,
counted by hand from the kernel source (pathtracer_gb300/csrc/kernel): add,
sub, mul, div and sqrt count 1, fma counts 2; comparisons, min/max, abs,
selects and integer work count 0; the pt_mathf functions count their own
arithmetic (sincos ~25, exp ~15, log ~18).  The counts are estimates to
about +-20%; they fix what "achieved TFLOP/s" means for the roofline.

Each event is attributed to the wavefront stage kernel that executes it, so
a stage's achieved rate is its work divided by its measured device time.
"""
from __future__ import annotations

import json
import os

# FP32 operations per event, and the stage kernel that performs it.
OPS = {
    # isect: analytic primitives (SC:263-364, SC:450-541) and SDF bounding boxes
    "sphere": (19, "isect"),           # oc, 2 dots, discriminant
    "plane": (4, "isect"),
    "bounding_sphere": (15, "isect"),
    "box": (45, "isect"),              # rotate into the box frame + slabs
    "cyclide": (400, "isect"),         # quartic solve
    "aabb": (21, "isect"),             # RayIntersectAABB
    # gen: camera lens slices (TracePathLens, SC:1409-1444)
    "lens_slice": (35, "gen"),
    # march: SphereTracing (SC:779-860) and the plug-ins (sdfs/*.glsl)
    "march_steps": (15, "march"),      # over-relaxation update, 2 divisions
    "sdf_mandelbulb": (34, "march"),   # initial length + 0.5*log(r)*r/dr
    "mandelbulb_iters": (67, "march"),  # r^7, 2 divisions, sqrt, Chebyshev 8th powers, length
    "sdf_menger": (135, "march"),
    "sdf_blob": (66, "march"),
    "sdf_terrain": (470, "march"),     # 22 sines
    # the run-time compiled power-8 mandelbulb of scenes/mandelbulb12_plane.json
    # (the only GLSL text in a workload with a work model)
    "sdf_custom": (33, "march"),       # offset, initial length, 0.5*log(r)*r/dr
    "bulb8_iters": (68, "march"),      # r^8 and r^7 by products, 1/l and 1/r from one division, 2 lengths, 2 Chebyshev pairs
    "sdf_material": (23, "march"),     # sdfmaterial + normal normalisation
    # shade: emission, BRDF, sampling and next-event estimation
    "emit": (100, "shade"),            # Planck at 4 wavelengths
    "brdf": (84, "shade"),             # Gaussian spectrum at 4 wavelengths
    "surface_hits": (200, "shade"),    # cosine + cone sampling, ToWorld, pdfs, MIS, RR, throughput
    # gen: per camera sample (wavelengths, disk sample, camera ray, XYZ)
    "samples": (150, "gen"),
}

STAGES = ("isect", "march", "shade", "gen")


def fp32_ops_per_sample(counters_per_sample: dict) -> dict:
    """FP32 operations per path sample by stage (and 'total')."""
    out = {s: 0.0 for s in STAGES}
    for name, (ops, stage) in OPS.items():
        out[stage] += ops * float(counters_per_sample.get(name, 0.0))
    out["total"] = sum(out[s] for s in STAGES)
    return out


def load(workload: str) -> dict:
    """Per-sample event counts of a committed workload fixture."""
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with open(os.path.join(here, "tests", "golden", f"work_{workload}.json")) as f:
        return json.load(f)
