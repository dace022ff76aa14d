"""Writes generated_jobs.json: the seeded job generator's output (scene JSON
of a few seeds, specs of the first 64 sphere jobs and 16 SDF jobs), pinning
pt_scene_generate against unintended change.

    python tests/golden/make_generated.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from pathtracer_gb300 import native, renderer  # noqa: E402


def spec_dict(spec):
    return {k: getattr(spec, k) for k, _ in native.PtJobSpec._fields_ if k != "pad"}


def main():
    out = {"scenes": [], "sphere_specs": [], "sdf_specs": []}
    for kind, seed in ((native.PT_GEN_SPHERES, 0), (native.PT_GEN_SPHERES, 1), (native.PT_GEN_SDF, 0),
                       (native.PT_GEN_SDF, 1), (native.PT_GEN_SDF, 2)):
        scene, spec = renderer.Scene.generate(kind, seed)
        out["scenes"].append({"spec": spec_dict(spec), "json": scene.to_json()})
    for seed in range(64):
        out["sphere_specs"].append(spec_dict(renderer.Scene.generate(native.PT_GEN_SPHERES, seed)[1]))
    for seed in range(16):
        out["sdf_specs"].append(spec_dict(renderer.Scene.generate(native.PT_GEN_SDF, seed)[1]))
    with open(os.path.join(HERE, "generated_jobs.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
