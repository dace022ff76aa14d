"""bench.py's reference arm (the CPU restatement timed on the host cores) on
a tiny case of each single-scene workload: one JSON line in the bench
contract, the workload's SDF text restated for the oracle."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("workload", ["mandelbulb12", "mandelbulb"])
def test_reference_arm_prints_one_contract_line(built, workload):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          workload, "--res", "32", "--spp", "2", "--steps", "1", "--warmup", "3", "--cpu-rows", "2"],
                         capture_output=True, text=True, timeout=600, check=True).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"].startswith(workload + "_plane_32x32_2spp")
    # the reference's own shader built for the CPU for the GLSL scene, the oracle port for the keyed plug-in
    from oracle import ref_shader

    want = "reference" if workload == "mandelbulb12" and os.path.exists(ref_shader.shader_path()) else "port"
    assert d["cpu_baseline"]["kind"] == want and d["e2e"]["h2d_bytes_per_step"] == 0


def test_batch_cpu_baseline(built):
    """The batch workload's CPU figure: rows of generated sphere jobs through
    the reference's own shader where it was built (kind "reference"), else
    the oracle port."""
    sys.path.insert(0, ROOT)
    import bench
    from oracle import ref_shader

    jobs, _ = bench.make_jobs(3, 0)
    v, n, dt, kind = bench.batch_cpu_baseline(jobs, 4, rows_per_job=1, njobs=3)
    assert v > 0 and n == sum(spec.width * spec.spp for _, spec, _, _ in jobs) and dt > 0
    assert kind == ("reference" if os.path.exists(ref_shader.shader_path()) else "port")


@pytest.mark.parametrize("workload", ["mandelbulb12", "mandelbulb"])
def test_reference_arm_loads_no_product_library(built, workload):
    """The reference arm packs the scene and builds its CIE table with the
    oracle's restatement (oracle/pack.py): only libraries under oracle/
    are mapped into the process, none of the product's."""
    code = (
        "import sys; sys.argv = ['bench.py', '--impl', 'reference', '--workload', %r, '--res', '32', '--spp', '2',"
        " '--steps', '1', '--warmup', '3', '--cpu-rows', '2']\n"
        "sys.path.insert(0, %r)\n"
        "import bench\n"
        "args = bench.parse_args()\n"
        "assert bench.run_reference(args, 0, 1) == 0\n"
        "libs = sorted({l.split()[-1] for l in open('/proc/self/maps') if l.rstrip().endswith('.so')"
        " and l.split()[-1].startswith(%r)})\n"
        "print('LIBS', libs)\n" % (workload, ROOT, ROOT))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, check=True,
                         cwd=ROOT).stdout
    libs = eval([ln for ln in out.splitlines() if ln.startswith("LIBS")][0][5:])
    assert libs, out
    assert all(os.path.relpath(p, ROOT).startswith("oracle" + os.sep) for p in libs), libs
