"""The N > 1 path on CPU: two gloo ranks split a set of generated jobs, each
renders its share with the CPU restatement at a tiny size, and rank 0 gathers
the per-job results: every job rendered exactly once, results identical to a
single-rank run, timings combined by max over ranks."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _render(seed):
    from oracle import compare
    from pathtracer_gb300 import Scene, cie_analytic

    scene, spec = Scene.generate(0, seed)
    push = scene.push_constants(12, 8, 2, 2, 2, spec.pathLength)
    acc, _ = compare.run_oracle(scene.pack_ubo(cie_analytic()), push, compare.plugins_for(scene), nthreads=1)
    return float(np.float64(acc[..., :3]).sum()), acc.tobytes()


def _worker(rank, world, port, n_jobs, out_path):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    from pathtracer_gb300 import replicas

    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = list(replicas.job_range(rank, world, n_jobs))
    results = {j: _render(100 + j) for j in mine}
    secs = [0.1 * (rank + 1), 1.0]
    worst = replicas.max_over_ranks(secs)
    gathered = replicas.gather_to_root(results)
    if rank == 0:
        import pickle

        with open(out_path, "wb") as f:
            pickle.dump({"gathered": gathered, "worst": worst}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_job_range_partitions():
    from pathtracer_gb300 import replicas

    for n in (0, 1, 5, 64, 65):
        for world in (1, 2, 3, 8):
            got = [j for r in range(world) for j in replicas.job_range(r, world, n)]
            assert got == list(range(n))
            sizes = [len(replicas.job_range(r, world, n)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1
    assert list(replicas.job_seeds(1, 64)) == list(range(64, 128))
    assert replicas.frame_base(0, 8, 1, 64) == 0 and replicas.frame_base(1, 8, 1, 64) == 16 * 64
    assert replicas.whole_job_rate(10.0, 4, 2.0) == 20.0
    assert replicas.max_over_ranks([1.0, 2.0]) == [1.0, 2.0]  # no process group
    with pytest.raises(ValueError):
        replicas.job_range(2, 2, 4)


def test_two_gloo_ranks_render_each_job_once(built, tmp_path):
    n_jobs, world = 5, 2
    out = str(tmp_path / "gathered.pkl")
    mp.start_processes(_worker, args=(world, _free_port(), n_jobs, out), nprocs=world, start_method="spawn")
    import pickle

    with open(out, "rb") as f:
        res = pickle.load(f)
    merged = {}
    for part in res["gathered"]:
        assert not set(part) & set(merged)  # no job on two ranks
        merged.update(part)
    assert sorted(merged) == list(range(n_jobs))
    for j in range(n_jobs):
        assert merged[j] == _render(100 + j)  # same bytes as a single-rank render
    assert res["worst"] == [0.2, 1.0]
