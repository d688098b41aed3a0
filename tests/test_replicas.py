"""The multi-GPU path ("replicas only": the paths are i.i.d.; the one
exchange step sums the ranks' accumulators) on CPU with gloo, world size 2:
the bench's barrier, its sum / max reductions over ranks, the accumulator
merge, the per-rank seeds, and the reference arm launched through
torch.distributed.run, where rank 0 alone prints its line."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, ws: int, port: int, out_dir: str):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    dist, r, n = bench._dist()
    bench._barrier(dist)
    res = {
        "rank": r, "world": n, "backend": dist.get_backend(),
        "sum": bench._sum_over_ranks(dist, float(r + 1)),
        "max": bench._max_over_ranks(dist, [1.5, 2.5][r]),
        "seed": bench._workload(seed=1000 * r, paths_log2=10)[0]["simulation"]["seed"],
    }
    import numpy as np
    u = np.full((3, 2, 4, 1), (r + 1) + 1j * (10 * (r + 1)))
    um, itm = bench._merge_over_ranks(dist, u, np.array([100.0 * (r + 1)]))
    res["merged"] = [float(um.real.max()), float(um.real.min()), float(um.imag.max()), float(itm[0]), list(um.shape)]
    bench._barrier(dist)
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
        json.dump(res, f)


def test_reductions_and_seeds_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for r, x in enumerate(res):
        assert x["rank"] == r and x["world"] == 2 and x["backend"] == "gloo"
        assert x["sum"] == 3.0          # contributions: summed over ranks
        assert x["max"] == 2.5          # time: the slowest rank
    assert res[0]["seed"] != res[1]["seed"]   # disjoint path sets per replica
    for x in res:   # the exchange step: every rank holds the sum of both accumulators and iteration counts
        assert x["merged"] == [3.0, 3.0, 30.0, 300.0, [3, 2, 4, 1]]


def test_reference_arm_prints_on_rank0_only():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port),
           "bench.py", "--gpus", "2", "--impl", "reference", "--steps", "1", "--warmup", "0", "--ref-sample", "64"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
