"""The multi-GPU path is replicas: one independent problem per rank, with gloo barriers and
max / sum reductions as the only control plane (bench.Dist).  These tests run two gloo ranks on
the CPU (127.0.0.1 rendezvous): the reductions the bench uses for the whole-job value, and the
reference arm under torchrun, where rank 0 alone runs and prints one JSON line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist(world)
    d.barrier()
    local_ms = 10.0 * (rank + 1)           # per-rank timed region
    max_ms = d.max(local_ms)
    pts = d.sum(float(32 ** 3) * 5)          # units all ranks processed
    d.barrier()
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"max_ms": max_ms, "pts": pts, "value": pts / (max_ms / 1e3)}, f)
    d.close()


def test_dist_reductions_two_gloo_ranks(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0 = json.load(open(tmp_path / "r0.json"))
    r1 = json.load(open(tmp_path / "r1.json"))
    assert r0 == r1
    assert r0["max_ms"] == 20.0                       # max over ranks
    assert r0["pts"] == 2 * 32 ** 3 * 5                # whole-job units
    assert r0["value"] == pytest.approx(2 * 32 ** 3 * 5 / 0.020)


def test_reference_arm_two_ranks_prints_once():
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--grid", "32", "--steps", "1", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="1", MHD_ORACLE_WORKERS="2")
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
