"""The multi-rank paths of bench.py on CPU with gloo, world size 2: the
collectives the timing uses (barrier, max and sum over ranks), independent
replicas per rank, and the reference arm under torchrun (rank 0 alone works
and prints; every rank exits 0)."""
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


def _rank_main(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    r, ws, _, dist = bench.dist_setup()
    bench.barrier(dist)
    res = {"rank": r, "ws": ws, "max": bench.allreduce_max(dist, 1.5 + r), "sum": bench.allreduce_sum(dist, 1.0 + r)}
    with open(os.path.join(out_dir, f"r{r}.json"), "w") as f:
        json.dump(res, f)
    dist.destroy_process_group()


def test_collectives_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp

    mp.spawn(_rank_main, args=(_free_port(), str(tmp_path)), nprocs=2, join=True)
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in (0, 1)]
    for r in res:
        assert r["ws"] == 2 and r["max"] == 2.5 and r["sum"] == 3.0


def test_replicas_are_independent_clusters():
    sys.path.insert(0, ROOT)
    import bench

    cfg = bench.CONFIGS["plummer1e5"]
    (n0, ic0, s0), = bench.make_clusters(cfg, 2000, 0)
    (n1, ic1, s1), = bench.make_clusters(cfg, 2000, 1)
    assert n0 == n1 == 2000 and s0 != s1
    assert not (ic0["r"] == ic1["r"]).all()


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--config", "plummer1e5",
           "--cpu-sample", "2000"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
