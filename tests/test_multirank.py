"""Multi-rank host logic on CPU with the gloo backend (world size 2).

* i-partition (tupan_gb300.sharding): each rank evaluates its i-slice
  against the full j-set (here with the CPU oracle) and the gathered result
  equals the single-process evaluation bit for bit.
* bench.py's rank handling under torch.distributed.run: the reference arm
  runs on rank 0 only and prints one JSON line; rank 1 exits 0.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from tupan_gb300.sharding import i_slice

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_i_slice_covers_range():
    for n in (0, 1, 7, 100):
        for world in (1, 2, 3, 8):
            parts = [i_slice(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[k][1] == parts[k + 1][0] for k in range(world - 1))


def _worker(rank, world, port, path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.oracle import Oracle
    from tupan_gb300.sharding import sharded_calc
    rng = np.random.default_rng(5)
    n = 301
    d = {k: torch.tensor(rng.normal(size=n)) for k in ("rx", "ry", "rz", "vx", "vy", "vz")}
    d["mass"] = torch.tensor(rng.random(n) / n)
    d["eps2"] = torch.full((n,), 1e-4)
    orc = Oracle()

    def fn(iset, jset):
        out = orc.calc("acc_jerk", {k: v.numpy() for k, v in iset.items()},
                       {k: v.numpy() for k, v in jset.items()})
        return [torch.tensor(o) for o in out]

    got = sharded_calc(fn, d, d, rank, world)
    if rank == 0:
        want = fn(d, d)
        ok = all(torch.equal(a, b) for a, b in zip(got, want))
        with open(path, "w") as f:
            f.write("ok" if ok else "mismatch")
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_evaluation_matches_single_process(tmp_path):
    path = str(tmp_path / "result")
    mp.spawn(_worker, args=(2, 29517, path), nprocs=2, join=True)
    assert open(path).read() == "ok"


def test_bench_reference_arm_under_torchrun():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", "29533", os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--cpu-seconds", "0.2", "--particles", "2048"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2 and rec["value"] > 0
