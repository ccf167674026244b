"""The multi-rank path of bench.py on CPU: gloo, world size 2.

bench.py runs one independent replica per rank (no data-path collective); the
ranks meet only at barriers and in the max-over-ranks of the timed region.  A
batch of replicas is split over the ranks (replica r on rank r mod N), each rank
timing its own share.  The reference arm (the CPU restatement) runs on rank 0
alone and the other ranks exit 0.  All are exercised here with two CPU processes.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _max_worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    os.environ["RANK"] = str(rank)
    os.environ["WORLD_SIZE"] = str(world)
    os.environ["LOCAL_RANK"] = str(rank)
    sys.path.insert(0, ROOT)
    import bench

    ws, r, _ = bench.dist_setup()
    bench.barrier(ws)
    q.put((r, bench.max_over_ranks(ws, 10.0 + 5.0 * r)))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_max_over_ranks_gloo_two_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_max_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 15.0), (1, 15.0)]


def test_reference_arm_under_torchrun_two_ranks():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--cells", "4"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["value"] > 0 and rec["unit"] == "atom-steps/s"
    assert rec["cpu_baseline"]["kind"] == "port" and rec["e2e"]["h2d_bytes_per_step"] == 0


def test_replica_share_partitions_the_batch():
    sys.path.insert(0, ROOT)
    import bench

    for n_rep, ws in ((4096, 2), (4096, 8), (64, 3), (5, 8)):
        shares = [bench.replica_share(n_rep, ws, r) for r in range(ws)]
        flat = sorted(x for sh in shares for x in sh)
        assert flat == list(range(n_rep))  # every replica once
        assert max(map(len, shares)) - min(map(len, shares)) <= 1


def _share_worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    os.environ["RANK"] = str(rank)
    os.environ["WORLD_SIZE"] = str(world)
    os.environ["LOCAL_RANK"] = str(rank)
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "caviar-v2_gb300"))
    import numpy as np

    import bench
    import workloads as W

    ws, r, _ = bench.dist_setup()
    sets = W.replica_set(12, nmin=256, nmax=600)
    mine = bench.replica_share(len(sets), ws, r)
    atoms = sum(len(sets[k][0]) for k in mine)
    total = bench.sum_over_ranks(ws, atoms)
    # replica k is generated from seed 1004 + k whichever rank builds it
    ref = W.replica_set(12, nmin=256, nmax=600)
    same = all(np.array_equal(sets[k][0], ref[k][0]) for k in mine)
    bench.barrier(ws)
    q.put((r, mine, atoms, total, same))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_replica_split_gloo_two_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_share_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    (r0, m0, a0, t0, s0), (r1, m1, a1, t1, s1) = got
    assert m0 == list(range(0, 12, 2)) and m1 == list(range(1, 12, 2))
    assert t0 == t1 == a0 + a1 and s0 and s1


def test_gpus_n_without_launcher_starts_n_ranks():
    """`bench.py --gpus 2` outside torchrun starts two ranks itself (the reference arm:
    rank 0 prints one line, rank 1 exits 0)."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--cells", "4"]
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1 and json.loads(lines[0])["n_gpus"] == 2
