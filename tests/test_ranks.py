"""Multi-rank host logic on the CPU (gloo, world_size 2).

Queries shard across ranks with no exchange (replicas): every rank gets the same
corpus and its own queries, the timed region's duration reduces by max over the
ranks, and under torchrun the reference arm prints one JSON line from rank 0
while the other rank exits 0.
"""
import json
import os
import socket
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    v = bench.reduce_max(10.0 + 3.0 * rank, dist, "cpu")
    out.put((rank, v))
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_max_over_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 13.0, 1: 13.0}


def test_replica_sharding_same_corpus_own_queries():
    sys.path.insert(0, ROOT)
    import bench
    w = bench.WORKLOADS["uniform64k"]
    c0, q0 = bench.gen_data(w, 0)
    c1, q1 = bench.gen_data(w, 1)
    np.testing.assert_array_equal(c0, c1)
    assert q0.shape == q1.shape and not np.array_equal(q0, q1)


def test_reference_arm_under_torchrun_two_ranks():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--workload", "uniform64k"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
