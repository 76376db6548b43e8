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


# ---------------------------------------------------------------- corpus split across ranks
def _np_search(oracle_mod):
    """Stand-in for the device search on CPU ranks: the oracle's re-ranked kNN (the engine's convention)."""
    import torch

    def search(shard, queries, kb, **_):
        d, i = oracle_mod.knn_gemm(shard.numpy(), queries.numpy(), kb, kp=max(32, (kb + 8 + 15) // 16 * 16),
                                   rerank=True)
        return torch.from_numpy(d), torch.from_numpy(i)
    return search


def _np_merge(run_d, run_i, have, blk_d, blk_i, kb, k):
    """Stand-in for the device merge: first min(k, have + kb) of the union by (distance, index)."""
    import torch
    d = torch.cat([run_d[:, :have], blk_d], 1).numpy()
    i = torch.cat([run_i[:, :have], blk_i], 1).numpy()
    n = min(k, have + kb)
    out_d = np.full((d.shape[0], k), np.inf, np.float32)
    out_i = np.full((d.shape[0], k), -1, np.int32)
    for q in range(d.shape[0]):
        o = np.lexsort((i[q], d[q]))[:n]
        out_d[q, :n], out_i[q, :n] = d[q][o], i[q][o]
    return torch.from_numpy(out_d), torch.from_numpy(out_i)


def _shard_rank_main(rank, world, port, n, k, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    for p in (os.path.join(ROOT, "knn-toolbox_gb300"), os.path.join(ROOT, "oracle")):
        sys.path.insert(0, p)
    import torch
    import torch.distributed as dist
    import oracle
    from cuknns import shard as S
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(n)
    X = rng.integers(0, 8, (n, 24)).astype(np.float32)   # integer data: exact, many ties
    Qs = rng.integers(0, 8, (37, 24)).astype(np.float32)
    r0, r1 = S.shard_bounds(n, world, rank)
    d, i = S.sharded_search(torch.from_numpy(X[r0:r1]), r0, torch.from_numpy(Qs), k,
                            search=_np_search(oracle), merge=_np_merge)
    out.put((rank, d.numpy(), i.numpy()))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_bounds_cover_the_corpus():
    sys.path.insert(0, os.path.join(ROOT, "knn-toolbox_gb300"))
    from cuknns import shard as S
    for n, w in [(10, 3), (7, 8), (1_000_000, 8), (0, 2)]:
        b = [S.shard_bounds(n, w, r) for r in range(w)]
        assert b[0][0] == 0 and b[-1][1] == n
        assert all(b[r][1] == b[r + 1][0] for r in range(w - 1))
        assert max(r1 - r0 for r0, r1 in b) - min(r1 - r0 for r0, r1 in b) <= 1


def test_corpus_split_over_gloo_ranks_equals_one_search(oracle):
    # two CPU ranks hold halves of the corpus; after the all-gather and the rank-order merge
    # both hold the answer of one search over the whole corpus (ties by the lower global index);
    # the small corpus leaves each shard with fewer rows than k
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    for n, k in [(3000, 20), (30, 20)]:
        out = ctx.Queue()
        port = free_port()
        procs = [ctx.Process(target=_shard_rank_main, args=(r, 2, port, n, k, out)) for r in range(2)]
        for p in procs:
            p.start()
        got = {r: (d, i) for r, d, i in (out.get(timeout=120) for _ in procs)}
        for p in procs:
            p.join(timeout=60)
            assert p.exitcode == 0
        rng = np.random.default_rng(n)
        X = rng.integers(0, 8, (n, 24)).astype(np.float32)
        Qs = rng.integers(0, 8, (37, 24)).astype(np.float32)
        od, oi = oracle.knn_f64(X, Qs, k)
        for r in (0, 1):
            np.testing.assert_array_equal(got[r][1], oi)
            np.testing.assert_array_equal(got[r][0].astype(np.float64), od)


def test_bench_refuses_a_world_size_that_is_not_gpus():
    env = dict(os.environ, WORLD_SIZE="3", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--impl", "reference",
                        "--workload", "uniform64k"], capture_output=True, text=True, timeout=120, env=env, cwd=ROOT)
    assert r.returncode == 2 and "WORLD_SIZE=3" in r.stderr


def test_bench_launches_its_own_ranks_for_gpus_n():
    # `--gpus 2` without a launcher: bench.py starts the two ranks itself (torch.distributed.run);
    # the reference arm prints one line from rank 0, whose n_gpus is 2
    env = {k_: v for k_, v in os.environ.items() if k_ not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "3", "--workload", "uniform64k"], capture_output=True, text=True,
                       timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1 and json.loads(lines[0])["n_gpus"] == 2
