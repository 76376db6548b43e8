"""Host-buffer searches over corpora streamed in blocks (the reference's
host-side corpus blocking, src/cuknnBitonic.cu:493-512,550-589): each block is
searched and merged into the running top-k by (distance, index).

Bar: identical distances and indices to one search over the whole corpus, for
block sizes that divide the corpus, that leave a last block smaller than k, and
for both the threshold-scan (integer data) and shortlist (FP32 data) paths.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def data(kind, n, q, d, seed):
    rng = np.random.default_rng(seed)
    if kind == "int":
        return rng.integers(0, 64, (n, d)).astype(np.float32), rng.integers(0, 64, (q, d)).astype(np.float32)
    return rng.random((n, d), dtype=np.float32), rng.random((q, d), dtype=np.float32)


@pytest.mark.parametrize("kind,N,block_rows,k", [("int", 50_000, 7_000, 16), ("int", 21_050, 7_000, 100),
                                                 ("uniform", 40_000, 10_000, 32), ("uniform", 9_001, 3_000, 1),
                                                 ("int", 140_000, 70_000, 100)])
def test_blocked_equals_whole(engine, oracle, kind, N, block_rows, k):
    X, Qs = data(kind, N, 150, 64, N + k)
    d0, i0 = engine.search_host(X, Qs, k)
    kp = engine.last_stats()["kp"]
    d1, i1 = engine.search_host(X, Qs, k, block_rows=block_rows)
    np.testing.assert_array_equal(i1, i0)
    np.testing.assert_array_equal(d1, d0)
    if kind == "int":
        od, oi = oracle.knn_gemm(X, Qs[:20], k, kp=kp, rerank=True)
        np.testing.assert_array_equal(i1[:20], oi)


def test_block_rows_validation(engine):
    X, Qs = data("int", 5_000, 10, 32, 1)
    with pytest.raises(engine.KnnsError):
        engine.search_host(X, Qs, 4, block_rows=-1)
    # a block smaller than k is widened to k rows
    d0, i0 = engine.search_host(X, Qs, 40)
    d1, i1 = engine.search_host(X, Qs, 40, block_rows=10)
    np.testing.assert_array_equal(i1, i0)
    np.testing.assert_array_equal(d1, d0)


@pytest.mark.parametrize("kind,N,D,k,prec,pinned", [("int", 400_003, 128, 100, "exact", True),
                                                    ("int", 150_000, 64, 16, "bf16", True),
                                                    ("aniso", 300_001, 256, 32, "fp8", True),
                                                    ("uniform", 200_000, 96, 10, "bf16", True),
                                                    ("uniform", 180_000, 32, 20, "exact", True),
                                                    ("int", 250_000, 128, 100, "exact", False)])
def test_host_search_overlapping_copy_equals_resident(engine, kind, N, D, k, prec, pinned):
    # Host-buffer searches on the threshold-scan path copy the corpus in blocks and prepare and
    # scan each block as it lands (the seeding sample read in place from page-locked memory, or
    # copied ahead of the blocks from pageable memory); the answers must be those of the same
    # search on the resident corpus, bit for bit -- including FP32 data in the exact form, where
    # the scan stands down and the TF32 path runs after the last block.
    import torch
    import cuknns.synth as S
    if kind == "aniso":
        X, Qs = S.anisotropic(N, D, seed=N, nq=300)
    else:
        X, Qs = data(kind, N, 300, D, N + D)
    p = {"exact": engine.PREC_EXACT, "bf16": engine.PREC_BF16, "fp8": engine.PREC_FP8}[prec]
    keep = (torch.from_numpy(X).pin_memory(), torch.from_numpy(Qs).pin_memory()) if pinned else None
    hx, hq = (keep[0].numpy(), keep[1].numpy()) if pinned else (X, Qs)
    for _ in range(2):  # the second call reuses the engine's buffers and streams
        d1, i1 = engine.search_host(hx, hq, k, precision=p, shortlist=2 if prec != "exact" else 0)
    st = engine.last_stats()
    d0, i0 = engine.search(torch.from_numpy(X).cuda(), torch.from_numpy(Qs).cuda(), k, precision=p,
                           shortlist=2 if prec != "exact" else 0)
    assert st["scan"] == 1
    np.testing.assert_array_equal(i1, i0.cpu().numpy())
    np.testing.assert_array_equal(d1, d0.cpu().numpy())


@pytest.mark.parametrize("kind,N,shards,k", [("int", 300_000, 4, 100), ("uniform", 70_000, 3, 16),
                                             ("int", 250, 3, 100)])
def test_corpus_shards_merged_on_device_equal_whole(engine, kind, N, shards, k):
    # The multi-GPU corpus split, its ranks run one after another on this GPU: each shard is
    # searched, its indices made global, and the per-shard lists merged in rank order by the
    # device merge (knns_merge_topk) -- the answer of one search over the whole corpus.
    import torch
    from cuknns import shard as S
    X, Qs = data(kind, N, 200, 64, N + k)
    c, q = torch.from_numpy(X).cuda(), torch.from_numpy(Qs).cuda()
    ds, idxs, counts = [], [], []
    for r in range(shards):
        r0, r1 = S.shard_bounds(N, shards, r)
        d, i = S.sharded_search(c[r0:r1], r0, q, k)  # no process group: this rank's padded list
        ds.append(d)
        idxs.append(i)
        counts.append(min(k, r1 - r0))
    d1, i1 = S.merge_rank_lists(ds, idxs, counts, k, lambda rd, ri, h, bd, bi, kb, kk:
                                engine.merge_topk(rd, ri, h, bd, bi, kb, kk))
    d0, i0 = engine.search(c, q, k)
    np.testing.assert_array_equal(i1.cpu().numpy(), i0.cpu().numpy())
    np.testing.assert_array_equal(d1.cpu().numpy(), d0.cpu().numpy())
