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
