"""The 3xTF32 threshold scan: the exact form on tensor cores for rows wider than 128
and for k above 128 (the reference's demo shapes reach d = 1024 and 2048,
demo/knnTest.m:9,39,63,87; its selections take k up to 512, readme.txt:80).

Bars as in test_gpu_parity.py: indices identical to the oracle's except where the
FP64 distances of the competing candidates differ by less than 1e-6 relative,
distances within 1e-5 relative of FP64; bit-exact on integer data (every TF32
product and FP32 sum exact) and wherever the oracle's convention is shared.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAP = 1e-6
DIST_REL = 1e-5


def run(engine, X, Qs, k, **kw):
    import torch
    c = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    q = torch.from_numpy(np.ascontiguousarray(Qs)).cuda()
    d, i = engine.search(c, q, k, **kw)
    return d.cpu().numpy(), i.cpu().numpy(), engine.last_stats()


@pytest.mark.parametrize("D,k", [(1024, 16), (2048, 16), (256, 128), (1024, 128), (160, 50)])
def test_wide_rows_on_tensor_cores(engine, oracle, D, k):
    # the reference's demo shape: 32,768 uniform [0, 1) vectors, 256 queries
    rng = np.random.default_rng(D + k)
    X = rng.random((32768, D), dtype=np.float32)
    Qs = rng.random((256, D), dtype=np.float32)
    d, i, st = run(engine, X, Qs, k)
    assert st["algo"] == engine.ALGO_TC and st["scan"] == 1
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    oracle.check_parity(X, Qs, k, d, i, ref_idx=oi, gap_rel=GAP, dist_rel=DIST_REL)
    assert (i == oi).mean() > 0.999
    assert engine.last_fixups() <= 2


@pytest.mark.parametrize("D,k", [(128, 256), (43, 512), (96, 200), (64, 129)])
def test_large_k_on_tensor_cores(engine, oracle, D, k):
    rng = np.random.default_rng(7 * D + k)
    X = rng.random((40000, D), dtype=np.float32)
    Qs = rng.random((300, D), dtype=np.float32)
    d, i, st = run(engine, X, Qs, k)
    assert st["algo"] == engine.ALGO_TC and st["scan"] == 1 and st["kp"] >= k
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    oracle.check_parity(X, Qs, k, d, i, ref_idx=oi, gap_rel=GAP, dist_rel=DIST_REL)
    assert (i == oi).mean() > 0.999


@pytest.mark.parametrize("D,k", [(300, 200), (1000, 32)])
def test_integer_data_bit_exact(engine, oracle, D, k):
    rng = np.random.default_rng(D)
    X = rng.integers(0, 256, (30000, D)).astype(np.float32)
    Qs = rng.integers(0, 256, (200, D)).astype(np.float32)
    d, i, st = run(engine, X, Qs, k)
    assert st["scan"] == 1
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


def test_duplicates_overflow_into_the_fixup(engine, oracle):
    # every query equals 3,000 corpus rows: the segments overflow, every query is answered
    # by the CUDA-core fix-up (compacted, two launches for 60 queries) -- bit-exact, ties by index
    rng = np.random.default_rng(3)
    base = rng.integers(0, 32, (8, 200)).astype(np.float32)
    X = np.repeat(base, 3000, axis=0)
    rng.shuffle(X)
    Qs = base[rng.integers(0, 8, 60)]
    k = 150
    d, i, st = run(engine, X, Qs, k)
    assert st["scan"] == 1
    assert engine.last_fixups() == 60
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


def test_reference_semantics_on_wide_rows(engine, oracle):
    # rank by the GEMM-form key, distance = key + ||q||^2 (the reference's output)
    rng = np.random.default_rng(11)
    X = rng.random((32768, 1024), dtype=np.float32)
    Qs = rng.random((128, 1024), dtype=np.float32)
    k = 16
    d, i, st = run(engine, X, Qs, k, rerank=False)
    assert st["scan"] == 1
    od, oi = oracle.knn_gemm(X, Qs, k)
    # the TF32 and the oracle's FP32 key differ by a few FP32 ulps of ||q||^2 + ||c||^2
    oracle.check_parity(X, Qs, k, d, i, ref_idx=oi, gap_rel=2e-5, dist_rel=1e-4)


def test_dropin_and_index_on_wide_rows(engine, oracle):
    import torch
    rng = np.random.default_rng(12)
    X = rng.random((20000, 200), dtype=np.float32)
    Qs = rng.random((150, 200), dtype=np.float32)
    k = 128
    vals, idxf, t = engine.gpuknnsBitonic(Qs, X, k, 1)
    oracle.check_parity(X, Qs, k, vals, idxf.astype(np.int64), gap_rel=GAP, dist_rel=DIST_REL)
    ix = engine.Index(torch.from_numpy(X).cuda())
    d, i = ix.search(torch.from_numpy(Qs).cuda(), k)
    np.testing.assert_array_equal(i.cpu().numpy(), idxf.astype(np.int32))
    np.testing.assert_array_equal(d.cpu().numpy(), vals)
    ix.close()


@pytest.mark.parametrize("N,D,k", [(150_000, 128, 100), (140_003, 96, 10)])
def test_fp32_data_beside_the_bf16_scan(engine, oracle, N, D, k):
    # Large corpora of FP32 data in the exact form: the BF16 threshold scan and the 3xTF32 one
    # are both launched and the data's BF16-exactness, found on the device, lets only the TF32
    # scan run.  Its answers are those of the TF32 scan alone (same plan, bit for bit), of a
    # host-buffer search (the corpus copied, prepared and scanned in blocks), and of the shortlist
    # kernel up to ties.
    rng = np.random.default_rng(N + D)
    X = rng.random((N, D), dtype=np.float32)
    Qs = rng.random((300, D), dtype=np.float32)
    d, i, st = run(engine, X, Qs, k)
    assert st["scan"] == 1 and st["scan_keys"] == 3
    d1, i1 = engine.search_host(X, Qs, k)
    assert engine.last_stats()["scan_keys"] == 3
    np.testing.assert_array_equal(i1, i)
    np.testing.assert_array_equal(d1, d)
    d2, i2, st2 = run(engine, X, Qs, k, scan=engine.SCAN_TF32)
    assert st2["scan_keys"] == 2
    np.testing.assert_array_equal(i2, i)
    np.testing.assert_array_equal(d2, d)
    d3, i3, _ = run(engine, X, Qs, k, scan=engine.SCAN_OFF)
    assert (i3 == i).mean() > 0.999
    sub = np.arange(0, 300, 3)
    od, oi = oracle.knn_gemm(X, Qs[sub], k, kp=st["kp"], rerank=True)
    oracle.check_parity(X, Qs[sub], k, d[sub], i[sub], ref_idx=oi, gap_rel=GAP, dist_rel=DIST_REL)


def test_small_corpus_fp32_and_integer_data_on_the_tf32_scan(engine, oracle):
    # Below the BF16 scan's default size (16,384 <= N < 131,072) the exact form runs the TF32
    # scan for data of every kind: parity on FP32 data, bit-exact on integer data.
    import cuknns.synth as S
    X, Qs = S.uniform(65536, 128, seed=0, nq=1024)
    d, i, st = run(engine, X, Qs, 16)
    assert st["scan_keys"] == 2
    od, oi = oracle.knn_gemm(X, Qs[:256], 16, kp=st["kp"], rerank=True)
    oracle.check_parity(X, Qs[:256], 16, d[:256], i[:256], ref_idx=oi, gap_rel=GAP, dist_rel=DIST_REL)
    rng = np.random.default_rng(5)
    Xi = rng.integers(0, 200, (70000, 64)).astype(np.float32)
    Qi = rng.integers(0, 200, (129, 64)).astype(np.float32)
    d, i, st = run(engine, Xi, Qi, 24)
    assert st["scan_keys"] == 2
    od, oi = oracle.knn_gemm(Xi, Qi, 24, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


@pytest.mark.parametrize("D,Q,k", [(96, 300, 16), (32, 257, 10), (64, 130, 40), (128, 300, 16), (100, 200, 20)])
def test_two_issuer_tiles_integer_data_bit_exact(engine, oracle, D, Q, k):
    # rows of up to 128 columns: the queries sit in tensor memory and two MMA issuers alternate
    # the corpus tiles (sharing ring slots at 128 columns); integer data keep every TF32 product
    # and sum exact, so the answers are the oracle's bit for bit (many tiles per CTA, a ragged
    # last query tile)
    rng = np.random.default_rng(D + Q)
    X = rng.integers(0, 256, (120_000, D)).astype(np.float32)
    Qs = rng.integers(0, 256, (Q, D)).astype(np.float32)
    d, i, st = run(engine, X, Qs, k, scan=engine.SCAN_TF32)
    assert st["scan_keys"] == 2
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)
