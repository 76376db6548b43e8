"""Threshold-scan path (BF16 tensor cores, seeded per-query thresholds, candidate
segments, fix-up of failed queries) against the oracle and against the
shortlist path.  Bars as in test_gpu_parity.py: bit-exact where the arithmetic
is exact (integer data), otherwise indices identical except where the FP64
distances of competing candidates differ by < 1e-6 relative, distances within
1e-5 relative of FP64; the BF16 precision form is held to recall@k >= 0.99 with
exact distances for the returned indices.
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


def ints(n, q, d, seed, hi=256):
    rng = np.random.default_rng(seed)
    return (rng.integers(0, hi, (n, d)).astype(np.float32), rng.integers(0, hi, (q, d)).astype(np.float32))


def test_auto_scan_matches_shortlist_path_and_oracle(engine, oracle):
    import cuknns.synth as S
    X, Qs = S.int_descriptor(150_000, 128, seed=8, nq=300)
    k = 100
    d, i, st = run(engine, X, Qs, k)
    assert st["scan"] == 1
    d0, i0, st0 = run(engine, X, Qs, k, scan=engine.SCAN_OFF)
    assert st0["scan"] == 0
    np.testing.assert_array_equal(i, i0)
    np.testing.assert_array_equal(d, d0)
    sub = np.arange(0, 300, 7)
    od, oi = oracle.knn_gemm(X, Qs[sub], k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i[sub], oi)
    np.testing.assert_array_equal(d[sub], od)


@pytest.mark.parametrize("N,Q,D,k", [(20000, 300, 128, 16), (20011, 130, 64, 10), (16384, 1, 128, 100),
                                     (30000, 257, 96, 32), (25000, 64, 40, 1)])
def test_forced_scan_integer_data_bit_exact(engine, oracle, N, Q, D, k):
    X, Qs = ints(N, Q, D, N + D)
    d, i, st = run(engine, X, Qs, k, scan=engine.SCAN_ON)
    assert st["scan"] == 1
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


@pytest.mark.parametrize("boxes", [1, 2])
def test_ring_geometry_does_not_change_results(engine, oracle, boxes):
    X, Qs = ints(40000, 200, 128, 31)
    k = 20
    d, i, st = run(engine, X, Qs, k, scan=engine.SCAN_ON, scan_boxes=boxes)
    assert st["scan_ring"] % 100 == boxes
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


@pytest.mark.parametrize("Q", [40, 600])
def test_duplicate_rows_overflow_and_fixup(engine, oracle, Q):
    # Each query equals 2,000 corpus rows: every segment overflows, every query
    # fails the scan and is searched again by the fix-up (600 > 512 queries
    # also exercises the second fix-up launch).  Ties go to the lower index.
    rng = np.random.default_rng(5)
    base = rng.integers(0, 64, (10, 64)).astype(np.float32)
    X = np.repeat(base, 2000, axis=0)
    rng.shuffle(X)
    Qs = base[rng.integers(0, 10, Q)]
    k = 16
    d, i, st = run(engine, X, Qs, k, scan=engine.SCAN_ON)
    assert st["scan"] == 1
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


def test_ties_past_the_sort_at_the_boundary_key(engine, oracle):
    # Every distinct row appears 48 times (shuffled): with k = 100 (shortlist 112, sort
    # buffer 128 words) the boundary key K of rank 112 is shared by a whole group, so
    # the 144 words with keys up to K overflow the sort and the selection resolves K's
    # ties by a rank search over the index half (lower index first).  The scan itself
    # answers the queries: no segment overflows.
    rng = np.random.default_rng(12)
    base = rng.integers(0, 256, (3000, 64)).astype(np.float32)
    X = np.repeat(base, 48, axis=0)
    rng.shuffle(X)
    Qs = rng.integers(0, 256, (200, 64)).astype(np.float32)
    k = 100
    d, i, st = run(engine, X, Qs, k, scan=engine.SCAN_ON)
    assert st["scan"] == 1 and st["kp"] == 112
    assert engine.last_fixups() <= 20
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


def test_unrepresentative_sample_fixup(engine, oracle):
    # Only every 32nd row (exactly the finest seeding sample) lies near the
    # queries, so the seeded threshold admits fewer than kp rows and the fix-up
    # must take over.
    rng = np.random.default_rng(78)
    N, D, Q, k = 32 * 4096, 64, 150, 10
    Qs = rng.integers(0, 32, (Q, D)).astype(np.float32)
    X = rng.integers(200, 256, (N, D)).astype(np.float32)
    near = np.arange(0, N, 32)
    X[near] = Qs[rng.integers(0, Q, near.size)] + rng.integers(0, 2, (near.size, D)).astype(np.float32)
    d, i, st = run(engine, X, Qs, k)
    assert st["scan"] == 1
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


def test_exact_form_on_fp32_data_stays_on_tf32(engine, oracle):
    # The scan is launched but stands down on the device: data not BF16-exact.
    import cuknns.synth as S
    X, Qs = S.uniform(140_000, 128, seed=12, nq=200)
    k = 16
    d, i, st = run(engine, X, Qs, k)
    assert st["scan"] == 1
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    oracle.check_parity(X, Qs, k, d, i, ref_idx=oi, gap_rel=GAP, dist_rel=DIST_REL)
    d0, i0, _ = run(engine, X, Qs, k, scan=engine.SCAN_OFF)
    np.testing.assert_array_equal(i, i0)
    np.testing.assert_array_equal(d, d0)


@pytest.mark.parametrize("D,c", [(96, 4), (200, 2), (256, 4)])
def test_bf16_precision_form_on_scan(engine, oracle, D, c):
    import cuknns.synth as S
    X, Qs = S.gauss_mixture(150_000, D, seed=6, nq=150, centres=512)
    k = 10
    d, i, st = run(engine, X, Qs, k, precision=engine.PREC_BF16, shortlist=c)
    assert st["scan"] == 1 and st["kp"] >= c * k
    ex = oracle.knn_f64(X, Qs, k)
    rec = oracle.recall_at_k(i, ex[1])
    assert rec >= 0.99, rec
    got64 = oracle.pair_dist_f64(X, Qs, i)
    assert (np.abs(d - got64) <= DIST_REL * got64 + 1e-6).all()
    assert (np.diff(d, axis=1) >= 0).all()
    # the shortlist path ranks by the same BF16 keys (its MMA shape differs, so
    # FP32 accumulation may differ in the last bit on near-ties)
    d0, i0, _ = run(engine, X, Qs, k, precision=engine.PREC_BF16, shortlist=c, scan=engine.SCAN_OFF)
    assert (i == i0).mean() >= 0.999


@pytest.mark.parametrize("D,hi", [(64, 256), (256, 256), (128, 1024)])
def test_integer_data_exact_and_reranked_keys(engine, oracle, D, hi):
    # 64 x 255^2 keeps every key an exact float integer (the re-rank is skipped);
    # 256 x 255^2 does not, and values up to 1023 are not BF16-exact: both re-rank
    X, Qs = ints(30000, 140, D, 7 * D + hi, hi=hi)
    k = 12
    d, i, st = run(engine, X, Qs, k, precision=engine.PREC_BF16, shortlist=4, scan=engine.SCAN_ON)
    assert st["scan"] == 1
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    if hi <= 256:
        np.testing.assert_array_equal(i, oi)
        np.testing.assert_array_equal(d, od)
    else:
        # BF16 keys pick the shortlist: recall against the exact answer, exact distances returned
        assert oracle.recall_at_k(i, oracle.knn_f64(X, Qs, k)[1]) >= 0.99
        got64 = oracle.pair_dist_f64(X, Qs, i)
        assert (np.abs(d - got64) <= DIST_REL * got64 + 1e-6).all()


@pytest.mark.parametrize("form", ["int128", "mix96_bf16", "mix256_bf16", "aniso128_fp8", "aniso256_fp8"])
def test_scan_answers_nearly_every_query(engine, form):
    # the fix-up pass is exact, so a scan whose segments overflow for every query
    # (wrong keys, segments sized for another column split) passes every parity
    # test while running several times slower: bound the fix-up count directly
    import cuknns.synth as S
    Q = 1000
    if form == "int128":
        X, Qs = S.int_descriptor(300_000, 128, seed=3, nq=Q)
        kw, k = {}, 100
    elif form.startswith("mix"):
        X, Qs = S.gauss_mixture(300_000, int(form[3:].split("_")[0]), seed=2, nq=Q)
        kw, k = dict(precision=engine.PREC_BF16, shortlist=4), 10
    else:
        X, Qs = S.anisotropic(300_000, int(form[5:].split("_")[0]), seed=5, nq=Q)
        kw, k = dict(precision=engine.PREC_FP8, shortlist=2), 32
    d, i, st = run(engine, X, Qs, k, **kw)
    assert st["scan"] == 1
    fix = engine.last_fixups()
    assert fix <= Q // 100, (form, fix)
    assert (np.diff(d, axis=1) >= 0).all()


# ---------------------------------------------------------------- shortlists above 128 (precision forms)
@pytest.mark.parametrize("form,D,k,c", [("bf16", 128, 100, 2), ("bf16", 96, 100, 4), ("fp8", 256, 64, 4),
                                        ("bf16", 64, 500, 1)])
def test_precision_forms_long_shortlists(engine, oracle, form, D, k, c):
    # c*k above 128 (up to 512): the shortlist lives only in the scan's candidate segments;
    # recall against FP64 and exact distances as for the short lists
    import cuknns.synth as S
    if form == "fp8":
        X, Qs = S.anisotropic(150_000, D, seed=D + k, nq=200)
        p = engine.PREC_FP8
    else:
        X, Qs = S.gauss_mixture(150_000, D, seed=D + k, nq=200, centres=512)
        p = engine.PREC_BF16
    kp = (max(32, c * k) + 15) // 16 * 16 if c > 1 else 512
    d, i, st = run(engine, X, Qs, k, precision=p, shortlist=c, kp=kp if c == 1 else 0)
    assert st["scan"] == 1 and st["kp"] == kp and st["kp"] > 128
    ex = oracle.knn_f64(X, Qs, k)
    assert oracle.recall_at_k(i, ex[1]) >= 0.99
    got64 = oracle.pair_dist_f64(X, Qs, i)
    assert (np.abs(d - got64) <= DIST_REL * got64 + 1e-6).all()
    assert (np.diff(d, axis=1) >= 0).all()
    assert engine.last_fixups() <= 2


@pytest.mark.parametrize("Q", [20, 100])
def test_long_shortlist_fixup_on_cuda_cores(engine, oracle, Q):
    # Duplicated rows overflow every segment, so every query fails the scan; with a shortlist
    # above 128 the fix-up is the CUDA-core kernel with exact keys, compacted to the failed
    # queries (100 > 32 also runs its second launch).  Integer data: bit-exact.
    rng = np.random.default_rng(9)
    base = rng.integers(0, 64, (10, 64)).astype(np.float32)
    X = np.repeat(base, 3000, axis=0)
    rng.shuffle(X)
    Qs = base[rng.integers(0, 10, Q)]
    k = 100
    d, i, st = run(engine, X, Qs, k, precision=engine.PREC_BF16, shortlist=2)
    assert st["scan"] == 1 and st["kp"] == 208
    assert engine.last_fixups() == Q
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


def test_long_shortlist_needs_the_scan(engine):
    X, Qs = ints(5000, 10, 32, 3)
    with pytest.raises(engine.KnnsError) as e:
        run(engine, X, Qs, 100, precision=engine.PREC_BF16, shortlist=2)
    assert e.value.code == engine.ERR_UNSUPPORTED


# ---------------------------------------------------------------- accumulator variants of the scan
@pytest.mark.parametrize("D,form", [(128, "exact"), (256, "exact"), (72, "exact"), (128, "fp8"), (256, "bf16")])
def test_scan_accumulator_variants_agree(engine, oracle, D, form):
    # two accumulators of 224 (192) columns or four of 96: same keys, same candidates, same answers
    # (integer data: bit-exact against the oracle; E4M3-exact data for the FP8 form)
    rng = np.random.default_rng(D + len(form))
    if form == "fp8":
        # integers in [-7, 7] with one +-7 per row: E4M3 codes and scales are exact
        X = rng.integers(-7, 8, (60000, D)).astype(np.float32)
        X[:, 0] = 7.0
        Qs = rng.integers(-7, 8, (300, D)).astype(np.float32)
        Qs[:, 0] = -7.0
        kw = dict(precision=engine.PREC_FP8, shortlist=2)
    else:
        X, Qs = ints(60000, 300, D, 3 * D)
        kw = {} if form == "exact" else dict(precision=engine.PREC_BF16, shortlist=2)
    k = 32
    out = {}
    for accs in (2, 4):
        d, i, st = run(engine, X, Qs, k, scan=engine.SCAN_ON, scan_accs=accs, **kw)
        assert st["scan"] == 1
        out[accs] = (d, i)
    np.testing.assert_array_equal(out[2][1], out[4][1])
    np.testing.assert_array_equal(out[2][0], out[4][0])
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(out[4][1], oi)
    assert engine.last_fixups() <= 3
