"""Parity of the CUDA engine against the CPU oracle (run on a GB300).

Bars, as written in each test:
* indices: identical to the oracle's, except where the FP64 distances of the
  two competing candidates differ by less than 1e-6 relative;
* distances: within 1e-5 relative of the FP64 oracle (re-rank mode);
* bit-exact equality where the arithmetic is exact or shares the oracle's
  convention (CUDA-core path; integer-valued data on the tensor-core path).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAP = 1e-6
DIST_REL = 1e-5


def _torch():
    import torch
    return torch


def run(engine, X, Qs, k, **kw):
    torch = _torch()
    c = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    q = torch.from_numpy(np.ascontiguousarray(Qs)).cuda()
    d, i = engine.search(c, q, k, **kw)
    return d.cpu().numpy(), i.cpu().numpy(), engine.last_stats()


def data_uniform(n, q, d, seed):
    rng = np.random.default_rng(seed)
    return rng.random((n, d), dtype=np.float32), rng.random((q, d), dtype=np.float32)


def data_int(n, q, d, seed, hi=256):
    rng = np.random.default_rng(seed)
    return (rng.integers(0, hi, (n, d)).astype(np.float32), rng.integers(0, hi, (q, d)).astype(np.float32))


# ---------------------------------------------------------------- tensor-core dot tile
@pytest.mark.parametrize("D", [128, 96, 43, 8])
def test_tc_dot_tile_matches_fp64(engine, D):
    torch = _torch()
    X, Qs = data_uniform(200, 150, D, 10 + D)
    X = (X - 0.5).astype(np.float32)
    dump = engine.debug_tc_dot_tile(torch.from_numpy(X).cuda(), torch.from_numpy(Qs).cuda()).cpu().numpy()
    ref = Qs[:128].astype(np.float64) @ X[:128].astype(np.float64).T
    scale = np.abs(Qs[:128]).astype(np.float64) @ np.abs(X[:128]).astype(np.float64).T
    err = np.abs(dump.astype(np.float64) - ref)
    # 3xTF32 with FP32 accumulation: a few FP32 ulps of sum |q_d c_d|
    assert (err <= 2e-6 * scale + 1e-30).all(), float((err / scale).max())


def test_tc_dot_tile_integers_exact(engine):
    torch = _torch()
    X, Qs = data_int(128, 128, 128, 5)
    dump = engine.debug_tc_dot_tile(torch.from_numpy(X).cuda(), torch.from_numpy(Qs).cuda()).cpu().numpy()
    ref = Qs.astype(np.float64) @ X.astype(np.float64).T
    assert np.array_equal(dump.astype(np.float64), ref)


# ---------------------------------------------------------------- CUDA-core path: bit-exact vs oracle
@pytest.mark.parametrize("N,Q,D,k", [(3000, 77, 43, 16), (1000, 130, 128, 8), (777, 33, 5, 1)])
def test_simt_reference_semantics_bit_exact(engine, oracle, N, Q, D, k):
    X, Qs = data_uniform(N, Q, D, N + D)
    d, i, st = run(engine, X, Qs, k, algo=engine.ALGO_SIMT, rerank=False)
    assert st["algo"] == engine.ALGO_SIMT
    od, oi = oracle.knn_gemm(X, Qs, k)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


@pytest.mark.parametrize("N,Q,D,k,kp", [(3000, 77, 43, 16, 32), (2048, 64, 200, 100, 128),
                                        (4000, 40, 64, 200, 256)])
def test_simt_rerank_bit_exact(engine, oracle, N, Q, D, k, kp):
    X, Qs = data_uniform(N, Q, D, N * 3 + D)
    d, i, st = run(engine, X, Qs, k, algo=engine.ALGO_SIMT, kp=kp)
    od, oi = oracle.knn_gemm(X, Qs, k, kp=kp, rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)
    oracle.check_parity(X, Qs, k, d, i, gap_rel=GAP, dist_rel=DIST_REL)


# ---------------------------------------------------------------- tensor-core path
@pytest.mark.parametrize("N,Q,D,k", [(5000, 200, 128, 16), (4097, 129, 96, 10), (1500, 64, 43, 32),
                                     (2000, 300, 128, 100), (300, 5, 8, 3)])
def test_tc_rerank_parity(engine, oracle, N, Q, D, k):
    X, Qs = data_uniform(N, Q, D, 7 * N + D)
    d, i, st = run(engine, X, Qs, k, algo=engine.ALGO_TC)
    assert st["algo"] == engine.ALGO_TC
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    oracle.check_parity(X, Qs, k, d, i, ref_idx=oi, gap_rel=GAP, dist_rel=DIST_REL)
    # same shortlist convention as the oracle: the results agree everywhere in practice
    assert (i == oi).mean() > 0.999


@pytest.mark.parametrize("N,Q,D,k", [(5000, 200, 128, 16), (2000, 300, 128, 100), (1000, 50, 96, 10)])
def test_tc_reference_semantics_parity(engine, oracle, N, Q, D, k):
    X, Qs = data_uniform(N, Q, D, 11 * N + D)
    d, i, st = run(engine, X, Qs, k, algo=engine.ALGO_TC, rerank=False)
    od, oi = oracle.knn_gemm(X, Qs, k)
    # Ranking by the FP32 GEMM-form key (the reference's own algorithm) carries
    # an absolute key error of a few FP32 ulps of ||q||^2 + ||c||^2, about 1e-6
    # of the distance on this data, so two FP32 implementations may order
    # candidates whose FP64 distances differ by less than ~2e-5 differently.
    # The default re-rank mode is held to the 1e-6 gap instead.
    oracle.check_parity(X, Qs, k, d, i, ref_idx=oi, gap_rel=2e-5, dist_rel=1e-4)
    np.testing.assert_allclose(d, od, rtol=2e-5, atol=2e-5 * np.abs(od).max())


@pytest.mark.parametrize("rerank", [True, False])
def test_tc_integer_data_bit_exact(engine, oracle, rerank):
    import cuknns.synth as S
    X, Qs = S.int_descriptor(20000, 128, seed=1, nq=300)
    k = 100
    d, i, st = run(engine, X, Qs, k, algo=engine.ALGO_TC, rerank=rerank)
    if rerank:
        od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    else:
        od, oi = oracle.knn_gemm(X, Qs, k)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


@pytest.mark.parametrize("splits", [1, 2, 3, 7])
@pytest.mark.parametrize("algo", [1, 2])
def test_splits_do_not_change_results(engine, oracle, splits, algo):
    X, Qs = data_int(3000, 140, 32, 3, hi=8)   # many exact ties
    k = 20
    d, i, st = run(engine, X, Qs, k, algo=algo, splits=splits)
    assert 1 <= st["splits"] <= splits
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


# ---------------------------------------------------------------- edge cases
@pytest.mark.parametrize("case", ["k_equals_n", "single_query", "n_below_kp", "duplicates", "all_equal",
                                  "d1", "d129_auto_simt", "k128_tc", "k512_simt"])
def test_edge_cases(engine, oracle, case):
    rng = np.random.default_rng(sum(map(ord, case)))
    k = 10
    if case == "k_equals_n":
        X, Qs = data_uniform(40, 17, 16, 1); k = 40
    elif case == "single_query":
        X, Qs = data_uniform(5000, 1, 128, 2)
    elif case == "n_below_kp":
        X, Qs = data_uniform(20, 50, 24, 3); k = 12
    elif case == "duplicates":
        base = rng.random((50, 64), dtype=np.float32)
        X = np.repeat(base, 20, axis=0)
        Qs = base[:30].copy()
        k = 25
    elif case == "all_equal":
        X = np.ones((500, 32), np.float32)
        Qs = np.zeros((10, 32), np.float32)
    elif case == "d1":
        X, Qs = data_uniform(3000, 100, 1, 4)
    elif case == "d129_auto_simt":
        X, Qs = data_uniform(1000, 40, 129, 5)
    elif case == "k128_tc":
        X, Qs = data_uniform(3000, 130, 64, 6); k = 128
    elif case == "k512_simt":
        X, Qs = data_uniform(3000, 40, 16, 7); k = 512
    d, i, st = run(engine, X, Qs, k)
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    oracle.check_parity(X, Qs, k, d, i, ref_idx=oi, gap_rel=GAP, dist_rel=DIST_REL, dist_abs=1e-6)
    if case in ("duplicates", "all_equal"):
        np.testing.assert_array_equal(i, oi)  # exact ties: lower index first
    if case == "d129_auto_simt":
        assert st["algo"] == engine.ALGO_SIMT


def test_empty_query_batch(engine):
    torch = _torch()
    X, _ = data_uniform(100, 1, 16, 0)
    d, i = engine.search(torch.from_numpy(X).cuda(), torch.empty((0, 16), device="cuda"), 5)
    assert d.shape == (0, 5)


def test_invalid_arguments(engine):
    torch = _torch()
    X, Qs = data_uniform(10, 3, 8, 0)
    c, q = torch.from_numpy(X).cuda(), torch.from_numpy(Qs).cuda()
    with pytest.raises(engine.KnnsError) as e:
        engine.search(c, q, 11)
    assert e.value.code == engine.ERR_INVALID
    with pytest.raises(engine.KnnsError) as e:
        engine.search(c, q, 4, kp=40)
    assert e.value.code == engine.ERR_INVALID
    with pytest.raises(engine.KnnsError) as e:
        engine.search(torch.zeros((600, 256), device="cuda"), torch.zeros((2, 256), device="cuda"), 4,
                      algo=engine.ALGO_TC)
    assert e.value.code == engine.ERR_UNSUPPORTED
    # the engine is still usable afterwards
    d, i = engine.search(c, q, 4)
    assert i.shape == (3, 4)


# ---------------------------------------------------------------- reference C API and toolbox
def test_dropin_c_api(engine, oracle):
    X, Qs = data_uniform(4096, 300, 128, 21)
    k = 32
    for fn in (engine.gpuknnsBitonic, engine.gpuknnsHeap):
        vals, idxf, t = fn(Qs, X, k, 1)
        assert t > 0
        i = idxf.astype(np.int64)
        assert np.array_equal(idxf, i.astype(np.float32))
        oracle.check_parity(X, Qs, k, vals, i, gap_rel=GAP, dist_rel=DIST_REL)
    plan = engine.knnsplan(4096, 300, 128, k)
    assert (plan.objects, plan.numQueries, plan.dimentions, plan.k) == (4096, 300, 128, k)
    KNNdist, KNNidx = engine.knnsexecute(plan, X, Qs)
    oracle.check_parity(X, Qs, k, KNNdist, KNNidx.astype(np.int64), gap_rel=GAP, dist_rel=DIST_REL)


def test_toolbox_semantics(engine, oracle):
    X, Qs = data_uniform(2000, 50, 43, 22)
    dist, idx, t = engine.gpuknnBitonic(Qs.T, X.T, 16, 1)
    assert dist.shape == (16, 50) and idx.shape == (16, 50)
    assert (idx >= 1).all()                       # 1-based
    assert (np.diff(dist, axis=0) >= 0).all()     # columns sorted
    od, oi = oracle.knn_f64(X, Qs, 16)
    ns = np.abs(od).max()
    assert np.linalg.norm(dist.T - od) / ns < 1e-2   # demo/knnTest.m:31 pass criterion


# ---------------------------------------------------------------- benchmark workloads
def test_uniform_65536x128_q1024_k16(engine, oracle):
    import cuknns.synth as S
    X, Qs = S.uniform(65536, 128, seed=0, nq=1024)
    d, i, st = run(engine, X, Qs, 16)
    assert st["algo"] == engine.ALGO_TC
    sub = slice(0, 256)
    od, oi = oracle.knn_gemm(X, Qs[sub], 16, kp=st["kp"], rerank=True)
    oracle.check_parity(X, Qs[sub], 16, d[sub], i[sub], ref_idx=oi, gap_rel=GAP, dist_rel=DIST_REL)


def test_int_1m_x128_q10000_k100(engine, oracle):
    import cuknns.synth as S
    X, Qs = S.int_descriptor(1_000_000, 128, seed=1, nq=10_000)
    d, i, st = run(engine, X, Qs, 100)
    assert st["algo"] == engine.ALGO_TC
    # size-independent properties on every query
    assert (np.diff(d, axis=1) >= 0).all()
    assert (i >= 0).all() and (i < X.shape[0]).all()
    srt = np.sort(i, axis=1)
    assert (np.diff(srt, axis=1) != 0).all()
    # exact integer arithmetic: bit-exact against the oracle on a query sample
    sub = np.arange(0, 10_000, 97)
    od, oi = oracle.knn_gemm(X, Qs[sub], 100, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i[sub], oi)
    np.testing.assert_array_equal(d[sub], od)


# ---------------------------------------------------------------- threshold seeding (pilot pass)
@pytest.mark.parametrize("algo", [1, 2])
@pytest.mark.parametrize("kind", ["uniform", "int"])
def test_pilot_does_not_change_results(engine, oracle, algo, kind):
    import cuknns.synth as S
    if kind == "uniform":
        X, Qs = S.uniform(70000, 64, seed=3, nq=200)
    else:
        X, Qs = S.int_descriptor(70000, 64, seed=4, nq=200)
    k = 24
    # the pilot belongs to the shortlist kernels (without the threshold scan)
    off = dict(algo=algo, scan=engine.SCAN_OFF)
    d0, i0, st0 = run(engine, X, Qs, k, pilot=False, **off)
    d1, i1, st1 = run(engine, X, Qs, k, pilot=True, **off)
    assert st0["pilot"] == 0 and st1["pilot"] == 1
    np.testing.assert_array_equal(i0, i1)
    np.testing.assert_array_equal(d0, d1)
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st1["kp"], rerank=True)
    oracle.check_parity(X, Qs, k, d1, i1, ref_idx=oi, gap_rel=GAP, dist_rel=DIST_REL)


@pytest.mark.parametrize("algo", [1, 2])
def test_pilot_fixup_on_unrepresentative_sample(engine, oracle, algo):
    # Only every 16th corpus row (the pilot's sample) lies near the queries, so
    # the seeded threshold admits fewer than kp rows: the fix-up pass must redo
    # those query tiles and the result must still be exact.
    rng = np.random.default_rng(77)
    N, D, Q, k = 16 * 4096, 32, 150, 10
    Qs = rng.random((Q, D), dtype=np.float32)
    X = (10.0 + rng.random((N, D), dtype=np.float32)).astype(np.float32)
    near = np.arange(0, N, 16)
    X[near] = Qs[rng.integers(0, Q, near.size)] + 0.01 * rng.random((near.size, D), dtype=np.float32)
    d, i, st = run(engine, X, Qs, k, algo=algo, scan=engine.SCAN_OFF)
    assert st["pilot"] == 1
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    oracle.check_parity(X, Qs, k, d, i, ref_idx=oi, gap_rel=GAP, dist_rel=DIST_REL, dist_abs=1e-6)
    d0, i0, _ = run(engine, X, Qs, k, algo=algo, pilot=False, scan=engine.SCAN_OFF)
    np.testing.assert_array_equal(i, i0)
    # the TF32 threshold scan (the default at this size) on the same unrepresentative sample
    if algo == engine.ALGO_TC:
        d2, i2, st2 = run(engine, X, Qs, k)
        assert st2["scan"] == 1
        np.testing.assert_array_equal(i2, i0)


# ---------------------------------------------------------------- precision form: BF16 shortlist + exact re-rank
@pytest.mark.parametrize("D,c", [(96, 4), (256, 2)])
def test_bf16_shortlist_recall_and_exact_distances(engine, oracle, D, c):
    import cuknns.synth as S
    X, Qs = S.gauss_mixture(60000, D, seed=5, nq=120, centres=256)
    k = 10
    d, i, st = run(engine, X, Qs, k, precision=engine.PREC_BF16, shortlist=c)
    assert st["algo"] == engine.ALGO_TC and st["kp"] >= c * k
    ex = oracle.knn_f64(X, Qs, k)
    rec = oracle.recall_at_k(i, ex[1])
    assert rec >= 0.99, rec
    # every returned distance is the exact distance of the returned index (re-rank in FP32)
    got64 = oracle.pair_dist_f64(X, Qs, i)
    assert (np.abs(d - got64) <= 1e-5 * got64 + 1e-6).all()
    assert (np.diff(d, axis=1) >= 0).all()


def test_bf16_shortlist_on_bf16_exact_data_is_exact(engine, oracle):
    X, Qs = data_int(20000, 200, 64, 9)
    k = 16
    d, i, st = run(engine, X, Qs, k, precision=engine.PREC_BF16, shortlist=2)
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st["kp"], rerank=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


# ---------------------------------------------------------------- 3xTF32 keys on request
@pytest.mark.parametrize("N,scan", [(20000, 2), (150000, 0), (150000, 1)])
def test_tf32_only_gives_the_same_answers(engine, oracle, N, scan):
    # integer data are exact in BF16: by default the BF16 kernels (the shortlist kernel's BF16
    # variant without the scan, the BF16 threshold scan at N >= 131072) rank them; tf32_only
    # sends them through the 3xTF32 kernels instead (the shortlist kernel's TF32 variant, the
    # TF32 threshold scan run beside the BF16 one), whose keys are exact on this data as
    # well -- same answers, bit for bit
    import cuknns.synth as S
    X, Qs = S.int_descriptor(N, 128, seed=12, nq=257)
    k = 100
    d0, i0, st0 = run(engine, X, Qs, k, scan=scan)
    d1, i1, st1 = run(engine, X, Qs, k, tf32_only=True, scan=scan)
    assert st0["scan"] == st1["scan"] == (scan != 2)
    np.testing.assert_array_equal(i0, i1)
    np.testing.assert_array_equal(d0, d1)
    od, oi = oracle.knn_gemm(X, Qs, k, kp=st1["kp"], rerank=True)
    np.testing.assert_array_equal(i1, oi)
    np.testing.assert_array_equal(d1, od)
