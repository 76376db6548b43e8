"""Parity with the reference's own CUDA library.

tests/golden/ref_uniform64k.npz and tests/golden/ref_int1m_q1000.npz hold the
answers of the reference's heap driver gpuknnsHeap (src/cuknnHeap.cu:394-575),
built from the reference's sources and run on a GB300 by
tests/golden/make_ref_fixtures.py (numStreams = 1; that script says why the
bitonic driver is not run):

* 65,536 x 128 uniform [0,1) corpus, its 1,024 queries, k = 16, seed 0;
* 1,000,000 x 128 integer-descriptor corpus, seed 1, the first 1,000 of its
  10,000 queries, k = 128 (the drivers need a power of two; the comparison
  sorts the reference's list by (distance, index) and keeps 100, the
  workload's k).

The bar (the reference's output contract: unordered top-k, distances including
||q||^2, readme.txt:61-69): both lists are ordered by FP64 direct-difference
distance (ties by index); wherever the engine's and the reference's indices
differ at a rank, the two candidates' FP64 distances differ by less than the
tie gap.  On the integer corpus every product and sum of the reference's FP32
SGEMM is exact, so the gap is the stated 1e-6 relative (in practice only exact
ties differ).  On the uniform corpus the reference ranks by its FP32 GEMM-form
key ||c||^2 - 2 q.c, whose rounding error is bounded by gamma_{D+2} (||c||^2 +
2 sum|q_d c_d| + ||q||^2) (gamma_n = n u / (1 - n u), u = 2^-24); the gap there
is the larger of 1e-6 relative and the sum of the two candidates' bounds.  The
engine's distances are held to 1e-5 relative of FP64 as everywhere.
"""
import hashlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
GAP = 1e-6
DIST_REL = 1e-5
U = 2.0 ** -24


def _fixture(name):
    p = os.path.join(GOLD, name)
    if not os.path.exists(p):
        pytest.fail(f"missing reference fixture {p} (tests/golden/make_ref_fixtures.py writes it)")
    return np.load(p)


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _inputs_uniform():
    import cuknns.synth as S
    return S.uniform(65_536, 128, seed=0, nq=1_024)


def _inputs_int(nq):
    import cuknns.synth as S
    X, Qs = S.int_descriptor(1_000_000, 128, seed=1, nq=10_000)
    return X, np.ascontiguousarray(Qs[:nq])


def _key_err_bound(X, Qs, idx):
    """Bound on the rounding error of the reference's FP32 key ||c||^2 - 2 q.c + ||q||^2 per pair."""
    D = X.shape[1]
    g = (D + 2) * U / (1 - (D + 2) * U)
    Xa, Qa = np.abs(X).astype(np.float64), np.abs(Qs).astype(np.float64)
    c2 = (X.astype(np.float64) ** 2).sum(1)
    q2 = (Qs.astype(np.float64) ** 2).sum(1)
    out = np.empty(idx.shape, np.float64)
    for q in range(idx.shape[0]):
        dots = Xa[idx[q]] @ Qa[q]
        out[q] = g * (c2[idx[q]] + 2 * dots + q2[q])
    return out


def _by_fp64(oracle, X, Qs, idx):
    """Sort each row of idx by (FP64 distance, index); returns (idx, d64)."""
    d64 = oracle.pair_dist_f64(X, Qs, idx.astype(np.int32))
    out_i, out_d = np.empty_like(idx), np.empty_like(d64)
    for q in range(idx.shape[0]):
        o = np.lexsort((idx[q], d64[q]))
        out_i[q], out_d[q] = idx[q][o], d64[q][o]
    return out_i, out_d


def _compare(oracle, X, Qs, got_idx, ref_idx, gap_fn):
    """Rank-by-rank comparison in FP64 order; returns (positions differing, largest relative gap there)."""
    gi, gd = _by_fp64(oracle, X, Qs, got_idx)
    ri, rd = _by_fp64(oracle, X, Qs, ref_idx)
    diff = gi != ri
    worst = 0.0
    for q, j in np.argwhere(diff):
        a, b = gd[q, j], rd[q, j]
        tol = gap_fn(q, gi[q, j], ri[q, j], a, b)
        rel = abs(a - b) / max(a, b, 1e-300)
        worst = max(worst, rel)
        assert abs(a - b) <= tol, (f"query {q} rank {j}: engine {gi[q, j]} (d={a!r}) vs reference "
                                   f"{ri[q, j]} (d={b!r}), gap {abs(a - b):.3e} > {tol:.3e}")
    return int(diff.sum()), worst


def _reference_topk(dist, idx, k):
    """The reference's k-leading list sorted by (its distance, index), first k kept."""
    out = np.empty((idx.shape[0], k), idx.dtype)
    for q in range(idx.shape[0]):
        o = np.lexsort((idx[q], dist[q]))
        out[q] = idx[q][o][:k]
    return out


# ---------------------------------------------------------------- fixtures themselves (CPU)
def test_reference_fixture_inputs_regenerate():
    # the seeded generators rebuild exactly the inputs the reference was run on
    f = _fixture("ref_uniform64k.npz")
    X, Qs = _inputs_uniform()
    assert _sha(X) == str(f["corpus_sha256"]) and _sha(Qs) == str(f["queries_sha256"])
    g = _fixture("ref_int1m_q1000.npz")
    X, Qs = _inputs_int(int(g["Q"]))
    assert _sha(X) == str(g["corpus_sha256"]) and _sha(Qs) == str(g["queries_sha256"])


def test_reference_answers_are_exact_on_integer_data(oracle):
    # the reference's own answers on the integer corpus: its FP32 arithmetic is exact there,
    # so its top-100 agrees with the FP64 oracle's up to exact ties (a sample of queries)
    g = _fixture("ref_int1m_q1000.npz")
    X, Qs = _inputs_int(int(g["Q"]))
    sub = np.arange(0, int(g["Q"]), 20)
    ref = _reference_topk(g["heap_dist"][sub], g["heap_idx"][sub], 100)
    ex_d, ex_i = oracle.knn_f64(X, Qs[sub], 100)
    n, worst = _compare(oracle, X, Qs[sub], ex_i, ref, lambda *a: 0.0)
    assert worst == 0.0
    # and its distances are the exact integers (key + ||q||^2 computed exactly)
    d64 = oracle.pair_dist_f64(X, Qs[sub], g["heap_idx"][sub].astype(np.int32))
    np.testing.assert_array_equal(g["heap_dist"][sub].astype(np.float64), d64)


# ---------------------------------------------------------------- the engine against the reference (GPU)
@pytest.mark.gpu
def test_engine_matches_reference_uniform_65536x128_k16(engine, oracle):
    import torch
    f = _fixture("ref_uniform64k.npz")
    X, Qs = _inputs_uniform()
    k = 16
    d, i = engine.search(torch.from_numpy(X).cuda(), torch.from_numpy(Qs).cuda(), k)
    d, i = d.cpu().numpy(), i.cpu().numpy()
    oracle.check_parity(X, Qs, k, d, i, gap_rel=GAP, dist_rel=DIST_REL)
    for drv in ("heap",):
        ref = f[f"{drv}_idx"]
        assert ref.shape == (1024, k)
        eps_g = _key_err_bound(X, Qs, i)
        eps_r = _key_err_bound(X, Qs, ref)
        gi, _ = _by_fp64(oracle, X, Qs, i)
        ri, _ = _by_fp64(oracle, X, Qs, ref)
        pos_g = {(q, n): e for q in range(len(i)) for n, e in zip(i[q], eps_g[q])}
        pos_r = {(q, n): e for q in range(len(ref)) for n, e in zip(ref[q], eps_r[q])}

        def gap(q, a_idx, b_idx, a, b):
            return max(GAP * max(a, b), pos_g[(q, a_idx)] + pos_r[(q, b_idx)])
        n, worst = _compare(oracle, X, Qs, i, ref, gap)
        # almost every rank agrees
        assert n <= 0.01 * ref.size, (drv, n)


@pytest.mark.gpu
def test_engine_matches_reference_int_1m_x128_k100(engine, oracle):
    import torch
    g = _fixture("ref_int1m_q1000.npz")
    X, Qs = _inputs_int(int(g["Q"]))
    k = 100
    d, i = engine.search(torch.from_numpy(X).cuda(), torch.from_numpy(Qs).cuda(), k)
    d, i = d.cpu().numpy(), i.cpu().numpy()
    ref = _reference_topk(g["heap_dist"], g["heap_idx"], k)
    n, worst = _compare(oracle, X, Qs, i, ref, lambda q, a_idx, b_idx, a, b: GAP * max(a, b))
    # differences only between exactly tied candidates
    assert worst == 0.0
    # distances: exact integers, equal to FP64
    d64 = oracle.pair_dist_f64(X, Qs, i)
    np.testing.assert_array_equal(d.astype(np.float64), d64)
