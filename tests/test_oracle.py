"""The CPU oracle against the known-answer fixtures and independent restatements (no GPU)."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "knn_known_answers.npz")
CASES = ["square", "line", "small_int", "descriptor", "duplicates"]


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_known_answers(oracle, golden, name):
    Y, X, k = golden[f"{name}_corpus"], golden[f"{name}_queries"], int(golden[f"{name}_k"])
    d, i = oracle.knn_gemm(Y, X, k)
    np.testing.assert_array_equal(i, golden[f"{name}_idx"])
    np.testing.assert_array_equal(d, golden[f"{name}_dist"])


@pytest.mark.parametrize("name", CASES)
def test_fp64_oracle_matches_known_answers(oracle, golden, name):
    Y, X, k = golden[f"{name}_corpus"], golden[f"{name}_queries"], int(golden[f"{name}_k"])
    d, i = oracle.knn_f64(Y, X, k)
    np.testing.assert_array_equal(i, golden[f"{name}_idx"])
    np.testing.assert_array_equal(d.astype(np.float32), golden[f"{name}_dist"])


def test_square_by_hand(golden):
    # corners (0,0),(1,0),(0,1),(1,1); query (0.5,0.5) ties all four -> 0,1,2,3
    np.testing.assert_array_equal(golden["square_idx"][1], [0, 1, 2, 3])
    np.testing.assert_array_equal(golden["square_dist"][1], [0.5, 0.5, 0.5, 0.5])
    np.testing.assert_array_equal(golden["square_idx"][0], [0, 1, 2, 3])
    np.testing.assert_array_equal(golden["square_dist"][0], [0, 1, 1, 2])


def test_merge_restatement(oracle, golden):
    md, mi = oracle.merge_replace_max(golden["merge_dist_in"], golden["merge_idx_in"])
    np.testing.assert_array_equal(md, golden["merge_dist"])
    np.testing.assert_array_equal(mi, golden["merge_idx"])


def test_transpose_restatement(oracle):
    src = np.arange(12, dtype=np.float32)   # N=3 rows of Q=4
    t = oracle.transpose(src, 3, 4)
    np.testing.assert_array_equal(t.reshape(4, 3), src.reshape(3, 4).T)


def test_gemm_oracle_against_numpy_float64(oracle):
    rng = np.random.default_rng(7)
    Y = rng.random((2500, 37), dtype=np.float32)
    X = rng.random((40, 37), dtype=np.float32)
    d, i = oracle.knn_gemm(Y, X, 12)
    cn = oracle.norms(Y).astype(np.float64)
    keys = cn[None, :] - 2 * (X.astype(np.float64) @ Y.astype(np.float64).T)
    ref = np.argsort(keys, axis=1, kind="stable")[:, :12]
    # FP32 GEMM-form keys versus FP64 keys: differences only between near-equal candidates
    d64 = oracle.pair_dist_f64(Y, X, i)
    r64 = oracle.pair_dist_f64(Y, X, ref.astype(np.int32))
    diff = i != ref
    assert np.all(np.abs(d64[diff] - r64[diff]) <= 1e-5 * np.abs(r64[diff]))


def test_rerank_mode_sorted_and_exact(oracle):
    rng = np.random.default_rng(8)
    Y = rng.random((3000, 64), dtype=np.float32)
    X = rng.random((30, 64), dtype=np.float32)
    d, i = oracle.knn_gemm(Y, X, 20, kp=32, rerank=True)
    assert (np.diff(d, axis=1) >= 0).all()
    st = oracle.check_parity(Y, X, 20, d, i, gap_rel=1e-6, dist_rel=1e-6)
    assert st["queries"] == 30


def test_parity_checker_catches_a_planted_mistake(oracle):
    rng = np.random.default_rng(9)
    Y = rng.random((1000, 16), dtype=np.float32)
    X = rng.random((10, 16), dtype=np.float32)
    d, i = oracle.knn_gemm(Y, X, 5, kp=32, rerank=True)
    bad = i.copy()
    bad[3, 2] = (bad[3, 2] + 500) % 1000          # a wrong neighbour
    with pytest.raises(AssertionError):
        oracle.check_parity(Y, X, 5, d, bad)
    dbad = d.copy()
    dbad[0, 0] *= 1.001                           # a wrong distance
    with pytest.raises(AssertionError):
        oracle.check_parity(Y, X, 5, dbad, i)


def test_oracle_rejects_bad_sizes(oracle):
    Y = np.zeros((5, 3), np.float32)
    X = np.zeros((2, 3), np.float32)
    with pytest.raises(ValueError):
        oracle.knn_gemm(Y, X, 6)
    with pytest.raises(ValueError):
        oracle.knn_f64(Y, X, 0)


def test_synthetic_generators_are_seeded():
    import cuknns.synth as S
    a, qa = S.int_descriptor(1000, 128, seed=1, nq=10)
    b, qb = S.int_descriptor(1000, 128, seed=1, nq=10)
    assert np.array_equal(a, b) and np.array_equal(qa, qb)
    assert a.min() == 0 and a.max() <= 255 and np.array_equal(a, np.rint(a))
    assert ((a == 0).sum(1) >= 10).all()
    u, _ = S.uniform(100, 128, seed=0)
    assert u.dtype == np.float32 and 0 <= u.min() and u.max() < 1


def _ref_merge_lib():
    # the reference's own host merges, compiled from its sources where they are
    # mounted (oracle/build_ref.py); absent elsewhere
    import build_ref
    if not build_ref.available():
        pytest.skip("reference sources not mounted: merge pin not built")
    build_ref.build_if_available()
    return build_ref.load()


@pytest.mark.parametrize("which", ["bitonic", "heap"])
def test_merge_restatement_pinned_to_reference_code(oracle, which):
    # mergeResBitonic (src/cuknnBitonic.cu:381-417) and mergeResHeap
    # (src/cuknnHeap.cu:26-59) run on the same per-stream lists as the oracle's
    # restatement: list 0 (values and indices, in its unsorted slot order) must match
    # bit for bit, ties included (a value equal to the current maximum never replaces it)
    import ctypes
    fn = getattr(_ref_merge_lib(), "ref_merge_" + which)
    fp = ctypes.POINTER(ctypes.c_float)
    fn.argtypes = [fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    fn.restype = None
    rng = np.random.default_rng(31 if which == "bitonic" else 32)
    for L, Q, k, tied in [(1, 5, 4, False), (2, 37, 1, True), (4, 37, 16, True), (7, 20, 5, False),
                          (3, 64, 32, True), (8, 9, 100, False)]:
        if tied:
            d = rng.integers(0, 6, (L, Q, k)).astype(np.float32)
        else:
            d = rng.standard_normal((L, Q, k)).astype(np.float32)
        i = rng.permutation(L * Q * k).astype(np.float32).reshape(L, Q, k)
        rd, ri = d.copy(), i.copy()
        fn(rd.ctypes.data_as(fp), ri.ctypes.data_as(fp), k, Q, L)
        od, oi = oracle.merge_replace_max(d, i)
        np.testing.assert_array_equal(od, rd[0])
        np.testing.assert_array_equal(oi, ri[0])


def test_reference_recipe_is_inert_without_the_sources(monkeypatch, tmp_path):
    # with neither a mounted reference nor a staged copy the recipe builds nothing and
    # reports it, so build() never depends on the reference
    import build_ref
    monkeypatch.setenv("KNN_REFERENCE_DIR", str(tmp_path / "absent"))
    monkeypatch.setattr(build_ref, "MOUNT", str(tmp_path / "absent"))
    monkeypatch.setattr(build_ref, "STAGED", str(tmp_path / "staged"))
    assert not build_ref.available()
    assert build_ref.stage() is False
    assert build_ref.build_if_available() is False


def test_reference_recipe_stages_unmodified_sources(monkeypatch, tmp_path):
    # a reference tree named by KNN_REFERENCE_DIR is staged file for file, byte for byte
    import build_ref
    ref = tmp_path / "ref"
    for f in build_ref.FILES:
        (ref / f).parent.mkdir(parents=True, exist_ok=True)
        (ref / f).write_bytes(("// " + f + "\n").encode())
    monkeypatch.setenv("KNN_REFERENCE_DIR", str(ref))
    monkeypatch.setattr(build_ref, "MOUNT", str(tmp_path / "absent"))
    monkeypatch.setattr(build_ref, "STAGED", str(tmp_path / "staged"))
    assert build_ref.mounted_dir() == str(ref)
    assert build_ref.stage() is True
    for f in build_ref.FILES:
        assert (tmp_path / "staged" / f).read_bytes() == (ref / f).read_bytes()
    monkeypatch.delenv("KNN_REFERENCE_DIR")
    assert build_ref.source_dir() == str(tmp_path / "staged")
