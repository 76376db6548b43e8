"""Double-precision library (the reference's libcuknn_double) and the file-based
drivers knn_test / knn_test_double (src/knnTest.cu interface).

Bar for the double library: the exact FP64 top-k by (direct-difference distance,
index) -- indices and distances identical to the FP64 oracle of the FP64 inputs
(oracle_knn_f64d: the same distance, summed in d order with separate multiply
and add).  The reference's own double tests hold distances to a 1e-7 / 1e-6
norm tolerance (demo/Testbin.m:86, demo/knnTestDouble.m:30); identity is
stronger.  The float driver is held to the parity bars of test_gpu_parity.py.
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "knn-toolbox_gb300", "_build")


@pytest.mark.parametrize("N,Q,D,k", [(3000, 40, 17, 5), (20000, 130, 128, 100), (150_000, 64, 96, 32),
                                     (500, 7, 3, 500)])
def test_double_library_exact(engine, oracle, N, Q, D, k):
    rng = np.random.default_rng(N + D)
    X = rng.standard_normal((N, D))
    Qs = rng.standard_normal((Q, D))
    d, i = engine.search_host_f64(X, Qs, k)
    od, oi = oracle.knn_f64d(X, Qs, k)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


def test_double_library_near_duplicates_fall_back(engine, oracle):
    # 200 rows per base vector that differ below FP32 resolution: more FP32 ties than the
    # shortlist holds, so the acceptance test fails and the FP64 search decides
    rng = np.random.default_rng(3)
    base = rng.standard_normal((50, 16))
    X = np.repeat(base, 200, axis=0) + 1e-12 * rng.standard_normal((10000, 16))
    Qs = base[:20] + 1e-13 * rng.standard_normal((20, 16))
    k = 60
    d, i = engine.search_host_f64(X, Qs, k)
    od, oi = oracle.knn_f64d(X, Qs, k)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


def test_double_dropin(engine, oracle):
    rng = np.random.default_rng(4)
    X = rng.random((6000, 50))
    Qs = rng.random((33, 50))
    vals, idxs, t = engine.gpuknnsBitonic_f64(Qs, X, 8)
    od, oi = oracle.knn_f64d(X, Qs, 8)
    np.testing.assert_array_equal(idxs.astype(np.int64), oi)
    np.testing.assert_array_equal(vals, od)
    assert t > 0


@pytest.mark.parametrize("double", [False, True])
def test_file_driver(engine, oracle, tmp_path, double):
    rng = np.random.default_rng(5)
    dt = np.float64 if double else np.float32
    N, Q, D, k = 4096, 60, 20, 12
    X = rng.random((N, D)).astype(dt)
    Qs = rng.random((Q, D)).astype(dt)
    X.tofile(tmp_path / "data.bin")
    Qs.tofile(tmp_path / "queries.bin")
    exe = os.path.join(BUILD, "knn_test_double" if double else "knn_test")
    r = subprocess.run([exe, "data.bin", "queries.bin", str(N), str(Q), str(D), str(k)], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Time Elapsed:" in r.stdout
    dist = np.fromfile(tmp_path / "KNNdist.bin", dt).reshape(Q, k)   # demo/importData.m: [k Q]
    idx = np.fromfile(tmp_path / "KNNidx.bin", dt).reshape(Q, k)
    if double:
        od, oi = oracle.knn_f64d(X, Qs, k)
        np.testing.assert_array_equal(idx.astype(np.int64), oi)
        np.testing.assert_array_equal(dist, od)
    else:
        oracle.check_parity(X, Qs, k, dist, idx.astype(np.int64), gap_rel=1e-6, dist_rel=1e-5)
    # a short input file is an error, not a search of uninitialised memory
    r = subprocess.run([exe, "data.bin", "queries.bin", str(N + 1), str(Q), str(D), str(k)], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 1
