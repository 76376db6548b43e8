"""CPU oracle for brute-force squared-L2 kNN -- test infrastructure only.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It is the checker, never the product: the
CUDA library under ``knn-toolbox_gb300/`` has no dependency on it.

The C restatement lives in ``oracle/knn_oracle.c`` (see its header for the
arithmetic conventions and the parity-pinning status).  This module builds it
with gcc and exposes numpy-level wrappers plus the parity checker used by the
tests (indices identical except where the FP64 gap between the competing
candidates is below a relative threshold; distances within a relative
tolerance of the FP64 oracle).
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile oracle/knn_oracle.c into oracle/_build/liboracle.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "knn_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-std=c11", "-Wall", "-Wno-unused-function"]
    if platform.machine() in ("x86_64", "AMD64"):
        # fmaf() is correctly rounded on every target; -mfma only makes it a
        # single instruction on x86 (aarch64 has FMA in its base ISA).
        cmd.append("-mfma")
    tmp = LIB_PATH + ".tmp"
    cmd += [src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        c_fp = ctypes.POINTER(ctypes.c_float)
        c_dp = ctypes.POINTER(ctypes.c_double)
        c_ip = ctypes.POINTER(ctypes.c_int32)
        L.oracle_norms.argtypes = [c_fp, ctypes.c_int64, ctypes.c_int, c_fp]
        L.oracle_knn_gemm.argtypes = [c_fp, ctypes.c_int64, c_fp, ctypes.c_int64, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, c_fp, c_ip,
                                      ctypes.c_int]
        L.oracle_knn_f64.argtypes = [c_fp, ctypes.c_int64, c_fp, ctypes.c_int64, ctypes.c_int,
                                     ctypes.c_int, c_dp, c_ip, ctypes.c_int]
        L.oracle_knn_f64d.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int64, ctypes.POINTER(ctypes.c_double),
                                      ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_int32), ctypes.c_int]
        L.oracle_pair_dist_f64.argtypes = [c_fp, ctypes.c_int64, c_fp, ctypes.c_int64,
                                           ctypes.c_int, c_ip, ctypes.c_int, c_dp]
        L.oracle_merge_replace_max.argtypes = [c_fp, c_fp, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int]
        L.oracle_merge_replace_max.restype = None
        L.oracle_transpose.argtypes = [c_fp, c_fp, ctypes.c_int, ctypes.c_int]
        L.oracle_transpose.restype = None
        L.oracle_max_threads.argtypes = []
        _lib = L
    return _lib


def _f(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def norms(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty(x.shape[0], np.float32)
    rc = lib().oracle_norms(_f(x), x.shape[0], x.shape[1], _f(out))
    assert rc == 0, rc
    return out


def knn_gemm(data, queries, k, kp=None, rerank=False, nthreads=0):
    """GEMM-form kNN (demo/knn.m).  Returns (dist[Q,k] float32, idx[Q,k] int32).

    ``kp=k, rerank=False`` is demo/knn.m exactly; ``rerank=True`` re-ranks the
    ``kp`` shortlist by the exact distance, as the CUDA engine's default mode.
    """
    data = np.ascontiguousarray(data, dtype=np.float32)
    queries = np.ascontiguousarray(queries, dtype=np.float32)
    N, D = data.shape
    Q = queries.shape[0]
    kp = k if kp is None else kp
    dist = np.empty((Q, k), np.float32)
    idx = np.empty((Q, k), np.int32)
    rc = lib().oracle_knn_gemm(_f(data), N, _f(queries), Q, D, k, kp, int(bool(rerank)),
                               _f(dist), _i(idx), nthreads)
    if rc != 0:
        raise ValueError(f"oracle_knn_gemm failed ({rc})")
    return dist, idx


def knn_f64(data, queries, k, nthreads=0):
    """Exact top-k by (FP64 direct-difference distance, index)."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    queries = np.ascontiguousarray(queries, dtype=np.float32)
    N, D = data.shape
    Q = queries.shape[0]
    dist = np.empty((Q, k), np.float64)
    idx = np.empty((Q, k), np.int32)
    rc = lib().oracle_knn_f64(_f(data), N, _f(queries), Q, D, k, _d(dist), _i(idx), nthreads)
    if rc != 0:
        raise ValueError(f"oracle_knn_f64 failed ({rc})")
    return dist, idx


def knn_f64d(data, queries, k, nthreads=0):
    """Exact top-k by (FP64 direct-difference distance, index) of FP64 inputs."""
    data = np.ascontiguousarray(data, dtype=np.float64)
    queries = np.ascontiguousarray(queries, dtype=np.float64)
    N, D = data.shape
    Q = queries.shape[0]
    dist = np.empty((Q, k), np.float64)
    idx = np.empty((Q, k), np.int32)
    rc = lib().oracle_knn_f64d(_d(data), N, _d(queries), Q, D, k, _d(dist), _i(idx), nthreads)
    if rc != 0:
        raise ValueError(f"oracle_knn_f64d failed ({rc})")
    return dist, idx


def pair_dist_f64(data, queries, idx):
    data = np.ascontiguousarray(data, dtype=np.float32)
    queries = np.ascontiguousarray(queries, dtype=np.float32)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    Q, m = idx.shape
    out = np.empty((Q, m), np.float64)
    rc = lib().oracle_pair_dist_f64(_f(data), data.shape[0], _f(queries), Q, data.shape[1],
                                    _i(idx), m, _d(out))
    assert rc == 0
    return out


def merge_replace_max(dist_lists, idx_lists):
    """Restatement of the reference host merge.  Inputs [L, Q, k]; returns list 0 merged."""
    d = np.ascontiguousarray(dist_lists, dtype=np.float32).copy()
    i = np.ascontiguousarray(idx_lists, dtype=np.float32).copy()
    L_, Q, k = d.shape
    lib().oracle_merge_replace_max(_f(d), _f(i), k, Q, L_)
    return d[0], i[0]


def transpose(src, N, Q):
    src = np.ascontiguousarray(src, dtype=np.float32)
    trg = np.empty(N * Q, np.float32)
    lib().oracle_transpose(_f(trg), _f(src), N, Q)
    return trg


# --------------------------------------------------------------------------
# Parity checker
# --------------------------------------------------------------------------

def check_parity(data, queries, k, got_dist, got_idx, ref_idx=None, gap_rel=1e-6,
                 dist_rel=1e-5, dist_abs=0.0, exact_f64=None):
    """Check a kNN result against the FP64 oracle.

    * every returned index is a valid, distinct corpus row;
    * the returned set equals the FP64 top-k set except for members whose FP64
      distance lies within ``gap_rel`` (relative) of the FP64 k-th distance
      (competing candidates at the boundary);
    * position by position, the returned index equals ``ref_idx`` (when given;
      else the FP64 order) unless the two candidates' FP64 distances differ by
      less than ``gap_rel`` relative;
    * returned distances are within ``dist_rel`` relative (+ ``dist_abs``) of
      the FP64 distance of the returned index.

    Returns a dict of statistics; raises AssertionError on a violation.
    """
    got_idx = np.asarray(got_idx).astype(np.int64)
    got_dist = np.asarray(got_dist, dtype=np.float64)
    Q = got_idx.shape[0]
    N = data.shape[0]
    assert got_idx.shape == (Q, k), got_idx.shape
    assert (got_idx >= 0).all() and (got_idx < N).all(), "index out of range"
    for q in range(Q):
        assert len(set(got_idx[q].tolist())) == k, f"duplicate index in query {q}"
    if exact_f64 is None:
        exact_f64 = knn_f64(data, queries, k)
    ex_d, ex_i = exact_f64
    got_d64 = pair_dist_f64(data, queries, got_idx.astype(np.int32))
    # distances
    err = np.abs(got_dist - got_d64)
    tol = dist_rel * np.abs(got_d64) + dist_abs
    bad = err > tol
    assert not bad.any(), (f"distance error: max rel {float((err / np.maximum(got_d64, 1e-300)).max()):.3e}"
                           f" at {np.argwhere(bad)[:5].tolist()}")
    # sets
    kth = ex_d[:, -1]
    set_mismatch = 0
    for q in range(Q):
        gs, es = set(got_idx[q].tolist()), set(ex_i[q].tolist())
        if gs == es:
            continue
        for n in gs ^ es:
            d = got_d64[q][list(got_idx[q]).index(n)] if n in gs else ex_d[q][list(ex_i[q]).index(n)]
            assert abs(d - kth[q]) <= gap_rel * max(abs(kth[q]), 1e-300), (
                f"query {q}: index {n} (d={d!r}) differs from FP64 top-k beyond the gap rule "
                f"(k-th={kth[q]!r})")
            set_mismatch += 1
    # positions
    cmp_idx = ex_i if ref_idx is None else np.asarray(ref_idx).astype(np.int64)
    cmp_d64 = pair_dist_f64(data, queries, cmp_idx.astype(np.int32))
    pos = got_idx != cmp_idx
    for q, j in np.argwhere(pos):
        a, b = got_d64[q, j], cmp_d64[q, j]
        assert abs(a - b) <= gap_rel * max(abs(a), abs(b), 1e-300), (
            f"query {q} rank {j}: index {got_idx[q, j]} (d={a!r}) vs {cmp_idx[q, j]} (d={b!r})")
    return {"queries": Q, "set_mismatch_within_gap": set_mismatch,
            "pos_mismatch_within_gap": int(pos.sum()),
            "max_dist_rel_err": float((err / np.maximum(got_d64, 1e-300)).max()) if err.size else 0.0}


def recall_at_k(got_idx, exact_idx):
    got_idx = np.asarray(got_idx)
    exact_idx = np.asarray(exact_idx)
    hit = 0
    for q in range(got_idx.shape[0]):
        hit += len(set(got_idx[q].tolist()) & set(exact_idx[q].tolist()))
    return hit / exact_idx.size
