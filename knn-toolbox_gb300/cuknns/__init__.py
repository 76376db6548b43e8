"""Python mirror of knn-toolbox's interface over the GB300 engine's C ABI.

The engine is the CUDA shared library built from ``knn-toolbox_gb300/csrc``
(``_build/libknngb300.so``); this module only binds its C entry points with
ctypes.  There is no fallback: if the library is missing or fails to load,
every call raises.

Reference interfaces mirrored here (paths within shengren/knn-toolbox):

* ``gpuknnsBitonic`` / ``gpuknnsHeap`` -- include/cuknns.h:75,83: host arrays,
  D-leading corpus and queries, k-leading outputs, 0-based float indices,
  returns elapsed seconds.
* ``knnsplan`` / ``knnsexecute`` -- include/cuknns.h:85,87.
* ``gpuknnBitonic`` / ``gpuknnHeap`` / ``gpuknns`` -- toolbox/*.m: MATLAB
  column matrices (d x n), 1-based indices, columns sorted ascending.
* ``search`` / ``search_host`` -- the engine's status-returning API
  (include/knn_gb300.h) on device tensors or host arrays.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "_build", "libknngb300.so")

ALGO_AUTO, ALGO_TC, ALGO_SIMT = 0, 1, 2
PREC_EXACT, PREC_BF16, PREC_FP8 = 0, 1, 2
SCAN_AUTO, SCAN_ON, SCAN_OFF, SCAN_TF32 = 0, 1, 2, 3
OK, ERR_INVALID, ERR_CUDA, ERR_UNSUPPORTED, ERR_DEVICE_TIMEOUT, ERR_NOMEM = range(6)

# Every symbol include/knn_gb300.h and include/cuknns.h declare.
EXPORTED = ["knns_default_options", "knns_search_device", "knns_search_host", "knns_check_device", "knns_merge_topk",
            "knns_last_error", "knns_last_stats", "knns_last_fixups", "knns_version", "knns_debug_tc_dot_tile",
            "knns_debug_stall_next_search",
            "knns_debug_prep", "knns_debug_scan_plan",
            "knns_timing_collect", "knns_timing_collect5", "knns_search_device_noalloc", "knns_noalloc_prepare",
            "knns_index_create", "knns_index_search", "knns_index_destroy", "knns_autotune_shortlist",
            "knns_server_default_config", "knns_server_create", "knns_server_submit", "knns_server_wait",
            "knns_server_stats", "knns_server_destroy", "knns_server_warmup",
            "gpuknnsBitonic", "gpuknnsHeap", "knnsplan", "knnsexecute"]


class KnnsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"knns error {code}: {msg}")
        self.code = code


class Options(ctypes.Structure):
    _fields_ = [("algo", ctypes.c_int), ("splits", ctypes.c_int), ("rerank", ctypes.c_int),
                ("kp", ctypes.c_int), ("timing", ctypes.c_int), ("pilot", ctypes.c_int),
                ("precision", ctypes.c_int), ("shortlist", ctypes.c_int), ("scan", ctypes.c_int),
                ("scan_boxes", ctypes.c_int), ("block_rows", ctypes.c_int), ("tf32_only", ctypes.c_int),
                ("scan_accs", ctypes.c_int), ("single_stream", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("algo", ctypes.c_int), ("splits", ctypes.c_int), ("kp", ctypes.c_int),
                ("stages", ctypes.c_int), ("launches", ctypes.c_int), ("pilot", ctypes.c_int),
                ("workspace_bytes", ctypes.c_int64), ("scan", ctypes.c_int), ("scan_splits", ctypes.c_int),
                ("scan_cap", ctypes.c_int), ("scan_ring", ctypes.c_int), ("scan_keys", ctypes.c_int)]


class ScanPlanInfo(ctypes.Structure):
    _fields_ = [("kp", ctypes.c_int), ("tile_rows", ctypes.c_int), ("levels", ctypes.c_int),
                ("level_rows", ctypes.c_int64 * 6), ("level_stride", ctypes.c_int64 * 6),
                ("level_rank", ctypes.c_int * 6), ("level_splits", ctypes.c_int * 6), ("level_cap", ctypes.c_int * 6),
                ("splits", ctypes.c_int), ("split_len", ctypes.c_int64), ("cap", ctypes.c_int),
                ("sel_words", ctypes.c_int)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_int), ("max_batch", ctypes.c_int), ("precision", ctypes.c_int),
                ("shortlist", ctypes.c_int), ("autotune", ctypes.c_int), ("reserved", ctypes.c_int * 3)]


KNNPTR2FUNCTION = ctypes.CFUNCTYPE(ctypes.c_double, *([ctypes.POINTER(ctypes.c_float)] * 4),
                                   *([ctypes.c_int] * 5))


class KnnPlan(ctypes.Structure):
    """include/cuknns.h:34-41 knnplan (binary layout kept)."""
    _fields_ = [("pt2Function", ctypes.c_void_p), ("objects", ctypes.c_int), ("numQueries", ctypes.c_int),
                ("dimentions", ctypes.c_int), ("k", ctypes.c_int), ("numStreams", ctypes.c_int)]


_lib = None


def library_path() -> str:
    return LIB_PATH


def lib():
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"GB300 kNN engine library not built: {LIB_PATH} (run __graft_entry__.build())")
    L = ctypes.CDLL(LIB_PATH)
    vp, i64, ci = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    fp = ctypes.POINTER(ctypes.c_float)
    L.knns_default_options.argtypes = [ctypes.POINTER(Options)]
    L.knns_default_options.restype = None
    L.knns_search_device.argtypes = [vp, i64, i64, vp, i64, i64, ci, ci, vp, vp, ctypes.POINTER(Options), vp]
    L.knns_search_host.argtypes = [vp, i64, vp, i64, ci, ci, vp, vp, ctypes.POINTER(Options)]
    L.knns_check_device.argtypes = [vp]
    L.knns_merge_topk.argtypes = [vp, vp, ci, vp, vp, ci, ctypes.c_int32, i64, ci, vp, vp, vp]
    L.knns_last_error.restype = ctypes.c_char_p
    L.knns_last_stats.argtypes = [ctypes.POINTER(Stats)]
    L.knns_last_fixups.argtypes = [ctypes.POINTER(ctypes.c_int64)]
    L.knns_debug_tc_dot_tile.argtypes = [vp, i64, vp, i64, ci, vp]
    L.knns_debug_stall_next_search.argtypes = [i64]
    L.knns_debug_prep.argtypes = [vp, i64, i64, ci, vp, vp, vp, vp, vp, vp]
    L.knns_debug_scan_plan.argtypes = [i64, i64, ci, ci, ci, ci, ctypes.POINTER(ScanPlanInfo)]
    L.knns_timing_collect.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]
    L.knns_timing_collect5.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]
    L.knns_search_device_noalloc.argtypes = [vp, i64, i64, vp, i64, i64, ci, ci, vp, vp, vp]
    L.knns_noalloc_prepare.argtypes = []
    L.knns_index_create.argtypes = [vp, i64, i64, ci, ci, ctypes.POINTER(vp), vp]
    L.knns_index_search.argtypes = [vp, vp, i64, i64, ci, vp, vp, ctypes.POINTER(Options), vp]
    L.knns_autotune_shortlist.argtypes = [vp, vp, i64, i64, ci, ci, ctypes.c_double, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_double), vp]
    L.knns_index_destroy.argtypes = [vp]
    L.knns_index_destroy.restype = None
    L.knns_server_default_config.argtypes = [ctypes.POINTER(ServerConfig)]
    L.knns_server_default_config.restype = None
    L.knns_server_create.argtypes = [vp, ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)]
    L.knns_server_submit.argtypes = [vp, vp, i64, ci]
    L.knns_server_submit.restype = i64
    L.knns_server_wait.argtypes = [vp, i64, vp, vp, ctypes.POINTER(ctypes.c_double)]
    L.knns_server_stats.argtypes = [vp, ctypes.POINTER(i64)]
    L.knns_server_warmup.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ci, ctypes.POINTER(ctypes.c_int), ci]
    L.knns_server_destroy.argtypes = [vp]
    L.knns_server_destroy.restype = None
    L.gpuknnsBitonic.argtypes = [fp, fp, fp, fp, ci, ci, ci, ci, ci]
    L.gpuknnsBitonic.restype = ctypes.c_double
    L.gpuknnsHeap.argtypes = [fp, fp, fp, fp, ci, ci, ci, ci, ci]
    L.gpuknnsHeap.restype = ctypes.c_double
    L.knnsplan.argtypes = [ctypes.POINTER(KnnPlan), ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_long]
    L.knnsplan.restype = None
    L.knnsexecute.argtypes = [KnnPlan, fp, fp, fp, fp]
    L.knnsexecute.restype = None
    _lib = L
    return L


def last_error() -> str:
    return lib().knns_last_error().decode()


def _check(rc):
    if rc != OK:
        raise KnnsError(rc, last_error())


def options(algo=ALGO_AUTO, splits=0, rerank=True, kp=0, timing=False, pilot=True, precision=PREC_EXACT,
            shortlist=0, scan=SCAN_AUTO, scan_boxes=0, block_rows=0, tf32_only=False, scan_accs=0,
            single_stream=False) -> Options:
    o = Options()
    lib().knns_default_options(ctypes.byref(o))
    o.algo, o.splits, o.rerank, o.kp = int(algo), int(splits), int(bool(rerank)), int(kp)
    o.timing = int(bool(timing))
    o.pilot = int(bool(pilot))
    o.precision, o.shortlist = int(precision), int(shortlist)
    o.scan, o.scan_boxes = int(scan), int(scan_boxes)
    o.block_rows = int(block_rows)
    o.tf32_only = int(bool(tf32_only))
    o.scan_accs = int(scan_accs)
    o.single_stream = int(bool(single_stream))
    return o


def timing_collect():
    """Sum of per-stage milliseconds of timed searches since the last call: (prep, fused, select, count)."""
    ms = (ctypes.c_double * 3)()
    n = ctypes.c_int(0)
    _check(lib().knns_timing_collect(ms, ctypes.byref(n)))
    return ms[0], ms[1], ms[2], n.value


def timing_collect5():
    """Per-stage milliseconds: (prep, seeding, fused, select, fixup, count) summed since the last call."""
    ms = (ctypes.c_double * 5)()
    n = ctypes.c_int(0)
    _check(lib().knns_timing_collect5(ms, ctypes.byref(n)))
    return ms[0], ms[1], ms[2], ms[3], ms[4], n.value


def last_fixups() -> int:
    """Queries of the last threshold-scan search that the fix-up pass answered (synchronises)."""
    n = ctypes.c_int64(0)
    _check(lib().knns_last_fixups(ctypes.byref(n)))
    return n.value


def last_stats() -> dict:
    s = Stats()
    _check(lib().knns_last_stats(ctypes.byref(s)))
    return {"algo": s.algo, "splits": s.splits, "kp": s.kp, "stages": s.stages, "launches": s.launches,
            "pilot": s.pilot, "workspace_bytes": s.workspace_bytes, "scan": s.scan, "scan_splits": s.scan_splits,
            "scan_cap": s.scan_cap, "scan_ring": s.scan_ring, "scan_keys": s.scan_keys}


# --------------------------------------------------------------------------
# engine API
# --------------------------------------------------------------------------

def search(corpus, queries, k, *, dist=None, idx=None, algo=ALGO_AUTO, splits=0, rerank=True, kp=0,
           stream=None, check=True, timing=False, pilot=True, precision=PREC_EXACT, shortlist=0, scan=SCAN_AUTO,
           scan_boxes=0, tf32_only=False, scan_accs=0, single_stream=False):
    """kNN on CUDA tensors (float32, rows contiguous).  Returns (dist[Q,k] f32, idx[Q,k] i32)."""
    import torch
    assert corpus.is_cuda and queries.is_cuda, "search() takes device tensors"
    assert corpus.dtype == torch.float32 and queries.dtype == torch.float32
    assert corpus.stride(1) == 1 and queries.stride(1) == 1
    N, D = corpus.shape
    Q = queries.shape[0]
    assert queries.shape[1] == D
    if dist is None:
        dist = torch.empty((Q, k), dtype=torch.float32, device=corpus.device)
    if idx is None:
        idx = torch.empty((Q, k), dtype=torch.int32, device=corpus.device)
    s = torch.cuda.current_stream(corpus.device) if stream is None else stream
    o = options(algo, splits, rerank, kp, timing, pilot, precision, shortlist, scan, scan_boxes,
                tf32_only=tf32_only, scan_accs=scan_accs, single_stream=single_stream)
    rc = lib().knns_search_device(corpus.data_ptr(), N, corpus.stride(0), queries.data_ptr(), Q,
                                  queries.stride(0), D, k, dist.data_ptr(), idx.data_ptr(), ctypes.byref(o),
                                  ctypes.c_void_p(s.cuda_stream))
    _check(rc)
    if check:
        _check(lib().knns_check_device(ctypes.c_void_p(s.cuda_stream)))
    return dist, idx


def merge_topk(run_d, run_i, have, blk_d, blk_i, kb, k, offset=0, stream=None):
    """Merge two per-query result lists on the device by (distance, index) (knns_merge_topk).

    run_d / run_i: Q x k (first `have` columns used); blk_d / blk_i: Q x kb, indices shifted by
    `offset`.  Returns new (dist Q x k, idx Q x k) CUDA tensors holding min(k, have + kb) entries.
    """
    import torch
    Q = run_d.shape[0] if have > 0 else blk_d.shape[0]
    dev = (run_d if have > 0 else blk_d).device
    out_d = torch.full((Q, k), float("inf"), dtype=torch.float32, device=dev)
    out_i = torch.full((Q, k), -1, dtype=torch.int32, device=dev)
    for t, cols in ((run_d, k), (run_i, k), (blk_d, kb), (blk_i, kb)):
        assert t is None or (t.is_cuda and t.is_contiguous() and t.shape == (Q, cols)), "merge_topk operands"
    s = torch.cuda.current_stream(dev) if stream is None else stream
    ptr = (lambda t: t.data_ptr() if t is not None else None)
    _check(lib().knns_merge_topk(ptr(run_d) if have else None, ptr(run_i) if have else None, have,
                                 ptr(blk_d) if kb else None, ptr(blk_i) if kb else None, kb, int(offset), Q, k,
                                 out_d.data_ptr(), out_i.data_ptr(), ctypes.c_void_p(s.cuda_stream)))
    return out_d, out_i


def search_host(corpus, queries, k, *, algo=ALGO_AUTO, splits=0, rerank=True, kp=0, **opts):
    """kNN on host arrays (N x D, Q x D float32).  Returns numpy (dist, idx).

    Further keyword options (precision, shortlist, scan, ...) as for search().
    """
    corpus = np.ascontiguousarray(corpus, dtype=np.float32)
    queries = np.ascontiguousarray(queries, dtype=np.float32)
    N, D = corpus.shape
    Q = queries.shape[0]
    dist = np.empty((Q, k), np.float32)
    idx = np.empty((Q, k), np.int32)
    o = options(algo, splits, rerank, kp, **opts)
    _check(lib().knns_search_host(corpus.ctypes.data, N, queries.ctypes.data, Q, D, k, dist.ctypes.data,
                                  idx.ctypes.data, ctypes.byref(o)))
    return dist, idx


def scan_plan(N, Q, D, k, sms=152, tf32=False) -> dict:
    """The threshold scan's plan for an exact-form search, computed on the host (no GPU): seeding
    levels coarsest first (rows, stride, rank, splits, cap) and the main pass."""
    p = ScanPlanInfo()
    _check(lib().knns_debug_scan_plan(N, Q, D, k, sms, int(bool(tf32)), ctypes.byref(p)))
    L = p.levels
    return {"kp": p.kp, "tile_rows": p.tile_rows, "levels": L,
            "level_rows": list(p.level_rows[:L]), "level_stride": list(p.level_stride[:L]),
            "level_rank": list(p.level_rank[:L]), "level_splits": list(p.level_splits[:L]),
            "level_cap": list(p.level_cap[:L]), "splits": p.splits, "split_len": p.split_len, "cap": p.cap,
            "sel_words": p.sel_words}


def debug_prep(x, norm_parts=False):
    """Preparation pass over a device matrix: (norms, bf16 copy, E4M3 codes, scales, words), all torch tensors;
    with norm_parts, also the [n][16] BF16 norm parts."""
    import torch
    n, D = x.shape
    dev = x.device
    norms = torch.empty(n, dtype=torch.float32, device=dev)
    bf = torch.empty((n, (D + 63) // 64 * 64), dtype=torch.bfloat16, device=dev)
    f8 = torch.empty((n, (D + 127) // 128 * 128), dtype=torch.uint8, device=dev)
    scales = torch.empty(n, dtype=torch.float32, device=dev)
    words = torch.zeros(3, dtype=torch.int32, device=dev)
    np_ = torch.empty((n, 16), dtype=torch.bfloat16, device=dev) if norm_parts else None
    _check(lib().knns_debug_prep(x.data_ptr(), n, x.stride(0), D, norms.data_ptr(), bf.data_ptr(), f8.data_ptr(),
                                 scales.data_ptr(), words.data_ptr(), np_.data_ptr() if norm_parts else None))
    if norm_parts:
        return norms, bf, f8, scales, words, np_
    return norms, bf, f8, scales, words


def debug_tc_dot_tile(corpus, queries):
    import torch
    dump = torch.empty((128, 128), dtype=torch.float32, device=corpus.device)
    _check(lib().knns_debug_tc_dot_tile(corpus.data_ptr(), corpus.shape[0], queries.data_ptr(), queries.shape[0],
                                        corpus.shape[1], dump.data_ptr()))
    return dump


# --------------------------------------------------------------------------
# reference C API (include/cuknns.h)
# --------------------------------------------------------------------------

def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _c_call(fn, query, data, k, numStreams):
    """query: Q x D (D leading), data: N x D.  Returns (values[Q,k], indices[Q,k] float, seconds)."""
    query = np.ascontiguousarray(query, dtype=np.float32)
    data = np.ascontiguousarray(data, dtype=np.float32)
    Q, D = query.shape
    N = data.shape[0]
    values = np.empty((Q, k), np.float32)
    indices = np.empty((Q, k), np.float32)
    t = fn(_fptr(query), _fptr(data), _fptr(values), _fptr(indices), N, Q, D, k, numStreams)
    if t >= 3.0e38:
        raise KnnsError(-1, last_error())
    return values, indices, t


def gpuknnsBitonic(query, data, k, numStreams=1):
    return _c_call(lib().gpuknnsBitonic, query, data, k, numStreams)


def gpuknnsHeap(query, data, k, numStreams=1):
    return _c_call(lib().gpuknnsHeap, query, data, k, numStreams)


def knnsplan(N, Q, D, k) -> KnnPlan:
    plan = KnnPlan()
    lib().knnsplan(ctypes.byref(plan), N, Q, D, k)
    if not plan.pt2Function:
        raise KnnsError(-1, last_error())
    return plan


def knnsexecute(plan: KnnPlan, data, queries):
    data = np.ascontiguousarray(data, dtype=np.float32)
    queries = np.ascontiguousarray(queries, dtype=np.float32)
    KNNdist = np.empty((plan.numQueries, plan.k), np.float32)
    KNNidx = np.empty((plan.numQueries, plan.k), np.float32)
    lib().knnsexecute(plan, _fptr(data), _fptr(queries), _fptr(KNNdist), _fptr(KNNidx))
    return KNNdist, KNNidx


# --------------------------------------------------------------------------
# double-precision library (libknngb300_double.so: the reference's libcuknn_double)
# --------------------------------------------------------------------------

LIB_F64_PATH = os.path.join(PKG, "_build", "libknngb300_double.so")
EXPORTED_F64 = ["gpuknnsBitonic", "gpuknnsHeap", "knnsplan", "knnsexecute", "knns_search_device_f64",
                "knns_search_host_f64", "knns_f64_last_error"]
_lib64 = None


def lib_f64():
    global _lib64
    if _lib64 is not None:
        return _lib64
    if not os.path.exists(LIB_F64_PATH):
        raise RuntimeError(f"double-precision library not built: {LIB_F64_PATH}")
    L = ctypes.CDLL(LIB_F64_PATH)
    vp, i64, ci = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    dp = ctypes.POINTER(ctypes.c_double)
    L.knns_search_device_f64.argtypes = [vp, i64, i64, vp, i64, i64, ci, ci, vp, vp, vp]
    L.knns_search_host_f64.argtypes = [vp, i64, vp, i64, ci, ci, vp, vp]
    L.knns_f64_last_error.restype = ctypes.c_char_p
    L.gpuknnsBitonic.argtypes = [dp, dp, dp, dp, ci, ci, ci, ci, ci]
    L.gpuknnsBitonic.restype = ctypes.c_double
    L.gpuknnsHeap.argtypes = [dp, dp, dp, dp, ci, ci, ci, ci, ci]
    L.gpuknnsHeap.restype = ctypes.c_double
    _lib64 = L
    return L


def search_host_f64(corpus, queries, k):
    """Exact FP64 kNN on host arrays (N x D, Q x D float64).  Returns numpy (dist f64, idx i32)."""
    corpus = np.ascontiguousarray(corpus, dtype=np.float64)
    queries = np.ascontiguousarray(queries, dtype=np.float64)
    N, D = corpus.shape
    Q = queries.shape[0]
    dist = np.empty((Q, k), np.float64)
    idx = np.empty((Q, k), np.int32)
    rc = lib_f64().knns_search_host_f64(corpus.ctypes.data, N, queries.ctypes.data, Q, D, k, dist.ctypes.data,
                                        idx.ctypes.data)
    if rc != OK:
        raise KnnsError(rc, lib_f64().knns_f64_last_error().decode())
    return dist, idx


def gpuknnsBitonic_f64(query, data, k, numStreams=1):
    """The double library's gpuknnsBitonic: query Q x D, data N x D (float64).  Returns (values, indices, s)."""
    query = np.ascontiguousarray(query, dtype=np.float64)
    data = np.ascontiguousarray(data, dtype=np.float64)
    Q, D = query.shape
    N = data.shape[0]
    vals = np.empty((Q, k), np.float64)
    idxs = np.empty((Q, k), np.float64)
    dp = ctypes.POINTER(ctypes.c_double)
    t = lib_f64().gpuknnsBitonic(query.ctypes.data_as(dp), data.ctypes.data_as(dp), vals.ctypes.data_as(dp),
                                 idxs.ctypes.data_as(dp), N, Q, D, k, numStreams)
    if t >= 1e300:
        raise KnnsError(-1, lib_f64().knns_f64_last_error().decode())
    return vals, idxs, t


# --------------------------------------------------------------------------
# MATLAB toolbox semantics (toolbox/gpuknnBitonic.m, gpuknnHeap.m, gpuknns.m)
# --------------------------------------------------------------------------

def _toolbox(fn, query, pdata, k, numStreams):
    """query: d x Q, pdata: d x N (columns are vectors).  Returns (dist k x Q, idx k x Q 1-based, time)."""
    q = np.asarray(query, dtype=np.float32).T
    c = np.asarray(pdata, dtype=np.float32).T
    values, indices, t = fn(q, c, k, numStreams)
    idx = indices + 1                                   # gpuknnBitonic.m:24
    order = np.argsort(values, axis=1, kind="stable")   # gpuknnBitonic.m:26-30
    values = np.take_along_axis(values, order, axis=1)
    idx = np.take_along_axis(idx, order, axis=1)
    return values[:, :k].T.copy(), idx[:, :k].T.copy(), t  # gpuknnBitonic.m:32-33


def gpuknnBitonic(query, pdata, k, numStreams=1):
    return _toolbox(gpuknnsBitonic, query, pdata, k, numStreams)


def gpuknnHeap(query, pdata, k, numStreams=1):
    return _toolbox(gpuknnsHeap, query, pdata, k, numStreams)


def gpuknns(plan: dict, queries, data):
    """toolbox/gpuknns.m: plan is {'function': gpuknnBitonic|gpuknnHeap, 'k': k, 'streams': s}."""
    return plan["function"](queries, data, plan["k"], plan["streams"])


# --------------------------------------------------------------------------
# resident index and the serving form
# --------------------------------------------------------------------------

INDEX_TF32 = 1
INDEX_FP8 = 2


class Index:
    """A device corpus prepared once (BF16 copy, norms, flags, TF32 copies, E4M3 codes): searches skip its preparation.

    The torch tensor is kept referenced: the engine reads it on every search.
    """

    def __init__(self, corpus, tf32=True, fp8=False, stream=None):
        import torch
        assert corpus.is_cuda and corpus.dtype == torch.float32 and corpus.stride(1) == 1
        self.corpus = corpus
        self.N, self.D = corpus.shape
        s = torch.cuda.current_stream(corpus.device) if stream is None else stream
        h = ctypes.c_void_p()
        _check(lib().knns_index_create(corpus.data_ptr(), self.N, corpus.stride(0), self.D,
                                       (INDEX_TF32 if tf32 else 0) | (INDEX_FP8 if fp8 else 0), ctypes.byref(h),
                                       ctypes.c_void_p(s.cuda_stream)))
        self.handle = h

    def search(self, queries, k, *, dist=None, idx=None, stream=None, check=True, **opts):
        import torch
        assert queries.is_cuda and queries.dtype == torch.float32 and queries.stride(1) == 1
        Q = queries.shape[0]
        if dist is None:
            dist = torch.empty((Q, k), dtype=torch.float32, device=queries.device)
        if idx is None:
            idx = torch.empty((Q, k), dtype=torch.int32, device=queries.device)
        s = torch.cuda.current_stream(queries.device) if stream is None else stream
        o = options(**opts)
        _check(lib().knns_index_search(self.handle, queries.data_ptr(), Q, queries.stride(0), k, dist.data_ptr(),
                                       idx.data_ptr(), ctypes.byref(o), ctypes.c_void_p(s.cuda_stream)))
        if check:
            _check(lib().knns_check_device(ctypes.c_void_p(s.cuda_stream)))
        return dist, idx

    def autotune_shortlist(self, queries, k, target=0.999, precision=PREC_BF16, stream=None):
        """Smallest shortlist factor c in {2, 4, 8} of the BF16 / FP8 form reaching recall@k >= target."""
        import torch
        s = torch.cuda.current_stream(queries.device) if stream is None else stream
        c = ctypes.c_int(0)
        r = ctypes.c_double(0.0)
        _check(lib().knns_autotune_shortlist(self.handle, queries.data_ptr(), queries.shape[0], queries.stride(0), k,
                                             precision, target, ctypes.byref(c), ctypes.byref(r),
                                             ctypes.c_void_p(s.cuda_stream)))
        return c.value, r.value

    def close(self):
        if getattr(self, "handle", None):
            lib().knns_index_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request server over an Index (see include/knn_gb300.h).

    submit() takes host queries (numpy, Q x D float32) and returns a request id;
    wait() blocks until that request is answered and returns (dist, idx, latency_ms).
    """

    def __init__(self, index, slots=2, max_batch=1024, precision=PREC_EXACT, shortlist=0, autotune=True):
        cfg = ServerConfig()
        lib().knns_server_default_config(ctypes.byref(cfg))
        cfg.slots, cfg.max_batch, cfg.precision, cfg.shortlist = slots, max_batch, precision, shortlist
        cfg.autotune = int(bool(autotune))
        h = ctypes.c_void_p()
        _check(lib().knns_server_create(index.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self.index = index
        self.handle = h
        self.D = index.D
        self._k = {}

    def submit(self, queries, k):
        q = np.ascontiguousarray(queries, dtype=np.float32)
        assert q.ndim == 2 and q.shape[1] == self.D
        rid = lib().knns_server_submit(self.handle, q.ctypes.data, q.shape[0], k)
        if rid <= 0:
            raise KnnsError(-rid, last_error())
        self._k[rid] = (q.shape[0], k)
        return rid

    def wait(self, rid):
        Q, k = self._k.pop(rid)
        dist = np.empty((Q, k), np.float32)
        idx = np.empty((Q, k), np.int32)
        lat = ctypes.c_double(0.0)
        _check(lib().knns_server_wait(self.handle, rid, dist.ctypes.data, idx.ctypes.data, ctypes.byref(lat)))
        return dist, idx, lat.value

    def warmup(self, buckets, ks):
        b = (ctypes.c_int * len(buckets))(*buckets)
        kk = (ctypes.c_int * len(ks))(*ks)
        _check(lib().knns_server_warmup(self.handle, b, len(buckets), kk, len(ks)))

    def stats(self):
        out = (ctypes.c_int64 * 4)()
        _check(lib().knns_server_stats(self.handle, out))
        return {"requests": out[0], "launches": out[1], "queries": out[2], "graphs": out[3]}

    def close(self):
        if getattr(self, "handle", None):
            lib().knns_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
