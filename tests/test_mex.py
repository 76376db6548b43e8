"""MEX gateways mexknns{,D}{Bitonic,Heap} (src/mexknnsGen.cu, src/mexknnsHeap.cu
interface) built against the fake mex.h shim in tests/mex_shim (MATLAB is not
installed).  Argument checking runs on the CPU; the searches need a GPU and are
held to the parity bars of test_gpu_parity.py (float) and to the FP64 oracle of
FP64 inputs (double: indices and distances identical).
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "tests", "mex_shim")
GATEWAY = os.path.join(ROOT, "knn-toolbox_gb300", "mex", "mexknns.cpp")
BUILD = os.path.join(ROOT, "knn-toolbox_gb300", "_build")
MX_DOUBLE, MX_SINGLE = 6, 7
NAMES = {"mexknnsBitonic": [], "mexknnsHeap": ["-DKNN_GATEWAY_HEAP"],
         "mexknnsDBitonic": ["-DKNN_GATEWAY_DOUBLE"], "mexknnsDHeap": ["-DKNN_GATEWAY_DOUBLE", "-DKNN_GATEWAY_HEAP"]}


@pytest.fixture(scope="session")
def mex(tmp_path_factory):
    """Builds the shim and the four gateways (g++, linked to the engine libraries)."""
    import build as engine_build  # knn-toolbox_gb300/build.py
    engine_build.build()
    d = str(tmp_path_factory.mktemp("mex"))
    shim = os.path.join(d, "libmexshim.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", os.path.join(SHIM, "mex_shim.cpp"), "-I", SHIM,
                    "-o", shim], check=True)
    S = ctypes.CDLL(shim, mode=ctypes.RTLD_GLOBAL)
    vp = ctypes.c_void_p
    S.shim_matrix.argtypes = [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, vp]
    S.shim_matrix.restype = vp
    S.shim_destroy.argtypes = [vp]
    S.shim_call.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, vp, ctypes.c_char_p, ctypes.c_size_t]
    S.mxGetM.argtypes = S.mxGetN.argtypes = S.mxGetData.argtypes = [vp]
    S.mxGetM.restype = S.mxGetN.restype = ctypes.c_size_t
    S.mxGetData.restype = vp
    gws = {}
    for name, flags in NAMES.items():
        lib = "knngb300_double" if "-DKNN_GATEWAY_DOUBLE" in flags else "knngb300"
        out = os.path.join(d, name + ".so")
        subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", GATEWAY, "-I", SHIM, "-I",
                        os.path.join(ROOT, "include")] + flags + ["-o", out, "-L", d, "-lmexshim", "-L", BUILD,
                                                                  "-l" + lib, "-Wl,-rpath," + BUILD,
                                                                  "-Wl,-rpath," + d], check=True)
        gws[name] = ctypes.CDLL(out)
    return S, gws


def call(mex, name, args, nlhs=5):
    """MATLAB-style call: args are numpy arrays (a Q x d array is MATLAB's d x Q matrix) or scalars."""
    S, gws = mex
    keep = []
    ptrs = []
    for a in args:
        a = np.ascontiguousarray(np.atleast_2d(np.asarray(a)))
        cls = MX_SINGLE if a.dtype == np.float32 else MX_DOUBLE
        if a.dtype not in (np.float32, np.float64):
            a = a.astype(np.float64)
        keep.append(a)
        # row-major (n, m) numpy = column-major m x n
        ptrs.append(S.shim_matrix(a.shape[1], a.shape[0], cls, a.ctypes.data))
    prhs = (ctypes.c_void_p * len(ptrs))(*ptrs)
    plhs = (ctypes.c_void_p * 5)()
    err = ctypes.create_string_buffer(1024)
    fn = ctypes.cast(gws[name].mexFunction, ctypes.c_void_p)
    rc = S.shim_call(fn, nlhs, plhs, len(ptrs), prhs, err, 1024)
    for p in ptrs:
        S.shim_destroy(p)
    if rc:
        return None, err.value.decode()
    outs = []
    for i in range(5):
        if not plhs[i]:
            continue
        m, n = S.mxGetM(plhs[i]), S.mxGetN(plhs[i])
        dt = np.float64 if (i >= 2 or name.startswith("mexknnsD")) else np.float32
        buf = (ctypes.c_char * (m * n * np.dtype(dt).itemsize)).from_address(S.mxGetData(plhs[i])) if m * n else b""
        outs.append(np.frombuffer(bytes(buf), dt).reshape(n, m).copy())
        S.shim_destroy(plhs[i])
    return outs, None


def test_gateways_check_arguments(mex):
    rng = np.random.default_rng(0)
    X = rng.random((100, 8), dtype=np.float32)
    Qs = rng.random((5, 8), dtype=np.float32)
    _, e = call(mex, "mexknnsBitonic", [Qs.astype(np.float64), X.astype(np.float64), 4, 1])
    assert e.startswith("knns:class")
    _, e = call(mex, "mexknnsDHeap", [Qs, X, 4, 1])
    assert e.startswith("knns:class")
    _, e = call(mex, "mexknnsBitonic", [Qs, X, 101, 1])
    assert e.startswith("knns:k")
    _, e = call(mex, "mexknnsBitonic", [Qs, X, 2.5, 1])
    assert e.startswith("knns:k")
    _, e = call(mex, "mexknnsHeap", [Qs, X[:, :7], 4, 1])
    assert e.startswith("knns:dims")
    _, e = call(mex, "mexknnsBitonic", [Qs, X, 4])
    assert e.startswith("knns:nrhs")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["mexknnsBitonic", "mexknnsHeap"])
def test_single_gateways(mex, oracle, name):
    rng = np.random.default_rng(1)
    X = rng.random((5000, 43), dtype=np.float32)
    Qs = rng.random((77, 43), dtype=np.float32)
    k = 16
    outs, e = call(mex, name, [Qs, X, k, 2])
    assert e is None, e
    dist, idx, t, td, ts = outs
    assert dist.shape == (77, k) and idx.shape == (77, k)   # MATLAB k x Q
    i = idx.astype(np.int64)
    assert np.array_equal(idx, i.astype(np.float32)) and i.min() >= 0   # 0-based like the reference's gateways
    oracle.check_parity(X, Qs, k, dist, i, gap_rel=1e-6, dist_rel=1e-5)
    assert t[0, 0] > 0 and td[0, 0] > 0 and ts[0, 0] >= 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["mexknnsDBitonic", "mexknnsDHeap"])
def test_double_gateways(mex, oracle, name):
    rng = np.random.default_rng(2)
    X = rng.random((4000, 24))
    Qs = rng.random((50, 24))
    k = 10
    outs, e = call(mex, name, [Qs, X, k, 1])
    assert e is None, e
    dist, idx, t, _, _ = outs
    od, oi = oracle.knn_f64d(X, Qs, k)
    np.testing.assert_array_equal(idx.astype(np.int64), oi)
    np.testing.assert_array_equal(dist, od)
    assert t[0, 0] > 0
