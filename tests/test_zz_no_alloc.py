"""The allocation-free entry point (knns_search_device_noalloc) against the
regular one, through the C ABI, on two calls in a row.

The allocation-free variant serves callers that must not have device memory
allocated during a search (their HBM is owned by another allocator, or a
cudaMalloc would stall a latency-critical path); it keeps its scratch in one
fixed device array instead.  This file sorts last so that a run stopping at
the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAP = 1e-6
DIST_REL = 1e-5


def _noalloc(engine, c, q, k, stream):
    import torch
    Q, D = q.shape
    dist = torch.full((Q, k), -1.0, dtype=torch.float32, device=c.device)
    idx = torch.full((Q, k), -7, dtype=torch.int32, device=c.device)
    rc = engine.lib().knns_search_device_noalloc(c.data_ptr(), c.shape[0], c.stride(0), q.data_ptr(), Q,
                                                 q.stride(0), D, k, dist.data_ptr(), idx.data_ptr(),
                                                 ctypes.c_void_p(stream.cuda_stream))
    assert rc == engine.OK, engine.last_error()
    assert engine.lib().knns_check_device(ctypes.c_void_p(stream.cuda_stream)) == engine.OK
    return dist.cpu().numpy(), idx.cpu().numpy()


def test_noalloc_matches_search_device_two_calls(engine, oracle):
    import torch
    stream = torch.cuda.current_stream()
    # the set-up a caller makes at start-up, before handing the HBM to its own allocator
    assert engine.lib().knns_noalloc_prepare() == engine.OK, engine.last_error()
    rng = np.random.default_rng(2027)
    # calls in a row, different sizes: stale scratch must not leak; k = 500 is served as by
    # the regular entry point (shortlist without the re-rank margin)
    shapes = [(20000, 300, 96, 16), (9000, 150, 43, 100), (6000, 40, 32, 500)]
    for N, Q, D, k in shapes:
        X = rng.random((N, D), dtype=np.float32)
        Qs = rng.random((Q, D), dtype=np.float32)
        c = torch.from_numpy(X).cuda()
        q = torch.from_numpy(Qs).cuda()
        d_ref, i_ref = engine.search(c, q, k, algo=engine.ALGO_SIMT)
        d_ref, i_ref = d_ref.cpu().numpy(), i_ref.cpu().numpy()
        d, i = _noalloc(engine, c, q, k, stream)
        # same kernels and conventions: identical, and within the parity bar of the FP64 oracle
        np.testing.assert_array_equal(i, i_ref)
        np.testing.assert_array_equal(d, d_ref)
        oracle.check_parity(X, Qs, k, d, i, gap_rel=GAP, dist_rel=DIST_REL)


def test_noalloc_rejects_oversize(engine):
    import torch
    c = torch.zeros((3_000_000, 8), device="cuda")
    q = torch.zeros((4, 8), device="cuda")
    dist = torch.empty((4, 8), device="cuda")
    idx = torch.empty((4, 8), dtype=torch.int32, device="cuda")
    rc = engine.lib().knns_search_device_noalloc(c.data_ptr(), c.shape[0], 8, q.data_ptr(), 4, 8, 8, 8,
                                                 dist.data_ptr(), idx.data_ptr(), None)
    assert rc == engine.ERR_UNSUPPORTED
    assert "scratch" in engine.last_error()
