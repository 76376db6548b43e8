"""Bounded waits of the tensor-core kernels, exercised without a GPU fault.

Every mbarrier wait in the engine's kernels gives up after a bound, records an
error code and winds the kernel down.  knns_debug_stall_next_search makes the
next search's shortlist kernels wait on copies that are never issued, under a
50 ms bound: the waits run out, knns_check_device must report
KNNS_ERR_DEVICE_TIMEOUT, and the following search must work and be exact.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_the_engine_recovers(engine, oracle):
    import torch
    rng = np.random.default_rng(404)
    X = rng.random((4096, 64), dtype=np.float32)
    Qs = rng.random((200, 64), dtype=np.float32)
    c, q = torch.from_numpy(X).cuda(), torch.from_numpy(Qs).cuda()
    k = 16
    stream = torch.cuda.current_stream()
    assert engine.lib().knns_debug_stall_next_search(50_000) == engine.OK
    engine.search(c, q, k, algo=engine.ALGO_TC, check=False)
    rc = engine.lib().knns_check_device(ctypes.c_void_p(stream.cuda_stream))
    assert rc == engine.ERR_DEVICE_TIMEOUT, (rc, engine.last_error())
    assert "bounded wait" in engine.last_error()
    # the error word is cleared and the context is intact: the next search is exact
    d, i = engine.search(c, q, k, algo=engine.ALGO_TC)
    assert engine.last_stats()["algo"] == engine.ALGO_TC
    od, oi = oracle.knn_gemm(X, Qs, k, kp=engine.last_stats()["kp"], rerank=True)
    oracle.check_parity(X, Qs, k, d.cpu().numpy(), i.cpu().numpy(), ref_idx=oi, gap_rel=1e-6, dist_rel=1e-5)


def test_stall_hook_rejects_bad_bounds(engine):
    assert engine.lib().knns_debug_stall_next_search(0) == engine.ERR_INVALID
    assert engine.lib().knns_debug_stall_next_search(20_000_000) == engine.ERR_INVALID
