"""The threshold scan's plan, computed on the host (knns_debug_scan_plan, no GPU): the seeding
levels and the main pass for the headline workload, and the planner's invariants over shapes."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def cuknns():
    sys.path.insert(0, os.path.join(ROOT, "knn-toolbox_gb300"))
    import build as B  # noqa: knn-toolbox_gb300/build.py
    B.build()
    import cuknns as C
    return C


def test_headline_plan(cuknns):
    # 1,000,000 x 128, 10,000 queries, k = 100 on 152 SMs: shortlist 112 (k + margin), samples of
    # every 8192nd, 512th and 32nd row with threshold ranks 5, 8 and 16, main pass in 15 splits
    p = cuknns.scan_plan(1_000_000, 10_000, 128, 100, sms=152)
    assert p["kp"] == 112 and p["tile_rows"] == 224
    assert p["level_stride"] == [8192, 512, 32]
    assert p["level_rows"] == [123, 1954, 31250]
    assert p["level_rank"] == [5, 8, 16]
    assert p["splits"] == 15 and p["split_len"] == 298 * 224


SHAPES = [(20_000, 300, 128, 16), (150_000, 300, 128, 100), (1_000_000, 10_000, 128, 100),
          (4_000_000, 10_000, 96, 10), (8_000_000, 16_384, 256, 32), (65_536, 1_024, 128, 16),
          (300_000, 500, 1024, 200), (2_000_000, 2_000, 64, 512), (17_000, 1, 40, 1)]


@pytest.mark.parametrize("N,Q,D,k", SHAPES)
@pytest.mark.parametrize("tf32", [False, True])
def test_plan_invariants(cuknns, N, Q, D, k, tf32):
    if not tf32 and D > 256:
        pytest.skip("the BF16 scan takes rows of up to 256 columns")
    p = cuknns.scan_plan(N, Q, D, k, sms=152, tf32=tf32)
    kp, L = p["kp"], p["levels"]
    assert kp >= k and kp % 16 == 0
    strides, rows = p["level_stride"], p["level_rows"]
    # nested samples: the finest stride 32 (64 from 6M rows; finer for long shortlists), x16 per
    # coarser level
    assert strides[-1] in ((4, 8, 16, 32, 64) if N >= 6_000_000 else (4, 8, 16, 32))
    for lv in range(L - 1):
        assert strides[lv] == 16 * strides[lv + 1]
    for lv in range(L):
        assert rows[lv] == -(-N // strides[lv])
        assert 1 <= p["level_rank"][lv] <= rows[lv]
    # the coarsest sample keeps every key (at most 256 rows: the selection ranks them in registers),
    # and is the first stride that small
    assert rows[0] <= 256
    if L > 1:
        assert rows[1] > 256
    assert p["level_splits"][0] * 4 * p["level_cap"][0] >= rows[0]
    # main pass: whole tiles per split, every row in exactly one split, at most 128 splits
    tn, S, sl = p["tile_rows"], p["splits"], p["split_len"]
    assert sl % tn == 0 and 1 <= S <= 128
    assert S * sl >= N > (S - 1) * sl
    assert p["cap"] >= 1 and kp <= p["sel_words"] <= 2048


def test_finest_stride_by_corpus_size(cuknns):
    # seeding cost grows with N / stride, the main pass's extra candidates do not: 64 from 6M rows
    assert cuknns.scan_plan(4_000_000, 10_000, 96, 10)["level_stride"][-1] == 32
    assert cuknns.scan_plan(8_000_000, 16_384, 256, 32)["level_stride"][-1] == 64


def test_plan_rejects_bad_arguments(cuknns):
    with pytest.raises(cuknns.KnnsError):
        cuknns.scan_plan(1000, 10, 128, 513)
    with pytest.raises(cuknns.KnnsError):
        cuknns.scan_plan(0, 10, 128, 10)
    # a successful call clears the library's last error (other tests read it)
    cuknns.scan_plan(1000, 10, 128, 10)
    assert cuknns.last_error() == ""
