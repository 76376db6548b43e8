"""Preparation pass (one read of the rows): norms, BF16 and E4M3 copies, flags.

Bars, all bit-exact:
 * norms equal the float rounding of the double sum of squares in column order
   (oracle_norms, the convention every kernel and the oracle share) on rows of
   every kind -- integers, uniform, Gaussian, a dynamic range of 10^+-15, sums
   past the float range, squares below it, all-zero rows -- for aligned
   (float4) and unaligned row pitches;
 * the BF16 copy equals round-to-nearest-even BF16, zero padded to 64 columns;
 * the E4M3 codes equal round-to-nearest-even E4M3 of x * (448 / max|x|),
   zero padded to 128 bytes, and the scale is max|x| / 448;
 * the flags (not BF16-exact, not integer, max |x|) match numpy;
 * the norm parts (the BF16 scan's norm operand) are three BF16 values whose sum, in any order,
   is the FP32 norm exactly (norms of 0 and of 2^-100 or more; smaller ones to within 2^-133,
   BF16's subnormal spacing), then zeros.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rows_of_every_kind(n, D, seed):
    rng = np.random.default_rng(seed)
    kind = rng.integers(0, 8, n)
    x = np.empty((n, D), np.float32)
    for r in range(n):
        k = kind[r]
        if k == 0:
            x[r] = rng.integers(0, 256, D)
        elif k == 1:
            x[r] = rng.random(D, dtype=np.float32)
        elif k == 2:
            x[r] = rng.standard_normal(D, dtype=np.float32)
        elif k == 3:
            x[r] = rng.standard_normal(D) * 10.0 ** rng.uniform(-15, 15, D)
        elif k == 4:
            x[r] = rng.standard_normal(D) * 3e18            # squares near the float limit, sums past it
        elif k == 5:
            x[r] = rng.standard_normal(D) * 1e-25           # squares below the float range
        elif k == 6:
            x[r] = 0.0
        else:
            x[r] = rng.integers(-7, 8, D) * np.float32(2.0 ** rng.integers(-30, 30))
    return x


@pytest.mark.parametrize("D", [1, 3, 64, 100, 128, 129, 200, 256, 383, 384])
@pytest.mark.parametrize("pad", [0, 5])
def test_prep_outputs_bit_exact(engine, oracle, D, pad):
    import torch
    n = 3000
    x = rows_of_every_kind(n, D, D * 7 + pad)
    buf = np.zeros((n, D + pad), np.float32)
    buf[:, :D] = x
    xt = torch.from_numpy(buf).cuda()[:, :D]
    norms, bf, f8, scales, words, parts = engine.debug_prep(xt, norm_parts=True)
    with np.errstate(over="ignore"):
        want = oracle.norms(x)
    got = norms.cpu().numpy()
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))

    xb = torch.from_numpy(x).to(torch.bfloat16)
    bfc = bf.cpu()
    assert torch.equal(bfc[:, :D].view(torch.int16), xb.view(torch.int16))
    assert (bfc[:, D:].float() == 0).all()

    mx = np.abs(x).max(axis=1)
    with np.errstate(divide="ignore"):
        inv = np.where(mx > 0, np.float32(448.0) / mx, np.float32(0.0)).astype(np.float32)
    y = (x * inv[:, None]).astype(np.float32)
    codes = torch.from_numpy(y).to(torch.float8_e4m3fn).view(torch.uint8).numpy()
    f8c = f8.cpu().numpy()
    np.testing.assert_array_equal(f8c[:, :D], codes)
    assert (f8c[:, D:] == 0).all()
    np.testing.assert_array_equal(scales.cpu().numpy(), (mx / np.float32(448.0)).astype(np.float32))

    p = parts.float().cpu().numpy().astype(np.float64)
    assert (p[:, 3:] == 0).all()
    fin = np.isfinite(want) & (want < 3.3e38)
    big = fin & ((want == 0) | (want >= 2.0 ** -100))
    tiny = fin & ~big
    np.testing.assert_array_equal(p[big, 0] + p[big, 1] + p[big, 2], want[big].astype(np.float64))
    assert (np.abs(p[tiny, 0] + p[tiny, 1] + p[tiny, 2] - want[tiny].astype(np.float64)) <= 2.0 ** -133).all()
    assert (p[~fin, 0] >= 3.3e38).all() and (p[~fin, 1:] == 0).all()

    w = words.cpu().numpy().view(np.uint32)
    assert w[0] == int((xb.float().numpy() != x).any())
    assert w[1] == int((x != np.rint(x)).any())
    assert w[2] == np.float32(mx.max()).view(np.uint32)
