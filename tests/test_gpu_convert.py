"""The mixed path's own FP64 <-> FP32 conversions on the integer pipes
(d2f_int, f2d_int in disco_gb300/csrc/cuda/dev_common.cuh) against the
hardware's conversions, over a bit-pattern sweep: every exponent, exact
ties, the neighbourhoods of FLT_MIN and FLT_MAX, zeros, infinities, NaN and
subnormals.

The documented behaviour is the bar: d2f_int equals round-to-nearest-even
except on exact ties, which it rounds away from zero (the same half-ulp
error); results below FLT_MIN flush to signed zero; overflow gives infinity
and NaN stays NaN.  f2d_int is exact for normal numbers, zeros, infinities
and NaN and flushes FP32 subnormals to signed zero."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLT_MIN = np.float64(np.finfo(np.float32).tiny)


def _doubles(rng):
    parts = []
    # uniform bit patterns over the whole FP64 range, and over the exponents
    # that map into FP32's range
    parts.append(rng.integers(0, 2 ** 64, 400_000, dtype=np.uint64))
    e = rng.integers(850, 1200, 400_000, dtype=np.uint64)
    m = rng.integers(0, 2 ** 52, 400_000, dtype=np.uint64)
    s = rng.integers(0, 2, 400_000, dtype=np.uint64)
    parts.append((s << np.uint64(63)) | (e << np.uint64(52)) | m)
    # exact ties: an FP32 mantissa followed by 1 and 28 zero bits
    e = rng.integers(897, 1151, 100_000, dtype=np.uint64)
    m = (rng.integers(0, 2 ** 23, 100_000, dtype=np.uint64) << np.uint64(29)) | np.uint64(1 << 28)
    s = rng.integers(0, 2, 100_000, dtype=np.uint64)
    parts.append((s << np.uint64(63)) | (e << np.uint64(52)) | m)
    # one ulp either side of ties
    parts.append(parts[-1] + np.uint64(1))
    parts.append(parts[-2] - np.uint64(1))
    # around FLT_MIN and FLT_MAX, every bit pattern in a window
    for c in (FLT_MIN, np.float64(np.finfo(np.float32).max)):
        b = np.array([c], dtype=np.float64).view(np.uint64)[0]
        w = np.arange(-(1 << 30), (1 << 30) + 1, 1 << 14, dtype=np.int64)
        parts.append((np.int64(b) + w).astype(np.uint64))
        parts.append(((np.int64(b) + w).astype(np.uint64)) | np.uint64(1 << 63))
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 1.0, -1.0,
                         np.finfo(np.float64).max], dtype=np.float64)
    parts.append(specials.view(np.uint64))
    return np.concatenate(parts).view(np.float64)


def _floats(rng, n):
    b = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 1.1754942e-38,
                   np.finfo(np.float32).tiny, np.finfo(np.float32).max], dtype=np.float32)
    b[:sp.size] = sp.view(np.uint32)
    return b.view(np.float32)


def test_conversions_match_hardware():
    import disco_gb300 as dg
    rng = np.random.default_rng(20261204)
    x = _doubles(rng)
    y = _floats(rng, x.size)
    out = dg.api.convert_check(x, y)
    fi, fh = out["f_int"], out["f_hw"]
    # FP64 -> FP32
    nan = np.isnan(x)
    assert np.all(np.isnan(fi[nan]))
    xb = x.view(np.uint64)
    a = xb & np.uint64(0x7FFFFFFFFFFFFFFF)
    e = (a >> np.uint64(52)).astype(np.int64)
    low = a & np.uint64((1 << 29) - 1)
    tie = (e >= 897) & (e <= 1150) & (low == np.uint64(1 << 28))
    small = ~nan & (np.abs(x) < FLT_MIN)
    # below FLT_MIN: signed zero
    assert np.all(fi[small] == 0)
    assert np.array_equal(np.signbit(fi[small]), np.signbit(x[small]))
    # everywhere else off ties: bit-equal to round-to-nearest-even
    rest = ~nan & ~small & ~tie
    assert np.array_equal(fi[rest].view(np.uint32), fh[rest].view(np.uint32))
    # exact ties: away from zero, the same distance as the hardware's choice
    t = tie & ~nan
    assert t.sum() > 50_000
    d_int = np.abs(fi[t].astype(np.float64) - x[t])
    d_hw = np.abs(fh[t].astype(np.float64) - x[t])
    assert np.array_equal(d_int, d_hw)
    assert np.all(np.abs(fi[t].astype(np.float64)) >= np.abs(x[t]))
    # FP32 -> FP64
    di, dh = out["d_int"], out["d_hw"]
    ynan = np.isnan(y)
    assert np.all(np.isnan(di[ynan]))
    sub = ~ynan & (y != 0) & (np.abs(y) < np.finfo(np.float32).tiny)
    assert sub.sum() > 0
    assert np.all(di[sub] == 0) and np.array_equal(np.signbit(di[sub]), np.signbit(y[sub]))
    ok = ~ynan & ~sub
    assert np.array_equal(di[ok].view(np.uint64), dh[ok].view(np.uint64))
