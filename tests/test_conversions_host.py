"""The integer-pipe FP64 bit operations of the mixed form (f2d, d2f, lt_zero,
le_threshold, finite64 in braids-hkt_gb300/csrc/brx_mixed.cu), restated on
the same 32-bit word operations in numpy and checked bit for bit against IEEE
arithmetic over random bit patterns, both rounding ties at every exponent,
rounding carries, the ends of the float range and special values:

* f2d equals the exact float -> double conversion (subnormals included);
* d2f equals round-to-nearest-even float -> the unit's flush-to-zero rule:
  results below the float normal range become a signed zero, results above
  it infinite, NaN stays NaN;
* lt_zero equals x < 0, le_threshold equals x <= t for positive t, finite64
  equals isfinite.
"""
import numpy as np

U32, U64 = np.uint32, np.uint64


def split(x):
    b = x.view(U64)
    return (b >> U64(32)).astype(U32), (b & U64(0xFFFFFFFF)).astype(U32)


def d2f_bits(x):
    hi, lo = split(x)
    sign = hi & U32(0x80000000)
    e = (hi >> U32(20)) & U32(0x7FF)
    top = ((hi & U32(0xFFFFF)) << U32(3)) | (lo >> U32(29))
    rem = lo & U32(0x1FFFFFFF)
    r = sign | (((e - U32(896)) & U32(0xFF)) << U32(23)) | top
    up = (rem > U32(0x10000000)) | ((rem == U32(0x10000000)) & ((top & U32(1)) == 1))
    r = r + up.astype(U32)
    r = np.where((e < 896) | ((r & U32(0x7F800000)) == 0), sign, r)
    r = np.where(e > 1150, sign | U32(0x7F800000), r)
    r = np.where((e == 0x7FF) & (((hi & U32(0xFFFFF)) | lo) != 0), sign | U32(0x7FC00000), r)
    return r


def f2d_bits(f):
    b = f.view(U32)
    sign = b & U32(0x80000000)
    e = (b >> U32(23)) & U32(0xFF)
    m = b & U32(0x7FFFFF)
    hi = sign | ((e + U32(896)) << U32(20)) | (m >> U32(3))
    lo = m << U32(29)
    hi = np.where(e == 0xFF, sign | U32(0x7FF00000) | (m >> U32(3)), hi)
    sub = (e == 0) & (m != 0)
    p = np.where(sub, np.floor(np.log2(np.maximum(m, 1))).astype(np.int64), 0)
    frac = (m.astype(U64) ^ (U64(1) << p.astype(U64))) << (U64(52) - p.astype(U64))
    hi = np.where(sub, sign | ((p + 874).astype(U32) << U32(20)) | (frac >> U64(32)).astype(U32), hi)
    lo = np.where(sub, (frac & U64(0xFFFFFFFF)).astype(U32), lo)
    zero = (e == 0) & (m == 0)
    hi = np.where(zero, sign, hi)
    lo = np.where(zero, U32(0), lo)
    return (hi.astype(U64) << U64(32)) | lo.astype(U64)


def _doubles(rng, n):
    bits = rng.integers(0, 2 ** 63, n, dtype=np.int64).astype(U64) | (rng.integers(0, 2, n).astype(U64) << U64(63))
    x = bits.view(np.float64)
    mant = rng.integers(0, 2 ** 23, n).astype(U64)
    exps = rng.integers(880, 1160, n).astype(U64)
    tie = (exps << U64(52)) | (mant << U64(29)) | U64(1 << 28)
    carry = (exps << U64(52)) | (U64(0x7FFFFF) << U64(29)) | U64(1 << 28) | U64(1)
    near = rng.standard_normal(n) * np.exp(rng.uniform(-90, 90, n))
    special = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 3.4028234663852886e38, 3.4028235677973366e38,
                        1.1754943508222875e-38, 1.1754942106924411e-38, 1e-45, 2.0 ** -149, 2.0 ** -150, 1e300, 5e-324])
    return np.concatenate([x, tie.view(np.float64), carry.view(np.float64), near, special])


def test_double_to_float_rounds_to_nearest_with_flush():
    rng = np.random.default_rng(1)
    x = _doubles(rng, 200_000)
    r = d2f_bits(x)
    with np.errstate(over="ignore", under="ignore", invalid="ignore"):
        want = x.astype(np.float32)
    wb = want.view(U32)
    flushed = (wb & U32(0x7F800000)) == 0                  # IEEE result is zero or subnormal
    wb = np.where(flushed, wb & U32(0x80000000), wb)
    nan = np.isnan(x)
    np.testing.assert_array_equal(r[~nan], wb[~nan])
    assert np.isnan(r[nan].view(np.float32)).all()
    assert (~flushed & ~nan & np.isfinite(want)).sum() > 300_000


def test_float_to_double_is_exact():
    rng = np.random.default_rng(2)
    f = rng.integers(0, 2 ** 32, 500_000, dtype=np.uint64).astype(U32).view(np.float32)
    f = np.concatenate([f, np.array([0.0, -0.0, 1.0, -2.5, np.inf, -np.inf, np.nan, 1e-45, 3.4e38], np.float32),
                        (np.arange(1, 1 << 12, dtype=U32) * U32(2047)).view(np.float32)])   # subnormals
    r = f2d_bits(f)
    with np.errstate(invalid="ignore"):
        want = f.astype(np.float64)
    nan = np.isnan(f)
    np.testing.assert_array_equal(r[~nan], want[~nan].view(U64))
    assert np.isnan(r[nan].view(np.float64)).all()


def test_sign_order_and_finite_tests_match_compares():
    rng = np.random.default_rng(3)
    x = _doubles(rng, 100_000)
    hi, lo = split(x)
    mh = hi & U32(0x7FFFFFFF)
    lt = (hi.view(np.int32) < 0) & ((mh | lo) != 0) & ((mh < U32(0x7FF00000)) | ((mh == U32(0x7FF00000)) & (lo == 0)))
    fin = (hi & U32(0x7FF00000)) != U32(0x7FF00000)
    with np.errstate(invalid="ignore"):
        np.testing.assert_array_equal(lt, x < 0)
        np.testing.assert_array_equal(fin, np.isfinite(x))
        for t in (1e-6, 0.5, 3.0, 1e300):
            th, tl = split(np.array([t]))
            le = (hi.view(np.int32) < th.view(np.int32)) | ((hi == th) & (lo <= tl))
            ok = ~np.isnan(x)
            np.testing.assert_array_equal(le[ok], (x <= t)[ok])
