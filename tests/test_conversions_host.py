"""The integer-pipe float <-> double conversions of the mixed form
(f2d / d2f in braids-hkt_gb300/csrc/brx_mixed.cu), restated on the same bit
operations in numpy and checked bit for bit against IEEE conversions (numpy's
astype rounds to nearest, ties to even, as the hardware does) over random bit
patterns, both rounding ties, the ends of the float range and special values.
Operands the kernels hand to the hardware conversion are marked and skipped.
"""
import numpy as np

U32, U64 = np.uint32, np.uint64


def d2f_bits(x):
    """double -> float bits; also a mask of the operands that take the hardware path."""
    b = x.view(U64)
    hi = (b >> U64(32)).astype(U32)
    lo = (b & U64(0xFFFFFFFF)).astype(U32)
    zero = ((hi & U32(0x7FFFFFFF)) | lo) == 0
    e = (hi >> U32(20)) & U32(0x7FF)
    hw = ~zero & ((e < 897) | (e > 1150))
    top = ((hi & U32(0xFFFFF)) << U32(3)) | (lo >> U32(29))
    rem = lo & U32(0x1FFFFFFF)
    r = (hi & U32(0x80000000)) | ((e - U32(896)) << U32(23)) | top
    up = (rem > U32(0x10000000)) | ((rem == U32(0x10000000)) & ((top & U32(1)) == 1))
    r = r + up.astype(U32)
    r = np.where(zero, hi & U32(0x80000000), r)
    return r, hw


def f2d_bits(f):
    b = f.view(U32)
    e = (b >> U32(23)) & U32(0xFF)
    zero = (b & U32(0x7FFFFFFF)) == 0
    hw = ~zero & ((e == 0) | (e == 0xFF))
    hi = (b & U32(0x80000000)) | ((e + U32(896)) << U32(20)) | ((b & U32(0x7FFFFF)) >> U32(3))
    lo = b << U32(29)
    hi = np.where(zero, b & U32(0x80000000), hi)
    lo = np.where(zero, U32(0), lo)
    return (hi.astype(U64) << U64(32)) | lo.astype(U64), hw


def _doubles(rng, n):
    bits = rng.integers(0, 2 ** 63, n, dtype=np.int64).astype(U64) | (rng.integers(0, 2, n).astype(U64) << U64(63))
    x = bits.view(np.float64)
    # values around the float range, ties at every exponent, rounding carries
    mant = rng.integers(0, 2 ** 23, n).astype(U64)
    exps = rng.integers(897, 1151, n).astype(U64)
    tie = (exps << U64(52)) | (mant << U64(29)) | U64(1 << 28)
    carry = (exps << U64(52)) | (U64(0x7FFFFF) << U64(29)) | U64(1 << 28) | U64(1)
    near = rng.standard_normal(n) * np.exp(rng.uniform(-80, 80, n))
    special = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 3.4028234663852886e38, 3.4028235677973366e38,
                        1.1754943508222875e-38, 1.1754942106924411e-38, 1e-45, 2.0 ** -149, 2.0 ** -150, 1e300, 5e-324])
    return np.concatenate([x, tie.view(np.float64), carry.view(np.float64), near, special])


def test_double_to_float_matches_ieee_round_to_nearest():
    rng = np.random.default_rng(1)
    x = _doubles(rng, 200_000)
    r, hw = d2f_bits(x)
    with np.errstate(over="ignore"):
        want = x.astype(np.float32).view(U32)
    ok = ~hw
    assert ok.sum() > 300_000
    np.testing.assert_array_equal(r[ok], want[ok])


def test_float_to_double_is_exact():
    rng = np.random.default_rng(2)
    f = rng.integers(0, 2 ** 32, 500_000, dtype=np.uint64).astype(U32).view(np.float32)
    f = np.concatenate([f, np.array([0.0, -0.0, 1.0, -2.5, np.inf, -np.inf, np.nan, 1e-45, 3.4e38], np.float32)])
    r, hw = f2d_bits(f)
    with np.errstate(invalid="ignore"):
        want = f.astype(np.float64).view(U64)
    ok = ~hw
    assert ok.sum() > 490_000
    np.testing.assert_array_equal(r[ok], want[ok])


def test_sign_test_matches_compare():
    """lt_zero (brx_mixed.cu): x < 0 from the bit pattern, false for -0 and NaN."""
    rng = np.random.default_rng(3)
    x = _doubles(rng, 100_000)
    b = x.view(np.int64)
    mag = b & np.int64(0x7FFFFFFFFFFFFFFF)
    got = (b < 0) & (mag != 0) & (mag <= np.int64(0x7FF0000000000000))
    with np.errstate(invalid="ignore"):
        np.testing.assert_array_equal(got, x < 0)
