"""The library's FP64 division (integer-pipe Newton-Raphson reciprocal with
a remainder-corrected last digit, used by the bit-exact assembly, correction,
momentum and geometry kernels) against IEEE division, bit for bit, through
the C-ABI diagnostic scf_diag_divide.

numpy's float64 division is IEEE-754 division rounded to nearest even, the
same operation the reference's Fortran `/` performs."""
import numpy as np
import pytest

from simcoflow_gb300 import projection as P

pytestmark = pytest.mark.gpu


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.uint64)


def check(a, b):
    q = P.divide(a, b)
    with np.errstate(all="ignore"):
        e = a / b
    same = (bits(q) == bits(e)) | (np.isnan(q) & np.isnan(e))
    if not same.all():
        k = np.flatnonzero(~same)[:5]
        raise AssertionError(f"{(~same).sum()} mismatches, e.g. "
                             + ", ".join(f"{a[i].hex()}/{b[i].hex()}: {q[i].hex()} vs {e[i].hex()}"
                                         for i in k))


def test_random_bit_patterns():
    """Every exponent and mantissa pattern, NaN/Inf/zero/subnormal included."""
    rng = np.random.default_rng(11)
    n = 4_000_000
    a = rng.integers(0, 2**64, n, dtype=np.uint64).view(np.float64)
    b = rng.integers(0, 2**64, n, dtype=np.uint64).view(np.float64)
    check(a, b)


def test_moderate_exponents():
    """The normal-range fast path: exponents within 2^+-60 of each other."""
    rng = np.random.default_rng(12)
    n = 4_000_000
    a = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-60, 61, n)) * rng.choice([-1, 1], n)
    b = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-60, 61, n)) * rng.choice([-1, 1], n)
    check(a, b)


def test_sparse_and_dense_mantissas():
    """Significands with few bits set or cleared (powers of two, 1 - ulp,
    all ones): the digit-correction and carry edges."""
    rng = np.random.default_rng(13)
    n = 1_000_000
    def pattern():
        m = np.zeros(n, dtype=np.uint64)
        for _ in range(3):
            on = rng.random(n) < 0.6
            m |= np.where(on, np.uint64(1) << rng.integers(0, 52, n).astype(np.uint64),
                          np.uint64(0))
        flip = rng.random(n) < 0.5
        m = np.where(flip, m ^ np.uint64(0xFFFFFFFFFFFFF), m)
        e = rng.integers(1013, 1033, n).astype(np.uint64)
        return ((e << np.uint64(52)) | m).view(np.float64)
    check(pattern(), pattern())


def test_near_exact_quotients():
    """a within a few ulps of b*q for short q: quotients on or next to
    representable values, where the remainder decides the last bit."""
    rng = np.random.default_rng(14)
    n = 1_000_000
    b = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-20, 21, n))
    q = rng.integers(1, 2**20, n) * np.exp2(rng.integers(-30, 10, n))
    a = (b * q).view(np.uint64) + rng.integers(-2, 3, n).astype(np.int64).view(np.uint64)
    check(a.view(np.float64), b)


def test_power_of_two_divisors():
    """Divisors 2^k (uniform grid spacings, unit densities), which take the
    exponent-only path, over the whole exponent range: quotients in the
    normal range, next to overflow and down into the subnormals."""
    rng = np.random.default_rng(16)
    n = 1_000_000
    a = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-1000, 1000, n)) * rng.choice([-1, 1], n)
    b = np.exp2(rng.integers(-1022, 1024, n).astype(np.float64)) * rng.choice([-1, 1], n)
    check(a, b)
    k = np.arange(-1074, 1024, dtype=np.float64)
    check(np.full(k.size, 1.5), np.exp2(k))
    check(np.full(k.size, 3.0 * 2.0**-1000), np.exp2(k))


def test_range_edges():
    """Results next to overflow and underflow, and the special operands."""
    big, tiny = np.finfo(np.float64).max, np.finfo(np.float64).tiny
    vals = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, big, -big, tiny, -tiny,
                     tiny / 3, 5e-324, 2.0, 0.5, 3.0, 1.0 + 2**-52, 2.0 - 2**-52,
                     1.7976931348623157e308 / 2, 2.2250738585072014e-308 * 2])
    a, b = np.meshgrid(vals, vals)
    check(a.ravel(), b.ravel())
    rng = np.random.default_rng(15)
    n = 200_000
    x = rng.uniform(1.0, 2.0, n)
    check(x * 2.0**1000, rng.uniform(0.1, 1.0, n) * 2.0**-23)   # overflow side
    check(x * 2.0**-1000, rng.uniform(1.0, 9.0, n) * 2.0**22)   # gradual underflow side
    check(x * 2.0**-1021, rng.uniform(0.5, 2.0, n))             # around the smallest normal


# ---------------------------------------------------------------------------
# The library's square root (integer-pipe Newton-Raphson reciprocal square
# root with a remainder-corrected last digit, used by the CLSVOF kernels)
# against numpy's float64 square root (IEEE, rounded to nearest even),
# through scf_diag_sqrt.
# ---------------------------------------------------------------------------
def check_sqrt(a):
    q = P.sqrt(a)
    with np.errstate(all="ignore"):
        e = np.sqrt(a)
    same = (bits(q) == bits(e)) | (np.isnan(q) & np.isnan(e))
    if not same.all():
        k = np.flatnonzero(~same)[:5]
        raise AssertionError(f"{(~same).sum()} mismatches, e.g. "
                             + ", ".join(f"sqrt({a[i].hex()}): {q[i].hex()} vs {e[i].hex()}"
                                         for i in k))


def test_sqrt_random_bit_patterns():
    rng = np.random.default_rng(21)
    check_sqrt(rng.integers(0, 2**64, 8_000_000, dtype=np.uint64).view(np.float64))


def test_sqrt_every_exponent_and_dense_mantissas():
    """All 2046 normal exponents (odd and even), significands near 1, 2 and
    4 (the root's carry into the exponent) and random."""
    rng = np.random.default_rng(22)
    e = np.repeat(np.arange(1, 2047, dtype=np.uint64), 2000)
    m = rng.integers(0, 2**52, e.size, dtype=np.uint64)
    edge = rng.random(e.size) < 0.3
    m = np.where(edge, rng.choice(np.array([0, 1, 2, 2**52 - 1, 2**52 - 2, 2**51, 2**51 - 1],
                                           dtype=np.uint64), e.size), m)
    check_sqrt(((e << np.uint64(52)) | m).view(np.float64))


def test_sqrt_near_squares():
    """x within a few ulps of q^2 for short and long q: roots on or next to
    representable values, where the remainder decides the last bit."""
    rng = np.random.default_rng(23)
    n = 2_000_000
    q = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-500, 500, n))
    q2 = np.floor(rng.uniform(1, 2**26, n)) * np.exp2(rng.integers(-200, 200, n))
    for r in (q, q2):
        a = (r * r).view(np.uint64) + rng.integers(-3, 4, n).astype(np.int64).view(np.uint64)
        check_sqrt(a.view(np.float64))


def test_sqrt_special_operands():
    big, tiny = np.finfo(np.float64).max, np.finfo(np.float64).tiny
    check_sqrt(np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, big, tiny, tiny / 3,
                         5e-324, 2.0, 4.0, 0.25, 3.0, 1.0 + 2**-52, 4.0 - 2**-50, 2.0 - 2**-52,
                         -tiny, -5e-324]))
