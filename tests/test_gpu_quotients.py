"""Division by constants in the exact kernels.

The PPM interface values divide by 6 (Source/Reconstruction_PPM_MHD_HelperModule.py:
the (dW_c - dW_l) / 6 terms).  The exact kernels compute x / 6 as one multiply and
two FMAs (``mhdk::div6``, Markstein's remainder correction with RN(1/6)); its
comment proves the result correctly rounded for normal-range quotients and routes
every other exponent through the IEEE division.  Here it is compared bit for bit
with NumPy's IEEE division -- the reference's own arithmetic -- on random bit
patterns (every exponent, zeros, subnormals, infinities, NaNs), on every exponent
of the range it handles, and on its edges.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _quotient6(x):
    from pythonmhd_gb300 import _lib
    lib = _lib.load()
    xd = torch.from_numpy(x).to("cuda:0")
    qd = torch.empty_like(xd)
    _lib.check(lib.mhd_quotient6(xd.data_ptr(), qd.data_ptr(), x.size), "mhd_quotient6")
    return qd.cpu().numpy()


def _assert_same(q, ref):
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(q), nan)
    bad = np.flatnonzero(q[~nan].view(np.int64) != ref[~nan].view(np.int64))
    assert bad.size == 0, (q[~nan][bad[:5]], ref[~nan][bad[:5]])


def test_div6_equals_the_ieee_division_on_random_bit_patterns():
    rng = np.random.default_rng(11)
    x = rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, 1 << 22, dtype=np.int64,
                     endpoint=True).view(np.float64)
    with np.errstate(all="ignore"):
        _assert_same(_quotient6(x), x / 6.0)


def test_div6_equals_the_ieee_division_on_every_exponent_and_near_midpoints():
    rng = np.random.default_rng(12)
    n = 1 << 22
    # significands uniform in [1, 2) at every exponent of the range and beyond it; x/6
    # then sits u/6 or u/2 from a rounding midpoint (u = ulp(x/6)), two thirds of them
    # at the proof's minimum distance
    e = rng.integers(-1030, 1024, n)
    x = np.sign(rng.standard_normal(n)) * np.ldexp(rng.uniform(1.0, 2.0, n), e)
    # exact quotients (multiples of 6) and the range's edges
    k = rng.integers(1, 1 << 40, 4096).astype(np.float64)
    edges = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                      np.ldexp(1.0, -999), np.ldexp(1.0, -1000), np.ldexp(1.9999999999999998, 999),
                      np.ldexp(1.0, 1000), np.finfo(np.float64).max, 6.0, -6.0, 3.0, 1.0])
    x = np.concatenate([x, 6.0 * k, -6.0 * k * 2.0 ** -500, edges])
    with np.errstate(all="ignore"):
        _assert_same(_quotient6(x), x / 6.0)


def _softfp(op, x, y=None):
    from pythonmhd_gb300 import _lib
    lib = _lib.load()
    xd = torch.from_numpy(x).to("cuda:0")
    yd = torch.from_numpy(y if y is not None else x).to("cuda:0")
    out = torch.empty_like(xd)
    _lib.check(lib.mhd_softfp(op, xd.data_ptr(), yd.data_ptr(), out.data_ptr(), x.size), "mhd_softfp")
    return out.cpu().numpy()


def _ieee(op, x, y):
    with np.errstate(all="ignore"):
        return [x + y, x - y, x * y, x / y, np.sqrt(x)][op]


def _runs(rng, n):
    """Significand fields made of runs of equal bits (rounding ties, carries, borrows)."""
    f = np.zeros(n, dtype=np.uint64)
    pos = np.zeros(n, dtype=np.int64)
    while (pos < 52).any():
        ln = rng.integers(1, 21, n)
        on = rng.integers(0, 2, n).astype(bool) & (pos < 52)
        mask = ((np.uint64(1) << np.minimum(ln, 52).astype(np.uint64)) - np.uint64(1)) << np.minimum(pos, 63).astype(np.uint64)
        f |= np.where(on, mask, np.uint64(0))
        pos += ln
    return f & np.uint64((1 << 52) - 1)


def _compose(rng, sign, exp, frac):
    return ((sign.astype(np.uint64) << np.uint64(63)) | (exp.astype(np.uint64) << np.uint64(52)) | frac).view(np.float64)


@pytest.mark.parametrize("op", [0, 1, 2, 3, 4], ids=["add", "sub", "mul", "div", "sqrt"])
def test_integer_pipe_arithmetic_equals_ieee_on_random_bit_patterns(op):
    rng = np.random.default_rng(20 + op)
    n = 1 << 22
    x = rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, n, dtype=np.int64, endpoint=True).view(np.float64)
    y = rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, n, dtype=np.int64, endpoint=True).view(np.float64)
    _assert_same(_softfp(op, x, y), _ieee(op, x, y))


@pytest.mark.parametrize("op", [0, 1, 2, 3, 4], ids=["add", "sub", "mul", "div", "sqrt"])
def test_integer_pipe_arithmetic_equals_ieee_on_structured_operands(op):
    """Moderate exponents with runs of equal bits, close magnitudes (cancellation),
    every exponent difference, exact and one-off quotients and squares, and exponents
    at the limits of the fast paths (subnormal and overflowing results)."""
    rng = np.random.default_rng(40 + op)
    n = 1 << 20
    fx = np.where(rng.integers(0, 2, n).astype(bool), _runs(rng, n),
                  rng.integers(0, 1 << 52, n, dtype=np.int64).astype(np.uint64))
    fy = np.where(rng.integers(0, 2, n).astype(bool), _runs(rng, n),
                  rng.integers(0, 1 << 52, n, dtype=np.int64).astype(np.uint64))
    sx, sy = rng.integers(0, 2, n), rng.integers(0, 2, n)
    ex = rng.integers(1023 - 60, 1023 + 61, n)
    moderate = (_compose(rng, sx, ex, fx), _compose(rng, sy, rng.integers(1023 - 60, 1023 + 61, n), fy))
    # y an exponent difference 0..70 below x, or x perturbed in its low bits
    close_y = _compose(rng, sy, np.maximum(ex - rng.integers(0, 71, n), 1), fy)
    flip = (moderate[0].view(np.uint64) ^ (rng.integers(0, 1 << 53, n, dtype=np.int64).astype(np.uint64)
                                          >> rng.integers(0, 53, n).astype(np.uint64)))
    near = flip.view(np.float64) * np.where(rng.integers(0, 2, n).astype(bool), -1.0, 1.0)
    # exact quotients y k and squares k^2, and their neighbours one ulp away
    k = (rng.integers(1, 1 << 40, n) >> rng.integers(0, 38, n)).astype(np.float64)
    prod = moderate[1] * k
    sq = k * k * np.ldexp(1.0, rng.integers(-100, 100, n))
    step = np.where(rng.integers(0, 2, n).astype(bool), 1, -1).astype(np.int64)
    prod1 = (prod.view(np.int64) + step).view(np.float64)
    sq1 = (sq.view(np.int64) + step).view(np.float64)
    # exponents at the limits: sums of exponents near the bottom and the top of the range
    elim = rng.integers(1, 2047, n)
    etop = np.clip(np.where(rng.integers(0, 2, n).astype(bool), 2046, 1) + 1023 - elim
                   + rng.integers(-3, 4, n), 0, 2046)
    lim = (_compose(rng, sx, elim, fx), _compose(rng, sy, etop, fy))
    xs = np.concatenate([moderate[0], moderate[0], moderate[0], prod, prod1, sq, sq1, lim[0]])
    ys = np.concatenate([moderate[1], close_y, near, moderate[1], moderate[1], moderate[1], moderate[1], lim[1]])
    _assert_same(_softfp(op, xs, ys), _ieee(op, xs, ys))
