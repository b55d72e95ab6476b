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
