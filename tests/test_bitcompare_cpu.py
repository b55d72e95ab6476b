"""The bit-pattern comparison rules of ``csrc/mhd_math.cuh`` (``okey``, ``is_pos``,
``is_nonpos``, ``is_neg``, ``is_nonneg``, ``is_zero``, ``dgt``, ``dlt``, ``dmax``,
``dmin``) and of the generated adjoint code (``dsl_*``), restated on int64 views in
NumPy and checked against IEEE float64 comparisons on every pair of a set of special
values (both zeros, subnormals, the extremes, infinities) and on random values.

The step's exact mode relies on these rules being equal to the IEEE comparisons for
every non-NaN operand; the GPU parity tests check the kernels themselves.
"""
import numpy as np

INT64_MIN = np.int64(-(2 ** 63))


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def okey(x):
    b = bits(x)
    # INT64_MIN - b for negative b: well defined (no overflow) for b in [INT64_MIN, -1]
    with np.errstate(over="ignore"):
        return np.where(b < 0, INT64_MIN - b, b)


def is_pos(x): return bits(x) > 0
def is_nonpos(x): return bits(x) <= 0
def is_neg(x): return okey(x) < 0
def is_nonneg(x): return okey(x) >= 0
def is_zero(x): return (bits(x).view(np.uint64) << np.uint64(1)) == 0
def dgt(a, b): return okey(a) > okey(b)
def dlt(a, b): return okey(a) < okey(b)
def dmax(a, b): return np.where(dgt(a, b), a, b)
def dmin(a, b): return np.where(dlt(a, b), a, b)


def _values():
    tiny = np.finfo(np.float64).tiny
    big = np.finfo(np.float64).max
    sub = np.float64(5e-324)
    special = np.array([0.0, -0.0, sub, -sub, 2 * sub, tiny, -tiny, tiny * (1 - 2 ** -52), 1e-300, -1e-300, 0.5,
                        -0.5, 1.0, -1.0, np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0), -np.nextafter(1.0, 2.0), 1e12,
                        -1e12, big, -big, np.inf, -np.inf])
    rng = np.random.default_rng(5)
    rand = np.concatenate([rng.standard_normal(400) * 10.0 ** rng.integers(-300, 300, 400),
                           rng.integers(-3, 4, 200).astype(np.float64)])
    return np.concatenate([special, rand])


def _same_bits(a, b):
    return np.array_equal(bits(a), bits(b))


def test_sign_tests_match_ieee():
    v = _values()
    assert np.array_equal(is_pos(v), v > 0.0)
    assert np.array_equal(is_nonpos(v), v <= 0.0)
    assert np.array_equal(is_neg(v), v < 0.0)
    assert np.array_equal(is_nonneg(v), v >= 0.0)
    assert np.array_equal(is_zero(v), v == 0.0)


def test_pair_compares_and_select_match_ieee():
    v = _values()
    a, b = np.meshgrid(v, v, indexing="ij")
    a, b = a.ravel(), b.ravel()
    assert np.array_equal(dgt(a, b), a > b)
    assert np.array_equal(dlt(a, b), a < b)
    assert np.array_equal(okey(a) == okey(b), a == b)
    assert np.array_equal(okey(a) >= okey(b), a >= b)
    assert np.array_equal(okey(a) <= okey(b), a <= b)
    # dmax / dmin are a > b ? a : b and a < b ? a : b, bit for bit (signed zeros included)
    assert _same_bits(dmax(a, b), np.where(a > b, a, b))
    assert _same_bits(dmin(a, b), np.where(a < b, a, b))


def test_zero_signs_are_kept_as_ieee_selects_keep_them():
    pz, nz = np.float64(0.0), np.float64(-0.0)
    # +0 > -0 is false in IEEE, so max(+0, -0) returns the second operand
    assert bits(dmax(pz, nz)) == bits(nz)
    assert bits(dmax(nz, pz)) == bits(pz)
    assert bits(dmin(pz, nz)) == bits(nz)
    assert bits(dmin(nz, pz)) == bits(pz)
