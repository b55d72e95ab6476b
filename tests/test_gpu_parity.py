"""GPU parity against the reference, through the C ABI (ctypes) and the drop-in
evolve functions.

* arith="exact": every output of every golden case equals the reference's own
  output bit for bit (the fixtures come from running Source/EvolveFunctions_*.py).
* arith="fast" (FMA contraction): every field within 1e-12 of the reference,
  relative to the field's largest magnitude, over the 1-3 cycles of a case.
"""
import numpy as np
import pytest

from tests.golden_io import HYDRO_KEYS, MHD_KEYS, case_id, golden_files, load
from tests.gpu_util import field_rel_err, run_dropin

FAST_TOL = 1e-12
# States whose eigen-branch choice in the reference is an exact floating-point tie
# (B == 0 everywhere: c_f^2 == a^2; B_t == 0: the slow/Alfven degeneracy).  Any
# change in the last bit of a^2 -- such as a fused multiply-add -- may take the
# other branch, so only the exact arithmetic mode can reproduce them.
EXACT_TIE_CASES = {"mhd_zero_b", "mhd_zero_btran"}

pytestmark = pytest.mark.gpu


def _fast_cases():
    out = []
    for f in golden_files("mhd") + golden_files("hydro"):
        marks = [pytest.mark.xfail(reason="exact tie in the reference's eigen-branch test", strict=False)] \
            if case_id(f) in EXACT_TIE_CASES else []
        out.append(pytest.param(f, marks=marks, id=case_id(f)))
    return out


@pytest.mark.parametrize("path", golden_files("mhd") + golden_files("hydro"), ids=case_id)
def test_exact_matches_reference_bitwise(path):
    physics = "mhd" if case_id(path).startswith("mhd") else "hydro"
    p, i, o = load(path)
    grid, res = run_dropin(physics, p, i, "exact")
    keys = MHD_KEYS if physics == "mhd" else HYDRO_KEYS
    bad = []
    for k, v in zip(keys, res):
        v = np.asarray(v)
        if v.shape != o[k].shape or not np.array_equal(v, o[k]):
            bad.append((k, field_rel_err(v, o[k]) if v.shape == o[k].shape else "shape"))
    assert not bad, bad


@pytest.mark.parametrize("path", _fast_cases())
def test_fast_within_tolerance(path):
    physics = "mhd" if case_id(path).startswith("mhd") else "hydro"
    p, i, o = load(path)
    grid, res = run_dropin(physics, p, i, "fast")
    keys = MHD_KEYS if physics == "mhd" else HYDRO_KEYS
    for k, v in zip(keys, res):
        if k in ("cycle",):
            assert int(v) == int(o[k])
            continue
        assert field_rel_err(v, o[k]) <= FAST_TOL, k


@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_dropin_aliasing_matches_reference(arith):
    """MHD updates grid.faceBx/faceBy in place; hydro updates grid.primVars/consVars in place."""
    path = [f for f in golden_files("mhd") if case_id(f) == "mhd_ot_ppm"][0]
    p, i, o = load(path)
    grid, res = run_dropin("mhd", p, i, arith)
    assert res[2] is grid.faceBx and res[3] is grid.faceBy
    assert res[0] is not grid.primVars
    path = [f for f in golden_files("hydro") if case_id(f) == "hydro_blast_ppm"][0]
    p, i, o = load(path)
    grid, res = run_dropin("hydro", p, i, arith)
    assert res[0] is grid.primVars and res[1] is grid.consVars
