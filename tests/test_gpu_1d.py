"""The 1D step (mhd1d_* in the C ABI, evolve.evolve_1D_mhd / evolve_1D_hydro)
against the reference's own outputs (tests/golden/*1d_*.npz, made by running
evolve_1D_mhd / evolve_1D_hydro) and against the oracle's 1D restatement on
larger runs, bit for bit in exact arithmetic; and the reference's aliasing."""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import evolve1d
from pythonmhd_gb300 import evolve
from tests.golden import cases
from tests.golden_io import HYDRO_KEYS, case_id, golden_files, load

pytestmark = pytest.mark.gpu


def _grid(prim, cons, dx, bcx):
    return SimpleNamespace(primVars=prim.copy(), consVars=cons.copy(), dx=dx, BcX=bcx, numXCells=prim.shape[1])


def _args(p):
    return (p["t_start"], p["t_end"], p["start_cycle"], p["max_cycles"], p["gamma"], p["cfl"], p["min_d"],
            p["min_p"], p["min_e"], p["order"], p["efix"], p["eps"])


@pytest.mark.parametrize("path", golden_files("mhd1d") + golden_files("hydro1d"), ids=case_id)
def test_1d_bitwise_vs_reference(path):
    p, i, o = load(path)
    mhd = case_id(path).startswith("mhd1d")
    fn = evolve.evolve_1D_mhd if mhd else evolve.evolve_1D_hydro
    got = fn(_grid(i["prim"], i["cons"], p["dx"], p["bcx"]), *_args(p), arith="exact")
    for k, v in zip(HYDRO_KEYS, got):
        assert np.array_equal(np.asarray(v), o[k]), k


@pytest.mark.parametrize("physics,order,bc", [("mhd", 2, 0), ("mhd", 0, 1), ("hydro", 2, 0), ("hydro", 2, 1)])
def test_1d_long_runs_bitwise_vs_oracle(physics, order, bc):
    n = 800
    if physics == "mhd":
        prim, cons = cases._brio_wu(n)
        gamma = 2.0
    else:
        prim, cons = cases._sod(n)
        gamma = 1.4
    if bc == 1:   # periodic: a smooth state instead of the jump (the reference's periodic
        x = (np.arange(n) + 0.5) / n   # hydro PPM raises, so this case is against the oracle only)
        prim[0] = 1.0 + 0.2 * np.sin(2 * np.pi * x)
        prim[1] = 0.3
        prim[-1] = 0.8
        from pythonmhd_gb300 import initial_conditions as ic
        cons = ic.prim_to_cons_mhd(prim, gamma) if physics == "mhd" else ic.prim_to_cons_hydro(prim, gamma)
    args = (0.0, 0.1, 0, 150, gamma, 0.8, 1e-12, 1e-12, 1e-12, order, False, 0.5)
    fn = evolve.evolve_1D_mhd if physics == "mhd" else evolve.evolve_1D_hydro
    got = fn(_grid(prim, cons, 1.0 / n, bc), *args, arith="exact")
    ofn = evolve1d.evolve_mhd if physics == "mhd" else evolve1d.evolve_hydro
    want = ofn(prim, cons, 1.0 / n, bc, *args)
    assert got[3] > 20
    for a, b in zip(got, want):
        assert np.array_equal(np.asarray(a), np.asarray(b))


def test_1d_aliasing_follows_the_reference():
    prim, cons = cases._sod(64)
    g = _grid(prim, cons, 1.0 / 64, 0)
    res = evolve.evolve_1D_hydro(g, 0.0, 0.01, 0, 5, 1.4, 0.8, 1e-12, 1e-12, 1e-12, 2, False, 0.5)
    assert res[0] is g.primVars and res[1] is g.consVars        # hydro: updated in place
    mprim, mcons = cases._brio_wu(64)
    mg = _grid(mprim, mcons, 1.0 / 64, 0)
    res = evolve.evolve_1D_mhd(mg, 0.0, 0.01, 0, 5, 2.0, 0.8, 1e-12, 1e-12, 1e-12, 2, False, 0.5)
    assert res[0] is not mg.primVars and np.array_equal(mg.primVars, mprim)   # MHD: new arrays
