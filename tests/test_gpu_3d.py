"""The 3D hydro step (mhd3d_* in the C ABI, evolve.evolve_3D_hydro).

* against the reference's own outputs (tests/golden/hydro3d_*.npz, made by running
  evolve_3D_hydro), bit for bit in exact arithmetic and to 1e-12 with FMA;
* against the oracle's restatement where the reference cannot run (outflow x,
  PLM) and on larger non-cubic runs, bit for bit;
* at full size through properties: a state uniform along z evolves exactly as
  the 2D step evolves its x-y slice, a uniform state stays uniform, and mass,
  momentum and energy are conserved to round-off on a periodic box.
"""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import hydro3d
from pythonmhd_gb300 import evolve
from pythonmhd_gb300 import initial_conditions as ic
from pythonmhd_gb300.solver import Grid2D, Grid3D
from tests.golden import cases
from tests.golden_io import HYDRO_KEYS, case_id, golden_files, load

pytestmark = pytest.mark.gpu


def _grid(prim, cons, p):
    ny, nx, nz = prim.shape[1:]
    return SimpleNamespace(primVars=prim.copy(), consVars=cons.copy(), dx=p["dx"], dy=p["dy"], dz=p["dz"],
                           BcX=p["bcx"], BcY=p["bcy"], BcZ=p["bcz"], numXCells=nx, numYCells=ny, numZCells=nz)


def _args(p):
    return (p["t_start"], p["t_end"], p["start_cycle"], p["max_cycles"], p["gamma"], p["cfl"], p["min_d"],
            p["min_p"], p["min_e"], p["order"], p["efix"], p["eps"])


@pytest.mark.parametrize("path", golden_files("hydro3d"), ids=case_id)
def test_3d_bitwise_vs_reference(path):
    p, i, o = load(path)
    grid = _grid(i["prim"], i["cons"], p)
    got = evolve.evolve_3D_hydro(grid, *_args(p), arith="exact")
    for k, v in zip(HYDRO_KEYS, got):
        assert np.array_equal(np.asarray(v), o[k]), k
    # the reference's aliasing: the grid's own arrays are updated and returned
    assert got[0] is grid.primVars and got[1] is grid.consVars


@pytest.mark.parametrize("path", golden_files("hydro3d"), ids=case_id)
def test_3d_fast_arith_close_to_reference(path):
    p, i, o = load(path)
    got = evolve.evolve_3D_hydro(_grid(i["prim"], i["cons"], p), *_args(p), arith="fast")
    for k in ("prim", "cons"):
        v = np.asarray(got[HYDRO_KEYS.index(k)])
        for f in range(5):
            scale = max(float(np.max(np.abs(o[k][f]))), 1e-300)
            assert float(np.max(np.abs(v[f] - o[k][f]))) <= 1e-12 * scale, (k, f)


def _rand(shape, seed, mach=0.5):
    ny, nx, nz = shape
    return cases._random_hydro_3d(ny, nx, nz, seed, mach=mach)


@pytest.mark.parametrize("order,bcs", [(2, (0, 1, 1)), (2, (0, 0, 0)), (0, (0, 1, 0)), (1, (1, 1, 1)),
                                       (1, (0, 0, 1))])
def test_3d_bitwise_vs_oracle_where_reference_cannot_run(order, bcs):
    """Outflow x (the reference raises there) and PLM (no reference counterpart)."""
    prim, cons = _rand((6, 7, 5), 21)
    p = dict(dx=1 / 7, dy=1 / 6, dz=1 / 5, bcx=bcs[0], bcy=bcs[1], bcz=bcs[2])
    args = (0.0, 10.0, 0, 4, 1.4, 0.4, 1e-12, 1e-12, 1e-12, order, False, 0.5)
    got = evolve.evolve_3D_hydro(_grid(prim, cons, p), *args[:9], evolve.PLM if order == 1 else order,
                                 *args[10:], arith="exact")
    want = hydro3d.evolve(prim, cons, p["dx"], p["dy"], p["dz"], *bcs, *args)
    for a, b in zip(got, want):
        assert np.array_equal(np.asarray(a), np.asarray(b))


@pytest.mark.parametrize("bcs", [(1, 1, 1), (1, 0, 1)])
def test_3d_larger_run_bitwise_vs_oracle(bcs):
    prim, cons = _rand((24, 32, 20), 22, mach=1.2)
    p = dict(dx=1 / 32, dy=1 / 24, dz=1 / 20, bcx=bcs[0], bcy=bcs[1], bcz=bcs[2])
    args = (0.0, 10.0, 0, 12, 1.4, 0.45, 1e-12, 1e-12, 1e-12, 2, True, 0.3)
    got = evolve.evolve_3D_hydro(_grid(prim, cons, p), *args, arith="exact")
    want = hydro3d.evolve(prim, cons, p["dx"], p["dy"], p["dz"], *bcs, *args)
    assert got[3] == 12
    for a, b in zip(got, want):
        assert np.array_equal(np.asarray(a), np.asarray(b))


@pytest.mark.parametrize("order", [2, 0])
def test_3d_z_uniform_state_evolves_as_the_2d_step(order):
    """A state uniform along a periodic z has equal z fluxes at every z face, so its
    z-flux differences vanish exactly; with dz large enough that the z CFL bound is
    not the smallest, each z slice follows the 2D step bit for bit."""
    ny, nx, nz = 96, 128, 4
    rng = np.random.default_rng(5)
    p2 = np.zeros((5, ny, nx))
    y, x = np.meshgrid((np.arange(ny) + 0.5) / ny, (np.arange(nx) + 0.5) / nx, indexing="ij")
    p2[0] = 1.0 + 0.3 * np.sin(2 * np.pi * x) * np.cos(4 * np.pi * y) + 0.01 * rng.standard_normal((ny, nx))
    p2[1] = 0.6 * np.sin(2 * np.pi * y)
    p2[2] = 0.4 * np.cos(2 * np.pi * x)
    p2[3] = 0.2 * np.sin(2 * np.pi * (x + y))
    p2[4] = 0.7 + 0.2 * np.cos(2 * np.pi * x) * np.sin(2 * np.pi * y)
    c2 = ic.prim_to_cons_hydro(p2, 1.4)
    p3 = np.ascontiguousarray(np.repeat(p2[..., None], nz, axis=3))
    c3 = np.ascontiguousarray(np.repeat(c2[..., None], nz, axis=3))
    g2 = Grid2D(ny, nx, 1 / nx, 1 / ny, 1, 0, 1.4, mhd=False, recon=order, arith="exact")
    g3 = Grid3D(ny, nx, nz, 1 / nx, 1 / ny, 1e3, 1, 0, 1, 1.4, recon=order, arith="exact")
    g2.upload(p2, c2)
    g3.upload(p3, c3)
    r2 = g2.advance(0.0, 10.0, 0, 40, 0.4)
    r3 = g3.advance(0.0, 10.0, 0, 40, 0.4)
    assert r2 == r3
    w2, u2 = g2.download(0)
    w3, u3 = g3.download(0)
    for k in range(nz):
        assert np.array_equal(w3[..., k], w2) and np.array_equal(u3[..., k], u2)
    g2.close()
    g3.close()


def test_3d_uniform_state_stays_uniform_and_totals_are_conserved():
    n = 64
    g = Grid3D(n, n, n, 1 / n, 1 / n, 1 / n, 1, 1, 1, 1.4, recon=2, arith="exact")
    prim = np.zeros((5, n, n, n))
    prim[0] = 1.3
    prim[1], prim[2], prim[3] = 0.2, -0.1, 0.05
    prim[4] = 0.9
    cons = ic.prim_to_cons_hydro(prim, 1.4)
    g.upload(prim, cons)
    g.advance(0.0, 10.0, 0, 6, 0.4)
    w, u = g.download(0)
    for f in range(5):
        assert np.ptp(w[f]) == 0.0 and np.ptp(u[f]) == 0.0
    prim, cons = _rand((n, n, n), 23, mach=1.0)
    g.upload(prim, cons)
    g.advance(0.0, 10.0, 0, 20, 0.4)
    w, u = g.download(0)
    for f in range(5):
        scale = float(np.sum(np.abs(cons[f])))
        assert abs(float(np.sum(u[f])) - float(np.sum(cons[f]))) <= 1e-12 * scale, f
    assert np.isfinite(u).all()
    g.close()
