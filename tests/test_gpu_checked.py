"""The bounds-checked build (arithmetic mode "checked"): the exact kernels with every
global index of the 2D, 1D and batched bodies checked before use.  On small, odd and
degenerate grids -- 8x8, 16x12, odd sizes, 2- and 3-cell sides -- with every
reconstruction, both physics and every boundary combination, no check fails (the
device error word stays clear, the advance returns MHD_OK) and the results equal the
exact build's bit for bit (the checks add no arithmetic)."""
import numpy as np
import pytest

from pythonmhd_gb300 import initial_conditions as ic
from pythonmhd_gb300.solver import Batch2D, Grid1D, Grid2D
from tests.golden.cases import _smooth_random

pytestmark = pytest.mark.gpu
G = 5.0 / 3.0
SHAPES = [(8, 8), (16, 12), (12, 16), (7, 5), (5, 9), (13, 11), (3, 2), (2, 3), (2, 2)]


def _state(ny, nx, mhd, bcx, bcy, seed):
    rng = np.random.default_rng(seed)
    nv = 8 if mhd else 5
    prim = np.zeros((nv, ny, nx))
    prim[0] = 0.5 + np.abs(1.0 + _smooth_random(rng, ny, nx))
    for k in (1, 2, 3):
        prim[k] = 0.5 * _smooth_random(rng, ny, nx)
    if mhd:
        for k in (4, 5, 6):
            prim[k] = 0.7 * _smooth_random(rng, ny, nx) + 0.3 * rng.standard_normal()
        prim[7] = 0.4 + np.abs(0.5 + _smooth_random(rng, ny, nx))
        fbx, fby = ic.faces_from_cells(prim[4], prim[5], bcx, bcy)
        return prim, ic.prim_to_cons_mhd(prim, G), fbx, fby
    prim[4] = 0.4 + np.abs(0.5 + _smooth_random(rng, ny, nx))
    return prim, ic.prim_to_cons_hydro(prim, G)


def _run(arith, shape, mhd, recon, bcx, bcy, st):
    ny, nx = shape
    g = Grid2D(ny, nx, 1.0 / nx, 1.0 / ny, bcx, bcy, G, mhd=mhd, recon=recon, arith=arith)
    try:
        g.upload(*st)
        t, c, _ = g.advance(0.0, 1e30, 0, 3, 0.4)
        info = g.check_info() if arith == "checked" else (0, 0)
        return (t, c), g.download(0), info
    finally:
        g.close()


@pytest.mark.parametrize("mhd", [True, False])
@pytest.mark.parametrize("recon", [0, 1, 2])
def test_checked_build_finds_nothing_and_matches_exact(mhd, recon):
    seed = 0
    for shape in SHAPES:
        for bcx, bcy in ((0, 0), (1, 1), (0, 1), (1, 0)):
            seed += 1
            st = _state(*shape, mhd, bcx, bcy, seed)
            tc_c, out_c, info = _run("checked", shape, mhd, recon, bcx, bcy, st)
            tc_e, out_e, _ = _run("exact", shape, mhd, recon, bcx, bcy, st)
            assert info == (0, 0), (shape, bcx, bcy)
            assert tc_c == tc_e
            for a, b in zip(out_c, out_e):
                assert np.array_equal(a, b), (shape, bcx, bcy)


@pytest.mark.parametrize("mhd", [True, False])
def test_checked_build_1d(mhd):
    for n in (2, 3, 7, 16):
        for bc in (0, 1):
            prim = np.zeros((8 if mhd else 5, n))
            prim[0] = 1.0 + 0.1 * np.arange(n)
            prim[-1] = 1.0 + 0.05 * np.arange(n)
            if mhd:
                prim[4] = 0.75
                prim[5] = 0.3
            cons = ic.prim_to_cons_mhd(prim[:, None, :], G)[:, 0] if mhd else \
                ic.prim_to_cons_hydro(prim[:, None, :], G)[:, 0]
            outs = []
            for arith in ("checked", "exact"):
                g = Grid1D(n, 1.0 / n, bc, G, mhd=mhd, recon=2, arith=arith)
                g.upload(prim, cons)
                g.advance(0.0, 1e30, 0, 3, 0.4)
                outs.append(g.download(0))
                if arith == "checked":
                    assert g.check_info() == (0, 0)
                g.close()
            for a, b in zip(*outs):
                assert np.array_equal(a, b)


def test_checked_build_batched():
    insts = ic.orszag_tang_batch(count=5, seed=4, sizes=(8, 12, 16, 20))
    insts[1]["bcx"] = 0
    insts[3]["bcy"] = 0
    outs = []
    for arith in ("checked", "exact"):
        b = Batch2D(insts, mhd=True, recon=2, arith=arith)
        for k, inst in enumerate(insts):
            fbx, fby = inst["fbx"], inst["fby"]
            if inst["bcx"] == 0 or inst["bcy"] == 0:
                fbx, fby = ic.faces_from_cells(inst["prim"][4], inst["prim"][5], inst["bcx"], inst["bcy"])
            b.upload(k, inst["prim"], inst["cons"], fbx, fby)
        b.advance(0.0, 1e30, 0, 3, 0.4)
        outs.append([b.download(k) for k in range(len(insts))])
        b.close()
    for a, w in zip(*outs):
        for x, y in zip(a, w):
            assert np.array_equal(x, y)
