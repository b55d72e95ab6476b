"""Batched form: many uneven grids advanced by one persistent launch per stage.

Each instance of a batch must end bitwise where the single-grid entry point
(itself bitwise equal to the reference in exact arithmetic) ends, with its own
dt, time and cycle count -- including instances whose stop times differ."""
import numpy as np
import pytest

from pythonmhd_gb300 import initial_conditions as ic
from pythonmhd_gb300.solver import Batch2D, Grid2D
from tests.gpu_util import field_rel_err

pytestmark = pytest.mark.gpu


def _single(inst, mhd, recon, t_end, cycles, arith):
    g = Grid2D(inst["ny"], inst["nx"], inst["dx"], inst["dy"], inst["bcx"], inst["bcy"], inst["gamma"], mhd=mhd,
               recon=recon, arith=arith)
    if mhd:
        g.upload(inst["prim"], inst["cons"], inst["fbx"], inst["fby"])
    else:
        g.upload(inst["prim"], inst["cons"])
    t, c, _ = g.advance(0.0, t_end, 0, cycles, 0.4)
    out = g.download(0)
    g.close()
    return out, t, c


@pytest.mark.parametrize("recon,arith", [(1, "exact"), (2, "exact"), (1, "fast"), (0, "exact")])
def test_batch_equals_single_grid_runs_mhd(recon, arith):
    insts = ic.orszag_tang_batch(count=7, seed=3, sizes=(16, 24, 40, 64, 72))
    insts[2]["bcx"] = 0            # mix boundary conditions too
    insts[4]["bcy"] = 0
    b = Batch2D(insts, mhd=True, recon=recon, arith=arith)
    for k, inst in enumerate(insts):
        b.upload(k, inst["prim"], inst["cons"], inst["fbx"], inst["fby"])
    t_end = np.array([1.0, 1.0, 0.01, 1.0, 1.0, 0.02, 1.0])
    max_cycles = np.array([6, 4, 6, 9, 6, 6, 1])
    t_out, c_out = b.advance(0.0, t_end, 0, max_cycles, 0.4)
    for k, inst in enumerate(insts):
        want, t, c = _single(inst, True, recon, t_end[k], max_cycles[k], arith)
        got = b.download(k)
        assert c_out[k] == c, k
        if arith == "exact":
            # same per-item bodies, no contraction: bitwise equal
            assert t_out[k] == t, k
            for a, w in zip(got, want):
                assert np.array_equal(a, w), k
        else:
            # FMA contraction may differ between the batched and single kernels' inlining
            assert abs(t_out[k] - t) <= 1e-12 * t
            for a, w in zip(got, want):
                assert field_rel_err(a, w) <= 1e-12, k
    b.close()


def test_batch_equals_single_grid_runs_hydro():
    insts = []
    rng = np.random.default_rng(1)
    for k, (ny, nx) in enumerate([(20, 36), (48, 16), (32, 32)]):
        prim = np.zeros((5, ny, nx))
        prim[0] = 1.0 + 0.1 * rng.standard_normal((ny, nx))
        prim[1] = 0.2 * rng.standard_normal((ny, nx))
        prim[4] = 1.0
        prim[4, ny // 3:ny // 2, nx // 3:nx // 2] = 8.0
        g = 1.4 + 0.1 * k
        insts.append(dict(prim=prim, cons=ic.prim_to_cons_hydro(prim, g), ny=ny, nx=nx, dx=1 / nx, dy=1 / ny,
                          bcx=k % 2, bcy=1, gamma=g))
    b = Batch2D(insts, mhd=False, recon=2, arith="exact")
    for k, inst in enumerate(insts):
        b.upload(k, inst["prim"], inst["cons"])
    t_out, c_out = b.advance(0.0, 1.0, 0, 5, 0.4)
    for k, inst in enumerate(insts):
        want, t, c = _single(inst, False, 2, 1.0, 5, "exact")
        got = b.download(k)
        assert c_out[k] == c and t_out[k] == t
        for a, w in zip(got, want):
            assert np.array_equal(a, w)
    b.close()


def test_batch_of_256_uneven_instances_runs_and_conserves():
    insts = ic.orszag_tang_batch(count=256, seed=0)
    b = Batch2D(insts, mhd=True, recon=1, arith="exact")
    for k, inst in enumerate(insts):
        b.upload(k, inst["prim"], inst["cons"], inst["fbx"], inst["fby"])
    t_out, c_out = b.advance(0.0, 1e30, 0, 3, 0.4)
    assert (c_out == 3).all() and (t_out > 0).all()
    for k in (0, 77, 255):
        p, c, bx, by = b.download(k)
        assert np.isfinite(c).all()
        assert abs(c[0].sum() - insts[k]["cons"][0].sum()) <= 1e-12 * insts[k]["cons"][0].sum()
        assert np.array_equal(bx[:, 0], bx[:, -1])
    b.close()
