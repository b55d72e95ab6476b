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


@pytest.mark.parametrize("tile_width,fuse", [(32, 1), (64, 2), (128, 2)])
def test_launch_shape_does_not_change_results(tile_width, fuse):
    insts = ic.orszag_tang_batch(count=5, seed=9, sizes=(16, 40, 72))
    outs = []
    for shape in [(128, 1, 304), (tile_width, fuse, 152)]:
        b = Batch2D(insts, mhd=True, recon=2, arith="exact")
        b.configure(*shape)
        for k, inst in enumerate(insts):
            b.upload(k, inst["prim"], inst["cons"], inst["fbx"], inst["fby"])
        b.advance(0.0, 1e30, 0, 4, 0.4)
        outs.append([b.download(k) for k in range(len(insts))])
        b.close()
    for a, w in zip(outs[0], outs[1]):
        for x, y in zip(a, w):
            assert np.array_equal(x, y)


def test_autotuner_picks_a_shape_and_restores_the_state(tmp_path, monkeypatch):
    from pythonmhd_gb300 import autotune
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "tune.json"))
    insts = ic.orszag_tang_batch(count=6, seed=2, sizes=(32, 64, 96))
    b = Batch2D(insts, mhd=True, recon=1, arith="exact")
    rec = autotune.tune_batch(b, insts, recon=1, cycles=1)
    assert rec["tile_width"] in (64, 128) and rec["fuse"] in (1, 2) and len(rec["trials"]) == 8
    b.advance(0.0, 1e30, 0, 2, 0.4)
    got = [b.download(k) for k in range(len(insts))]
    b.close()
    ref = Batch2D(insts, mhd=True, recon=1, arith="exact")
    for k, inst in enumerate(insts):
        ref.upload(k, inst["prim"], inst["cons"], inst["fbx"], inst["fby"])
    ref.advance(0.0, 1e30, 0, 2, 0.4)
    for k in range(len(insts)):
        for x, y in zip(got[k], ref.download(k)):
            assert np.array_equal(x, y)
    ref.close()
    again = Batch2D(insts, mhd=True, recon=1, arith="exact")
    assert autotune.tune_batch(again, insts, recon=1)["cached"]
    again.close()


@pytest.mark.parametrize("recon", [0, 1, 2])
def test_batch_equals_the_oracle_directly(recon):
    """Each batched instance against the oracle's own evolve loop (oracle/mhd2d.py, the
    reference's evolve_2D_mhd restated and pinned to it), not through the single-grid
    path: four uneven instances with their own gamma, B0, boundary conditions, stop
    times and cycle limits, PPM, PLM and first order, bit for bit in exact arithmetic."""
    from oracle import mhd2d
    insts = ic.orszag_tang_batch(count=4, seed=12, sizes=(16, 24, 40))
    insts[1]["bcx"] = 0
    insts[3]["bcy"] = 0
    t_end = np.array([1.0, 0.004, 1.0, 1.0])
    max_cycles = np.array([5, 6, 3, 4])
    b = Batch2D(insts, mhd=True, recon=recon, arith="exact")
    for k, inst in enumerate(insts):
        b.upload(k, inst["prim"], inst["cons"], inst["fbx"], inst["fby"])
    t_out, c_out = b.advance(0.0, t_end, 0, max_cycles, 0.4)
    for k, inst in enumerate(insts):
        r = mhd2d.evolve(inst["prim"], inst["cons"], inst["fbx"], inst["fby"], inst["dx"], inst["dy"], inst["bcx"],
                         inst["bcy"], 0.0, t_end[k], 0, max_cycles[k], inst["gamma"], 0.4, 1e-12, 1e-12, 1e-12,
                         recon, False, 0.5)
        assert (t_out[k], c_out[k]) == (r[4], r[5]), k
        for a, w in zip(b.download(k), r[:4]):
            assert np.array_equal(a, w), k
        for a, w in zip(b.download(k, which=1), r[6:10]):
            assert np.array_equal(a, w), k
    b.close()
