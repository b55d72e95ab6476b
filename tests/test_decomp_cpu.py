"""Spatial domain decomposition (pythonmhd_gb300/decomp.py), on the CPU.

* The halo width covers the step's footprint: one perturbed cell changes cells and
  faces at most FOOTPRINT[recon] cells away after one cycle (the oracle, which is
  the reference's step bit for bit).
* The halo plan is exact: blocks whose halos were spoiled get back, from the
  exchange alone, exactly the halos cut from the whole grid -- for periodic and
  outflow edges, splits along x, y and both, blocks of uneven sizes.
* Two gloo ranks run the decomposed evolve loop (halo exchange by point-to-point
  messages, dt by a MIN all-reduce) with the oracle's cycle on each block, and the
  assembled result equals the oracle's run of the whole grid bit for bit.
"""
import os
import tempfile

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from oracle import mhd2d
from pythonmhd_gb300 import decomp
from pythonmhd_gb300 import initial_conditions as ic
from tests.golden.cases import _smooth_random

G = 5.0 / 3.0
FLOORS = (1e-12, 1e-12, 1e-12)


def _state(ny, nx, seed, bcx=1, bcy=1):
    """A smooth random MHD state with face B from the cell B (the golden cases' generator)."""
    rng = np.random.default_rng(seed)
    prim = np.zeros((8, ny, nx))
    prim[0] = 0.5 + np.abs(1.0 + _smooth_random(rng, ny, nx))
    for k in (1, 2, 3):
        prim[k] = 0.5 * _smooth_random(rng, ny, nx)
    for k in (4, 5, 6):
        prim[k] = 0.7 * _smooth_random(rng, ny, nx) + 0.3 * rng.standard_normal()
    prim[7] = 0.4 + np.abs(0.5 + _smooth_random(rng, ny, nx))
    fbx, fby = ic.faces_from_cells(prim[4], prim[5], bcx, bcy)
    return prim, ic.prim_to_cons_mhd(prim, G), fbx, fby, 1.0 / nx, 1.0 / ny


@pytest.mark.parametrize("recon", [0, 1, 2])
def test_footprint_of_one_cycle(recon):
    prim, cons, fbx, fby, dx, dy = ic.turbulence(32, seed=3, gamma=G)
    dt = mhd2d.calc_dt(cons, fbx, fby, G, 0.4, dx, dy)
    base = mhd2d.cycle(prim, cons, fbx, fby, dt, dx, dy, 1, 1, G, *FLOORS, recon, False, 0.5)
    reach = 0
    rng = np.random.default_rng(recon)
    for _ in range(4):
        j0, i0 = (int(v) for v in rng.integers(8, 24, 2))
        p2, c2 = prim.copy(), cons.copy()
        p2[:, j0, i0] *= 1.001
        c2[:, j0, i0] *= 1.001
        out = mhd2d.cycle(p2, c2, fbx, fby, dt, dx, dy, 1, 1, G, *FLOORS, recon, False, 0.5)
        for a, b, dj, di in ((out[0], base[0], 0, 0), (out[1], base[1], 0, 0), (out[2], base[2], 0, 0),
                             (out[3], base[3], 0, 0)):
            diff = a != b
            if diff.ndim == 3:
                diff = diff.any(axis=0)
            js, is_ = np.nonzero(diff)
            reach = max(reach, int(np.max(np.abs(js - j0))), int(np.max(np.abs(is_ - i0))))
    assert 0 < reach <= decomp.FOOTPRINT[recon]
    assert decomp.default_halo(recon) > decomp.FOOTPRINT[recon]


@pytest.mark.parametrize("ny,nx,py,px,bcx,bcy", [
    (20, 24, 1, 2, 1, 1), (20, 24, 2, 1, 1, 1), (22, 27, 2, 3, 1, 1), (22, 27, 2, 3, 0, 1),
    (22, 27, 3, 2, 1, 0), (21, 25, 2, 2, 0, 0), (12, 30, 1, 3, 1, 0)])
def test_halo_plan_restores_every_halo(ny, nx, py, px, bcx, bcy):
    prim, cons, fbx, fby, dx, dy = _state(ny, nx, 5, bcx, bcy)
    dec = decomp.Decomposition(ny, nx, py, px, bcx, bcy, halo=4)
    want = [dec.local_state(r, prim, cons, fbx, fby) for r in range(dec.size)]
    got = []
    for r, st in enumerate(want):
        b = dec.blocks[r]
        iy, ix = b.interior
        spoiled = [np.full_like(a, np.nan) for a in st]
        spoiled[0][:, iy, ix] = st[0][:, iy, ix]
        spoiled[1][:, iy, ix] = st[1][:, iy, ix]
        spoiled[2][iy, ix.start:ix.stop + 1] = st[2][iy, ix.start:ix.stop + 1]
        spoiled[3][iy.start:iy.stop + 1, ix] = st[3][iy.start:iy.stop + 1, ix]
        # an outflow edge of the whole grid has no halo: its outer values are the block's own
        got.append(spoiled)
    decomp.exchange_local(decomp.halo_plan(dec), got)
    for r in range(dec.size):
        for a, w in zip(got[r], want[r]):
            np.testing.assert_array_equal(a, w)
    for a, w in zip(dec.assemble(want), (prim, cons, fbx, fby)):
        np.testing.assert_array_equal(a, w)


class OracleBlock:
    """One rank's extended block advanced by the oracle (the reference's step)."""

    def __init__(self, dec, rank, state, dx, dy, recon):
        self.b = dec.blocks[rank]
        self.state = tuple(torch.from_numpy(np.array(a)) for a in state)
        self.dx, self.dy, self.recon = dx, dy, recon

    def cfl_dt(self, cfl):
        p, c, bx, by = (t.numpy() for t in self.state)
        return mhd2d.calc_dt(c, bx, by, G, cfl, self.dx, self.dy)

    def step(self, t, t_end, cyc, dt):
        dt = decomp.clip_dt(t, dt, t_end)
        out = mhd2d.cycle(*(a.numpy() for a in self.state), dt, self.dx, self.dy, self.b.bcx, self.b.bcy, G,
                          *FLOORS, self.recon, False, 0.5)
        for a, o in zip(self.state, out):
            a.copy_(torch.from_numpy(o))
        return t + dt


def _rank_main(rank, world, port, cfg, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ny, nx, py, px, bcx, bcy, recon, steps = cfg
        prim, cons, fbx, fby, dx, dy = _state(ny, nx, 11, bcx, bcy)
        dec = decomp.Decomposition(ny, nx, py, px, bcx, bcy, halo=decomp.default_halo(recon))
        blk = OracleBlock(dec, rank, dec.local_state(rank, prim, cons, fbx, fby), dx, dy, recon)
        plan = decomp.halo_plan(dec)
        t, cyc = decomp.run_block(blk, lambda st: decomp.exchange_dist(plan, rank, st),
                                  lambda x: decomp.global_dt(x), 0.0, 1e30, 0, steps, 0.4)
        np.savez(os.path.join(out_dir, f"r{rank}.npz"), *[a.numpy() for a in blk.state], t=t, cyc=cyc)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("cfg", [(24, 30, 1, 2, 1, 1, 2, 4), (26, 20, 2, 1, 1, 0, 2, 4), (24, 30, 1, 2, 0, 1, 1, 3)])
def test_two_gloo_ranks_equal_the_whole_grid_bitwise(cfg):
    ny, nx, py, px, bcx, bcy, recon, steps = cfg
    port = 29500 + (os.getpid() % 1000) + 7 * recon + ny
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank_main, args=(2, port, cfg, d), nprocs=2, start_method="spawn")
        res = [np.load(os.path.join(d, f"r{r}.npz")) for r in range(2)]
        locals_ = [tuple(z[f"arr_{k}"] for k in range(4)) for z in res]
        t = [float(z["t"]) for z in res]
        cyc = [int(z["cyc"]) for z in res]
    prim, cons, fbx, fby, dx, dy = _state(ny, nx, 11, bcx, bcy)
    dec = decomp.Decomposition(ny, nx, py, px, bcx, bcy, halo=decomp.default_halo(recon))
    want = mhd2d.evolve(prim, cons, fbx, fby, dx, dy, bcx, bcy, 0.0, 1e30, 0, steps, G, 0.4, *FLOORS, recon, False,
                        0.5)
    assert t[0] == t[1] == want[4] and cyc[0] == cyc[1] == want[5]
    for a, w in zip(dec.assemble(locals_), want[:4]):
        np.testing.assert_array_equal(a, w)
