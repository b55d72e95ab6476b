"""The domain-decomposed step on the GPU: every block of the grid on its own handle
(ranks emulated in one process, in lock step: halo exchange by device copies, the
MIN of the blocks' CFL dts, one cycle each), assembled after several cycles, equals
a single handle's run of the whole grid bit for bit.  The same halo plan and loop
run across processes over torch.distributed (tests/test_decomp_cpu.py runs them on
gloo ranks)."""
import numpy as np
import pytest
import torch

from pythonmhd_gb300 import decomp
from pythonmhd_gb300 import initial_conditions as ic
from pythonmhd_gb300.solver import Grid2D

pytestmark = pytest.mark.gpu
G = 5.0 / 3.0


@pytest.mark.parametrize("ny,nx,py,px,bcx,bcy,recon,steps", [
    (64, 72, 2, 2, 1, 1, 2, 6), (48, 60, 1, 3, 0, 1, 1, 5), (50, 40, 3, 1, 1, 0, 2, 5), (40, 44, 2, 2, 0, 0, 0, 5)])
def test_decomposed_run_equals_the_whole_grid(ny, nx, py, px, bcx, bcy, recon, steps):
    prim, cons, fbx, fby, dx, dy = ic.orszag_tang(nx, ny, gamma=G, rho_perturb=0.02, seed=4)
    if bcx == 0 or bcy == 0:
        fbx, fby = ic.faces_from_cells(prim[4], prim[5], bcx, bcy)
    g = Grid2D(ny, nx, dx, dy, bcx, bcy, G, mhd=True, recon=recon, arith="exact")
    g.upload(prim, cons, fbx, fby)
    t_w, c_w, _ = g.advance(0.0, 1e30, 0, steps, 0.4)
    want = g.download(0)
    g.close()
    dec = decomp.Decomposition(ny, nx, py, px, bcx, bcy, halo=decomp.default_halo(recon))
    blocks = [decomp.DeviceBlock(dec, r, dx, dy, G, recon=recon, state=dec.local_state(r, prim, cons, fbx, fby))
              for r in range(dec.size)]
    try:
        t, c = decomp.run_local(blocks, decomp.halo_plan(dec), 0.0, 1e30, 0, steps, 0.4)
        got = dec.assemble([tuple(a.cpu().numpy() for a in b.state) for b in blocks])
    finally:
        for b in blocks:
            b.close()
    assert (t, c) == (t_w, c_w)
    for a, w in zip(got, want):
        np.testing.assert_array_equal(a, w)


def test_cfl_dt_and_advance_dt_match_the_step():
    """mhd2d_cfl_dt is the dt the step takes; mhd2d_advance_dt with it is the step."""
    prim, cons, fbx, fby, dx, dy = ic.turbulence(64, seed=5, gamma=G)
    a = Grid2D(64, 64, dx, dy, 1, 1, G, mhd=True, recon=2, arith="exact")
    b = Grid2D(64, 64, dx, dy, 1, 1, G, mhd=True, recon=2, arith="exact")
    try:
        a.upload(prim, cons, fbx, fby)
        b.upload(prim, cons, fbx, fby)
        t_a, _, _ = a.advance(0.0, 1e30, 0, 1, 0.4)
        dt = b.cfl_dt(0.4)
        assert dt == t_a
        assert b.advance_dt(0.0, 1e30, 0, dt) == t_a
        for x, y in zip(a.download(0), b.download(0)):
            assert np.array_equal(x, y)
        # the t_end clip applies to a given dt as to the step's own
        b.upload(prim, cons, fbx, fby)
        assert b.advance_dt(0.0, 0.25 * dt, 0, dt) == 0.25 * dt
        torch.cuda.synchronize()
    finally:
        a.close()
        b.close()
