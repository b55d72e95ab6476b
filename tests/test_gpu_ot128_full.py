"""Full-length runs of the plain CPU-runnable workload through ``evolve_2D_mhd``:
Orszag-Tang 128 x 128 periodic, gamma 5/3, CFL 0.4, from t = 0 to t = 0.5 (about
400 cycles), bit for bit against the digests of
* the reference's own PPM run (``reference_ppm``), and
* the oracle's PLM run (``oracle_plm``; the reference has no PLM),
made by ``tests/golden/make_ot128_digests.py``.  Equal SHA-256 digests of the final
prim, cons, faceBx and faceBy mean equal states after the whole run.
"""
import json
from types import SimpleNamespace

import numpy as np
import pytest

from pythonmhd_gb300 import evolve
from tests.golden import make_ot128_digests as ot

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("key,order", [("reference_ppm", 2), ("oracle_plm", evolve.PLM)])
def test_ot128_full_run_bitwise(key, order):
    with open(ot.OUT) as f:
        want = json.load(f)[key]
    prim, cons, fbx, fby, dx, dy = ot.initial_state()
    grid = SimpleNamespace(primVars=prim.copy(), consVars=cons.copy(), faceBx=fbx.copy(), faceBy=fby.copy(),
                           dx=dx, dy=dy, BcX=1, BcY=1)
    r = evolve.evolve_2D_mhd(grid, 0.0, ot.T_END, 0, ot.MAX_CYCLES, ot.GAMMA, ot.CFL, *ot.FLOORS, order, False,
                             0.5, arith="exact")
    assert (float(r[4]), int(r[5])) == (want["t"], want["cycle"])
    assert ot.digest(*r[:4]) == want["sha256"]
    # what the digest implies, stated as properties: point symmetry of the vortex and
    # div B at roundoff after ~400 cycles
    rho = r[0][0]
    assert np.max(np.abs(rho - rho[::-1, ::-1])) <= 1e-11 * np.max(rho)
    div = (r[2][:, 1:] - r[2][:, :-1]) / dx + (r[3][1:, :] - r[3][:-1, :]) / dy
    assert np.max(np.abs(div)) * dx <= 1e-13 * np.max(np.abs(r[2]))


def test_ot128_full_run_fast_arithmetic_per_cycle():
    """The fast arithmetic (FMA contraction, branch-deciding scalars uncontracted) along
    the whole reference PPM run: at every one of its ~400 cycles, one fast cycle from
    the reference's state (the exact chain, whose end is checked against the
    reference's digest) stays within 1e-12 of the reference's next state."""
    from pythonmhd_gb300.solver import Grid2D
    from tests.gpu_util import field_rel_err
    with open(ot.OUT) as f:
        want = json.load(f)["reference_ppm"]
    prim, cons, fbx, fby, dx, dy = ot.initial_state()
    ge = Grid2D(ot.N, ot.N, dx, dy, 1, 1, ot.GAMMA, mhd=True, recon=2, arith="exact")
    gf = Grid2D(ot.N, ot.N, dx, dy, 1, 1, ot.GAMMA, mhd=True, recon=2, arith="fast")
    try:
        st, t, c, worst = (prim, cons, fbx, fby), 0.0, 0, 0.0
        while t < ot.T_END and c < ot.MAX_CYCLES:
            ge.upload(*st)
            gf.upload(*st)
            te, ce, _ = ge.advance(t, ot.T_END, c, c + 1, ot.CFL)
            tf, cf, _ = gf.advance(t, ot.T_END, c, c + 1, ot.CFL)
            nxt = ge.download(0)
            assert cf == ce and abs(tf - te) <= 1e-12 * te
            worst = max(worst, max(field_rel_err(a, b) for a, b in zip(gf.download(0), nxt)))
            st, t, c = nxt, te, ce
        assert (t, c) == (want["t"], want["cycle"]) and ot.digest(*st) == want["sha256"]
        assert worst <= 1e-12, worst
    finally:
        ge.close()
        gf.close()
