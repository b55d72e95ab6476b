"""Failure detection without a GPU fault: a NaN planted in the host input reaches the
CFL reduction (a NaN signal speed wins the maximum), the timestep becomes NaN, and
the advance call returns MHD_ERR_NONFINITE, which the Python mirror raises as
MhdError.  The context stays usable: the same process then runs a clean grid."""
import numpy as np
import pytest

from pythonmhd_gb300 import _lib
from pythonmhd_gb300 import initial_conditions as ic
from pythonmhd_gb300.solver import Grid2D

pytestmark = pytest.mark.gpu
NONFINITE = 5


@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_nan_in_the_input_is_reported(arith):
    prim, cons, fbx, fby, dx, dy = ic.orszag_tang(32, 32)
    bad_p, bad_c = prim.copy(), cons.copy()
    bad_p[0, 5, 7] = np.nan
    bad_c[0, 5, 7] = np.nan
    g = Grid2D(32, 32, dx, dy, 1, 1, 5.0 / 3.0, mhd=True, recon=2, arith=arith)
    try:
        g.upload(bad_p, bad_c, fbx, fby)
        with pytest.raises(_lib.MhdError) as e:
            g.advance(0.0, 1e30, 0, 5, 0.4)
        assert e.value.status == NONFINITE
        # the handle and the context still work: a clean state advances
        g.upload(prim, cons, fbx, fby)
        t, c, _ = g.advance(0.0, 1e30, 0, 3, 0.4)
        assert c == 3 and np.isfinite(t)
    finally:
        g.close()


def test_nan_in_one_batched_instance_stops_only_that_instance():
    from pythonmhd_gb300.solver import Batch2D
    insts = ic.orszag_tang_batch(count=4, seed=5, sizes=(16, 24, 32))
    bad = 2
    b = Batch2D(insts, mhd=True, recon=1, arith="exact")
    try:
        for k, inst in enumerate(insts):
            p, c = inst["prim"].copy(), inst["cons"].copy()
            if k == bad:
                p[7, 3, 4] = np.nan
                c[7, 3, 4] = np.nan
            b.upload(k, p, c, inst["fbx"], inst["fby"])
        with pytest.raises(_lib.MhdError) as e:
            b.advance(0.0, 1.0, 0, 5, 0.4)
        assert e.value.status == NONFINITE
        assert list(e.value.instance_status) == [NONFINITE if k == bad else 0 for k in range(4)]
        assert np.isnan(e.value.t_out[bad])
        for k, inst in enumerate(insts):
            if k == bad:
                continue
            # the healthy instances ran all their cycles and match a single-grid run bit for bit
            assert e.value.cycle_out[k] == 5
            g = Grid2D(inst["ny"], inst["nx"], inst["dx"], inst["dy"], 1, 1, inst["gamma"], mhd=True, recon=1,
                       arith="exact")
            g.upload(inst["prim"], inst["cons"], inst["fbx"], inst["fby"])
            t, c, _ = g.advance(0.0, 1.0, 0, 5, 0.4)
            want = g.download(0)
            g.close()
            assert t == e.value.t_out[k]
            for a, w in zip(b.download(k), want):
                assert np.array_equal(a, w)
    finally:
        b.close()
