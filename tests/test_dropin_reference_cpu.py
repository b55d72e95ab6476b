"""The drop-in under the reference's own driver: ``dropin.install()`` into the real
``Source`` package, then the reference's unmodified ``Simulation(...).run()``
(Source/Simulation.py:277-434) picks the installed functions at
Source/Simulation.py:312-324 and calls them at :349-377.

The reference checkout is needed (``PYTHONMHD_REFERENCE`` names it; the test is
skipped without it).  This test runs on the CPU, so the device handle inside the
drop-in (``pythonmhd_gb300.evolve.Grid2D``) is replaced by a stand-in that keeps
its interface -- upload, advance, download with the second-last state,
last_cycles -- and computes with the oracle.  Everything else is the product's
host layer: argument checks, handle caching, the in-place updates of faceBx /
faceBy (MHD) and primVars / consVars (hydro), the no-cycle path and the return
tuples.  The run must reproduce the reference driver's recorded stops and final
state bit for bit (tests/golden/driver_digests.json).  The same drop-in with the
real device handle is checked on the GPU in tests/test_gpu_driver.py.
"""
import os
import sys
import tempfile
from unittest import mock

import numpy as np
import pytest

from oracle import hydro2d, mhd2d
from tests.golden import make_driver_digests as mdd
from tests.test_oracle_golden import _driver_digests

REF = os.environ.get("PYTHONMHD_REFERENCE")
pytestmark = pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF or "", "Source")),
                                reason="PYTHONMHD_REFERENCE does not name a PythonMHD checkout")


class OracleHandle:
    """Grid2D's interface, computed by the oracle (for this CPU test only)."""

    calls = 0

    def __init__(self, ny, nx, dx, dy, bcx, bcy, gamma, mhd=True, recon=2, entropy_fix=False, eps=0.5,
                 min_d=1e-12, min_p=1e-12, min_e=1e-12, arith=None):
        self.p = (dx, dy, bcx, bcy)
        self.q = (gamma, None, min_d, min_p, min_e, recon, entropy_fix, eps)
        self.mhd = mhd
        self.last_cycles = 0

    def upload(self, prim, cons, fbx=None, fby=None):
        self.state = tuple(np.array(a) for a in ((prim, cons, fbx, fby) if self.mhd else (prim, cons)))

    def advance(self, t0, t_end, cycle0, max_cycles, cfl):
        OracleHandle.calls += 1
        g, _, d, p, e, r, ef, eps = self.q
        if self.mhd:
            res = mhd2d.evolve(*self.state, *self.p, t0, t_end, cycle0, max_cycles, g, cfl, d, p, e, r, ef, eps)
            self.cur, t, cyc, self.sl, t_sl = res[:4], res[4], res[5], res[6:10], res[10]
        else:
            res = hydro2d.evolve(*self.state, *self.p, t0, t_end, cycle0, max_cycles, g, cfl, d, p, e, r, ef, eps)
            self.cur, t, cyc, self.sl, t_sl = res[:2], res[2], res[3], res[4:6], res[6]
        self.last_cycles = cyc - cycle0
        return t, cyc, t_sl

    def download(self, which=0):
        return tuple(np.array(a) for a in (self.cur if which == 0 else self.sl))

    def close(self):
        pass


@pytest.mark.parametrize("case", sorted(_driver_digests()))
def test_reference_simulation_runs_the_installed_dropin(case, monkeypatch, tmp_path):
    for m in mdd.STUBS:
        monkeypatch.setitem(sys.modules, m, mock.MagicMock())
    monkeypatch.syspath_prepend(REF)
    monkeypatch.setattr(sys, "dont_write_bytecode", True)
    import Source.EvolveFunctions_Hydro as ref_hydro
    import Source.EvolveFunctions_MHD as ref_mhd
    import Source.PythonMHD_Constants as C
    import Source.Simulation as S

    from pythonmhd_gb300 import dropin, evolve
    monkeypatch.setattr(evolve, "Grid2D", OracleHandle)
    evolve.clear_cache()
    dropin.install()
    try:
        assert ref_mhd.evolve_2D_mhd is evolve.evolve_2D_mhd
        assert ref_hydro.evolve_2D_hydro is evolve.evolve_2D_hydro
        assert S.evolveMHD is ref_mhd and S.evolveHydro is ref_hydro
        OracleHandle.calls = 0
        with tempfile.TemporaryDirectory(dir=tmp_path) as tmp:
            got = mdd.run_reference(case, S, C, tmp)
        assert OracleHandle.calls > 0           # the driver called the installed function
    finally:
        dropin.uninstall()
        evolve.clear_cache()
    want = _driver_digests()[case]
    assert got["initial_sha256"] == want["initial_sha256"]
    assert got["stops"] == want["stops"]
    assert got["final"] == want["final"]
