"""The device-resident driver loop (mhd2d_run through pythonmhd_gb300.driver)
against the oracle's restatement of the reference driver (Source/Simulation.py:
290-413): the same stops (time, cycle, kind), the same states at every stop and
at the end, bit for bit in exact arithmetic."""
import numpy as np
import pytest

from oracle import driver as odriver
from pythonmhd_gb300 import driver
from pythonmhd_gb300 import initial_conditions as ic
from pythonmhd_gb300.solver import Grid2D

pytestmark = pytest.mark.gpu


def _mhd_case():
    prim, cons, fbx, fby, dx, dy = ic.orszag_tang(32, 28, gamma=5.0 / 3.0)
    return dict(prim=prim, cons=cons, fbx=fbx, fby=fby, dx=dx, dy=dy, bcx=1, bcy=1, gamma=5.0 / 3.0)


def _hydro_case():
    prim = np.zeros((5, 24, 30))
    prim[0] = 1.0
    prim[4] = 0.1
    prim[4, 10:14, 13:17] = 10.0
    return dict(prim=prim, cons=ic.prim_to_cons_hydro(prim, 1.4), fbx=None, fby=None, dx=1 / 30, dy=1 / 24,
                bcx=0, bcy=0, gamma=1.4)


@pytest.mark.parametrize("physics,t_lim,max_cycles,save_dt,plot_dt,order", [
    ("mhd", 0.05, 1000, 0.01, -1.0, 2),
    ("mhd", 0.04, 1000, 0.01, 0.015, 1),
    ("mhd", 0.05, 9, 0.01, -1.0, 2),
    ("hydro", 0.03, 1000, 0.005, 0.0075, 2),
    ("hydro", 0.02, 1000, -1.0, -1.0, 0),
])
def test_driver_matches_oracle_driver(physics, t_lim, max_cycles, save_dt, plot_dt, order):
    c = _mhd_case() if physics == "mhd" else _hydro_case()
    mhd = physics == "mhd"
    sp = driver.time_precision(save_dt, t_lim) if save_dt > 0 else 0
    pp = driver.time_precision(plot_dt, t_lim) if plot_dt > 0 else 0
    args = (c["dx"], c["dy"], c["bcx"], c["bcy"], t_lim, max_cycles, c["gamma"], 0.4, 1e-12, 1e-12, 1e-12, order,
            False, 0.5)
    t_w, cyc_w, stops_w, final_w = odriver.run(c["prim"], c["cons"], c["fbx"], c["fby"], *args,
                                               save_dt=save_dt, save_prec=sp, plot_dt=plot_dt, plot_prec=pp)
    got = []

    def on_stop(t, cycle, kinds, grid):
        got.append((t, cycle, kinds, grid.download()))

    ny, nx = c["prim"].shape[1:]
    g = Grid2D(ny, nx, c["dx"], c["dy"], c["bcx"], c["bcy"], c["gamma"], mhd=mhd, recon=order, arith="exact")
    g.upload(c["prim"], c["cons"], c["fbx"], c["fby"])
    t, cyc, n = driver.run(g, t_lim, max_cycles, 0.4, save_dt=save_dt, plot_dt=plot_dt, on_stop=on_stop)
    final = g.download()
    g.close()
    assert (t, cyc) == (t_w, cyc_w)
    assert len(got) == len(stops_w) and n == len([s for s in stops_w if s[0] > 0.0 or s[1] > 0])
    for (tg, cg, kg, sg), (tw, cw, kw, sw) in zip(got, stops_w):
        assert (tg, cg, kg) == (tw, cw, kw)
        for a, b in zip(sg, sw):
            if b is not None:
                np.testing.assert_array_equal(a, b)
    for a, b in zip(final, final_w):
        if b is not None:
            np.testing.assert_array_equal(a, b)


def test_driver_stop_callback_can_end_the_run(tmp_path):
    c = _mhd_case()
    g = Grid2D(28, 32, c["dx"], c["dy"], 1, 1, c["gamma"], mhd=True, recon=2, arith="exact")
    g.upload(c["prim"], c["cons"], c["fbx"], c["fby"])
    seen = []

    def on_stop(t, cycle, kinds, grid):
        p, u, bx, by = grid.download()
        driver.save_mat(str(tmp_path / f"snap_{len(seen)}.mat"), p, u, bx, by)
        seen.append(t)
        return len(seen) == 3

    with pytest.raises(Exception) as e:
        driver.run(g, 0.05, 1000, 0.4, save_dt=0.01, on_stop=on_stop)
    assert "stop callback" in str(e.value)
    g.close()
    assert seen[0] == 0.0 and len(seen) == 3
    import scipy.io
    d = scipy.io.loadmat(str(tmp_path / "snap_0.mat"))
    np.testing.assert_array_equal(d["faceBx"], c["fbx"])
    np.testing.assert_array_equal(d["Density"], c["prim"][0])


@pytest.mark.parametrize("t_lim,save_dt,plot_dt,order", [(0.03, 0.01, 0.0075, 2), (0.02, -1.0, 0.005, 0)])
def test_3d_driver_matches_oracle_driver(t_lim, save_dt, plot_dt, order):
    """mhd3d_run on a 3D hydro blast against the oracle's driver around its 3D step."""
    from pythonmhd_gb300.solver import Grid3D
    ny, nx, nz = 10, 12, 8
    prim = np.zeros((5, ny, nx, nz))
    prim[0] = 1.0
    prim[4] = 0.1
    prim[4, 4:6, 5:7, 3:5] = 10.0
    cons = ic.prim_to_cons_hydro(prim, 1.4)
    sp = driver.time_precision(save_dt, t_lim) if save_dt > 0 else 0
    pp = driver.time_precision(plot_dt, t_lim) if plot_dt > 0 else 0
    args = (1 / nx, 1 / ny, 1 / nz, 1, 0, 1, t_lim, 1000, 1.4, 0.4, 1e-12, 1e-12, 1e-12, order, False, 0.5)
    t_w, cyc_w, stops_w, final_w = odriver.run3d(prim, cons, *args, save_dt=save_dt, save_prec=sp,
                                                 plot_dt=plot_dt, plot_prec=pp)
    got = []
    g = Grid3D(ny, nx, nz, 1 / nx, 1 / ny, 1 / nz, 1, 0, 1, 1.4, recon=order, arith="exact")
    g.upload(prim, cons)
    t, cyc, n = driver.run(g, t_lim, 1000, 0.4, save_dt=save_dt, plot_dt=plot_dt,
                           on_stop=lambda t, c, k, grid: got.append((t, c, k, grid.download())))
    final = g.download()
    g.close()
    assert (t, cyc) == (t_w, cyc_w) and cyc > 5
    assert len(got) == len(stops_w) and n == len(stops_w) - 1
    for (tg, cg, kg, sg), (tw, cw, kw, sw) in zip(got, stops_w):
        assert (tg, cg, kg) == (tw, cw, kw)
        for a, b in zip(sg, sw):
            assert np.array_equal(a, b)
    for a, b in zip(final, final_w):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("t_lim,save_dt,plot_dt,order", [(0.04, 0.01, 0.0075, 2), (0.03, -1.0, 0.005, 1)])
def test_3d_mhd_driver_matches_oracle_driver(t_lim, save_dt, plot_dt, order):
    """mhd3d_run on a 3D MHD grid against the oracle's driver around its 3D MHD step
    (FP64 predictor, as the CUDA step computes it)."""
    from pythonmhd_gb300.solver import Grid3D
    from tests.golden import cases
    ny, nx, nz = 8, 10, 6
    prim, cons, fbx, fby, fbz, dx, dy, dz = cases._random_mhd_3d(ny, nx, nz, seed=7)
    sp = driver.time_precision(save_dt, t_lim) if save_dt > 0 else 0
    pp = driver.time_precision(plot_dt, t_lim) if plot_dt > 0 else 0
    args = (dx, dy, dz, 1, 0, 1, t_lim, 1000, 5.0 / 3.0, 0.4, 1e-12, 1e-12, 1e-12, order, True, 0.5)
    t_w, cyc_w, stops_w, final_w = odriver.run3d_mhd(prim, cons, fbx, fby, fbz, *args, save_dt=save_dt,
                                                     save_prec=sp, plot_dt=plot_dt, plot_prec=pp,
                                                     long_double=False)
    got = []
    g = Grid3D(ny, nx, nz, dx, dy, dz, 1, 0, 1, 5.0 / 3.0, recon=order, entropy_fix=True, arith="exact", mhd=True)
    g.upload(prim, cons, fbx, fby, fbz)
    t, cyc, n = driver.run(g, t_lim, 1000, 0.4, save_dt=save_dt, plot_dt=plot_dt,
                           on_stop=lambda t, c, k, grid: got.append((t, c, k, grid.download())))
    final = g.download()
    g.close()
    assert (t, cyc) == (t_w, cyc_w) and cyc > 3
    assert len(got) == len(stops_w) and n == len(stops_w) - 1
    for (tg, cg, kg, sg), (tw, cw, kw, sw) in zip(got, stops_w):
        assert (tg, cg, kg) == (tw, cw, kw)
        for a, b in zip(sg, sw):
            assert np.array_equal(a, b)
    for a, b in zip(final, final_w):
        assert np.array_equal(a, b)


def _driver_cases():
    from tests.test_oracle_golden import _driver_digests
    return sorted(_driver_digests())


@pytest.mark.parametrize("case", _driver_cases())
def test_device_driver_matches_the_reference_driver(case):
    """mhd2d_run against the reference's own Simulation.run() (digests recorded by
    tests/golden/make_driver_digests.py): every stop's time, cycle, kind and state and the
    final state, bit for bit."""
    from tests.test_oracle_golden import run_driver_case

    def run(state, w, sp, pp):
        mhd = len(state) == 4
        ny, nx = state[0].shape[1:]
        g = Grid2D(ny, nx, w["dx"], w["dy"], w["bcx"], w["bcy"], w["gamma"], mhd=mhd,
                   recon=2 if w["order"] == 2 else 0, arith="exact")
        got = []
        try:
            g.upload(*state)
            t, cyc, _ = driver.run(g, w["t_lim"], w["max_cycles"], w["cfl"], save_dt=w["save_dt"], save_prec=sp,
                                   plot_dt=w["plot_dt"], plot_prec=pp,
                                   on_stop=lambda t, c, k, grid: got.append((t, c, k, grid.download())))
            return t, cyc, got, g.download()
        finally:
            g.close()

    run_driver_case(case, run)


@pytest.mark.parametrize("case", _driver_cases())
def test_dropin_evolve_under_the_driver_loop_matches_the_reference_driver(case):
    """The drop-in evolve functions (evolve_2D_mhd / evolve_2D_hydro on the GPU), called by
    the driver loop as Source/Simulation.py:345-413 calls them (the oracle's restatement
    of that loop, itself pinned to the reference's runs), reproduce the reference's stops."""
    from types import SimpleNamespace

    from pythonmhd_gb300 import evolve
    from tests.test_oracle_golden import run_driver_case

    def run(state, w, sp, pp):
        mhd = len(state) == 4
        ny, nx = state[0].shape[1:]

        def step(st, t0, t_end, cyc0):
            g = SimpleNamespace(primVars=st[0], consVars=st[1], dx=w["dx"], dy=w["dy"], BcX=w["bcx"], BcY=w["bcy"],
                                numXCells=nx, numYCells=ny)
            if mhd:
                g.faceBx, g.faceBy = st[2], st[3]
                r = evolve.evolve_2D_mhd(g, t0, t_end, cyc0, w["max_cycles"], w["gamma"], w["cfl"], 1e-12, 1e-12,
                                         1e-12, w["order"], False, 0.5, arith="exact")
                return tuple(np.copy(a) for a in r[:4]), r[4], r[5], tuple(r[6:10]), r[10]
            r = evolve.evolve_2D_hydro(g, t0, t_end, cyc0, w["max_cycles"], w["gamma"], w["cfl"], 1e-12, 1e-12,
                                       1e-12, w["order"], False, 0.5, arith="exact")
            return tuple(np.copy(a) for a in r[:2]), r[2], r[3], tuple(r[4:6]), r[6]

        return odriver._drive(tuple(a.copy() for a in state), step, w["t_lim"], w["max_cycles"], w["save_dt"], sp,
                              w["plot_dt"], pp)

    run_driver_case(case, run)
