"""The simulation driver's time loop with the state kept on the GPU.

The reference's ``Simulation.__run_sim`` (Source/Simulation.py:290-413) calls
the evolve function once per output interval: it evolves to the next save or
plot time, saves / plots there, and -- if the run goes on -- continues from the
state before the short cycle that reached the output time (keeping that
cycle's count).  ``run`` does the same through ``mhd2d_run`` in the C ABI: the
state stays on the device for the whole run and crosses to the host only at
the stops, where ``on_stop`` gets it.  ``save_mat`` writes a stop's state in the
reference's .mat layout (Source/FileSaver.py:212-231) with the face-centred B
added, which the reference's files lack and a restart needs.
"""
from __future__ import annotations

import ctypes

from . import _lib
from .solver import Grid2D, Grid3D, default_arith

STOP_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_double, ctypes.c_longlong, ctypes.c_int)
SAVE, PLOT = 1, 2


def _decimals(x):
    """Decimal places the reference gives a time value (Source/FileSaver.py:142-145,
    :160-166): the first p >= 1 with |10^p x - int(10^p x)| <= 1e-14, at most 10."""
    p = 1
    while abs(10 ** p * x - int(10 ** p * x)) > 0.00000000000001 and p < 10:
        p += 1
    return p


def time_precision(dt, t_lim):
    """The rounding precision of an output interval: max(decimals of t_lim, decimals
    of dt) (FileSaver dataTimePrec / figTimePrec, Source/FileSaver.py:160-168)."""
    return max(_decimals(t_lim), _decimals(dt))


def run(grid, t_lim, max_cycles, cfl, save_dt=-1.0, save_prec=None, plot_dt=-1.0, plot_prec=None,
        on_stop=None):
    """Run the driver loop on an uploaded ``Grid2D`` or ``Grid3D`` (``mhd2d_run`` /
    ``mhd3d_run``).

    ``on_stop(t, cycle, kinds, grid)`` is called at t = 0 and at every save/plot
    stop (``kinds`` bit 0 save, bit 1 plot) with the stop's state on the device
    (``grid.download()`` copies it); a truthy return ends the run early.
    Returns (t, cycle, stops).
    """
    lib = _lib.load()
    if save_prec is None:
        save_prec = time_precision(save_dt, t_lim) if save_dt > 0 else 0
    if plot_prec is None:
        plot_prec = time_precision(plot_dt, t_lim) if plot_dt > 0 else 0
    err = []

    def cb(_user, t, cycle, kinds):
        if on_stop is None:
            return 0
        try:
            return 1 if on_stop(float(t), int(cycle), int(kinds), grid) else 0
        except Exception as e:  # keep the exception for the caller; stop the run
            err.append(e)
            return 1

    fn = STOP_FN(cb)
    t = ctypes.c_double()
    c = ctypes.c_longlong()
    n = ctypes.c_longlong()
    three_d = isinstance(grid, Grid3D)
    entry = lib.mhd3d_run if three_d else lib.mhd2d_run
    rc = entry(grid._h if three_d else grid.handle, float(t_lim), int(max_cycles), float(cfl), float(save_dt),
               int(save_prec), float(plot_dt), int(plot_prec), fn, None, ctypes.byref(t), ctypes.byref(c),
               ctypes.byref(n))
    if err:
        raise err[0]
    _lib.check(rc, "mhd3d_run" if three_d else "mhd2d_run")
    return t.value, c.value, n.value


# the reference's variable names (Source/PythonMHD_Constants.py:86-104), the keys
# of its .mat files (Source/FileSaver.py:212-231)
MAT_KEYS_MHD = ("Density", "Vx", "Vy", "Vz", "Bx", "By", "Bz", "Pressure")
MAT_KEYS_HYDRO = ("Density", "Vx", "Vy", "Vz", "Pressure")


def save_mat(path, prim, cons, fbx=None, fby=None, fbz=None):
    """A stop's state in the reference's .mat layout (the primitive variables and the
    energy under the reference's keys), plus faceBx/faceBy (and faceBz for a 3D grid)
    for MHD, which a restart needs."""
    import scipy.io
    if prim.shape[0] == 8:
        d = dict(zip(MAT_KEYS_MHD, prim))
        d.update({"Energy": cons[7], "faceBx": fbx, "faceBy": fby})
        if fbz is not None:
            d["faceBz"] = fbz
    else:
        d = dict(zip(MAT_KEYS_HYDRO, prim))
        d["Energy"] = cons[4]
    scipy.io.savemat(path, d)


def simulate(prim, cons, fbx, fby, dx, dy, bcx, bcy, t_lim, max_cycles, gamma, cfl, min_d=1e-12, min_p=1e-12,
             min_e=1e-12, recon=2, entropy_fix=False, eps=0.5, save_dt=-1.0, plot_dt=-1.0, on_stop=None,
             arith=None):
    """Convenience wrapper: create the handle, upload, run the driver loop, download.

    Returns (t, cycle, stops, (prim, cons, faceBx, faceBy)) with the final state.
    """
    mhd = prim.shape[0] == 8
    ny, nx = prim.shape[1:]
    g = Grid2D(ny, nx, dx, dy, bcx, bcy, gamma, mhd=mhd, recon=recon, entropy_fix=entropy_fix, eps=eps,
               min_d=min_d, min_p=min_p, min_e=min_e, arith=arith or default_arith())
    try:
        g.upload(prim, cons, fbx, fby)
        t, c, n = run(g, t_lim, max_cycles, cfl, save_dt=save_dt, plot_dt=plot_dt, on_stop=on_stop)
        return t, c, n, g.download()
    finally:
        g.close()
