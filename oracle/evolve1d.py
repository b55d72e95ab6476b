"""CPU restatement of the reference's 1D evolve functions (test infrastructure only).

* evolve_mhd  -- evolve_1D_mhd   (Source/EvolveFunctions_MHD.py:195-340)
* evolve_hydro -- evolve_1D_hydro (Source/EvolveFunctions_Hydro.py:232-305)

A 1D cycle is the x sweep of the 2D step without the transverse (CTU) and CT
stages: reconstruction (PPM for reconstructOrder == 2, cell values otherwise),
floors on the face states, prim -> cons, the Roe flux, and the conservative
update cons -= dt/dx (F_right - F_left).  MHD keeps B_x uniform at the first
cell's value (Source/EvolveFunctions_MHD.py:201-205) and has no B source terms.
The x-sweep pieces are the oracle's 2D ones on (nvars, 1, N) arrays.
"""
from __future__ import annotations

import numpy as np

from . import hydro2d, mhd2d
from .common import FRAME_X, SMALL_VALUE, apply_floors_inplace


def calc_dt_mhd(cons, gamma, cfl, dx):
    """calcDt_1D_mhd (Source/TimestepCalculations_HelperModule.py:183-225)."""
    g1 = gamma - 1.0
    inv_d = 1.0 / cons[0]
    vx = cons[1] * inv_d
    vy = cons[2] * inv_d
    vz = cons[3] * inv_d
    vsq = vx * vx + vy * vy + vz * vz
    bx, by, bz = cons[4], cons[5], cons[6]
    bsq = bx * bx + by * by + bz * bz
    p = np.maximum(g1 * (cons[7] - 0.5 * cons[0] * vsq - 0.5 * bsq), SMALL_VALUE)
    a2 = gamma * p * inv_d
    ssum = bsq * inv_d + a2
    sdiff = bsq * inv_d - a2
    cf2 = 0.5 * (ssum + np.sqrt(sdiff * sdiff + 4.0 * a2 * (by * by + bz * bz) * inv_d))
    max_x = np.max(np.abs(vx) + np.sqrt(cf2))
    return cfl / (max_x / dx)


def calc_dt_hydro(cons, gamma, cfl, dx):
    """calcDt_1D_hydro (Source/TimestepCalculations_HelperModule.py:24-56)."""
    g1 = gamma - 1.0
    inv_d = 1.0 / cons[0]
    vx = cons[1] * inv_d
    vy = cons[2] * inv_d
    vz = cons[3] * inv_d
    vsq = vx * vx + vy * vy + vz * vz
    p = np.maximum(g1 * (cons[4] - 0.5 * cons[0] * vsq), SMALL_VALUE)
    a2 = gamma * p * inv_d
    max_x = np.max(np.abs(vx) + np.sqrt(a2))
    return cfl / (max_x / dx)


def _first_order(w, bc):
    return hydro2d.faces_from_cells(w, w, bc)


def cycle_mhd(prim, cons, bx, dt, dx, bcx, gamma, min_d, min_p, min_e, order, efix, eps):
    """One cycle; returns new (prim8, cons8)."""
    n = prim.shape[1]
    bx_cell = np.full(n, bx)
    fbx = np.full((1, n + 1), bx)
    wx = np.array([prim[0], prim[1], prim[2], prim[3], prim[5], prim[6], prim[7]])[:, None, :]
    ux = np.array([cons[0], cons[1], cons[2], cons[3], cons[5], cons[6], cons[7]])[:, None, :]
    if order == 2:
        xl, xr = mhd2d.ppm_sweep(wx, bx_cell[None, :], gamma, dt, dx, bcx, FRAME_X)
    else:
        xl, xr = _first_order(wx, bcx)
    xl, xr = xl.copy(), xr.copy()
    apply_floors_inplace(xl, min_d, min_p)
    apply_floors_inplace(xr, min_d, min_p)
    uxl = mhd2d.prim_to_cons7(xl, fbx, gamma)
    uxr = mhd2d.prim_to_cons7(xr, fbx, gamma)
    f = mhd2d.roe_flux(xl, xr, uxl, uxr, fbx, gamma, efix, eps, FRAME_X)
    ux = ux - (dt / dx) * (f[..., 1:] - f[..., :-1])
    wx = mhd2d.cons_to_prim7(ux, bx_cell[None, :], gamma)
    w, u = wx[:, 0], ux[:, 0]
    new_prim = np.array([w[0], w[1], w[2], w[3], bx_cell, w[4], w[5], w[6]])
    new_cons = np.array([u[0], u[1], u[2], u[3], bx_cell, u[4], u[5], u[6]])
    return new_prim, new_cons


def cycle_hydro(prim, cons, dt, dx, bcx, gamma, min_d, min_p, min_e, order, efix, eps):
    w = prim[:, None, :]
    if order == 2:
        xl, xr = hydro2d.ppm_sweep(w, gamma, dt, dx, bcx, False)
    else:
        xl, xr = _first_order(w, bcx)
    xl, xr = xl.copy(), xr.copy()
    apply_floors_inplace(xl, min_d, min_p)
    apply_floors_inplace(xr, min_d, min_p)
    f = hydro2d.roe_flux(xl, xr, gamma, efix, eps, False)
    u = cons[:, None, :] - (dt / dx) * (f[..., 1:] - f[..., :-1])
    w = hydro2d.cons_to_prim(u, gamma, False)
    return w[:, 0], u[:, 0]


def evolve_mhd(prim, cons, dx, bcx, t_start, t_end, start_cycle, max_cycles, gamma, cfl, min_d, min_p, min_e,
               order=0, efix=False, eps=0.5):
    """The evolve_1D_mhd loop; returns the reference's 7-tuple."""
    prim = np.array(prim, dtype=np.float64)
    cons = np.array(cons, dtype=np.float64)
    bx = prim[4][0]
    t, cyc = t_start, start_cycle
    sl = (prim.copy(), cons.copy(), t_start)
    while t < t_end and cyc < max_cycles:
        sl = (prim.copy(), cons.copy(), t)
        dt = calc_dt_mhd(cons, gamma, cfl, dx)
        if t + dt > t_end:
            dt = t_end - t
        prim, cons = cycle_mhd(prim, cons, bx, dt, dx, bcx, gamma, min_d, min_p, min_e, order, efix, eps)
        t += dt
        cyc += 1
    return (prim, cons, t, cyc) + sl


def evolve_hydro(prim, cons, dx, bcx, t_start, t_end, start_cycle, max_cycles, gamma, cfl, min_d, min_p, min_e,
                 order=0, efix=False, eps=0.5):
    """The evolve_1D_hydro loop; returns the reference's 7-tuple."""
    prim = np.array(prim, dtype=np.float64)
    cons = np.array(cons, dtype=np.float64)
    t, cyc = t_start, start_cycle
    sl = (prim.copy(), cons.copy(), t_start)
    while t < t_end and cyc < max_cycles:
        sl = (prim.copy(), cons.copy(), t)
        dt = calc_dt_hydro(cons, gamma, cfl, dx)
        if t + dt > t_end:
            dt = t_end - t
        prim, cons = cycle_hydro(prim, cons, dt, dx, bcx, gamma, min_d, min_p, min_e, order, efix, eps)
        t += dt
        cyc += 1
    return (prim, cons, t, cyc) + sl
