"""CPU oracle: one 3D CTU cycle of adiabatic hydrodynamics, restated in NumPy.

TEST INFRASTRUCTURE ONLY (see ``oracle/common.py``).  Arrays have the
reference's 3D layout (nvars, ny, nx, nz): x is axis 2, y axis 1, z axis 3.

The reference's 3D step (Source/EvolveFunctions_Hydro.py:559-806) is the 2D
step with a third sweep: every reconstruction, conversion and Roe solver works
along one axis of the 4D arrays with the same arithmetic as in 2D, so this
module moves each sweep's axis last and reuses ``oracle.hydro2d`` (whose
``yaxis`` argument selects the x, y or z form of each routine).  The CTU
predictor corrects each face state with the stage-1 fluxes of its two
transverse directions, one after the other, and no constrained transport is
involved.

Boundary handling where the reference cannot run: with an outflow x boundary
its transverse-flux padding reshapes a z-flux slab to a y-flux shape
(:700-703) and raises; this oracle, like the CUDA step, pads by clamping the
cell index, as every other outflow padding of the reference does.
"""
from __future__ import annotations

import numpy as np

from . import hydro2d
from .common import SMALL_VALUE, apply_floors_inplace, wrap_index

# numpy axis of each direction in (nvars, ny, nx, nz) arrays, and the routine
# variant (``yaxis``) the reference uses along it
AXIS = {0: 2, 1: 1, 2: 3}


def calc_dt(cons, gamma, cfl, dx, dy, dz):
    """calcDt_3D_hydro (Source/TimestepCalculations_HelperModule.py:121-181)."""
    g1 = gamma - 1.0
    inv_d = 1.0 / cons[0]
    vx = cons[1] * inv_d
    vy = cons[2] * inv_d
    vz = cons[3] * inv_d
    vsq = vx * vx + vy * vy + vz * vz
    p = np.maximum(g1 * (cons[4] - 0.5 * cons[0] * vsq), SMALL_VALUE)
    a2 = gamma * p * inv_d
    a = np.sqrt(a2)
    max_x = np.max(np.abs(vx) + a)
    max_y = np.max(np.abs(vy) + a)
    max_z = np.max(np.abs(vz) + a)
    dt_x = cfl / (max_x / dx)
    dt_y = cfl / (max_y / dy)
    dt_z = cfl / (max_z / dz)
    return np.minimum(dt_x, np.minimum(dt_y, dt_z))


def edge_states(prim, d, gamma, dt, dn, bc, order):
    """Face states along direction d (0 x, 1 y, 2 z): PPM (order 2,
    Source/Reconstruction_PPM_Hydro_HelperModule.py:86-371, :387-944, :945-1227),
    PLM (order 1, no reference counterpart) or first order (order 0,
    Source/EvolveFunctions_Hydro.py:622-664).  Returns (minus-side, plus-side)
    states at the n+1 faces of the direction."""
    ax = AXIS[d]
    w = np.ascontiguousarray(np.moveaxis(prim, ax, -1))
    if order in (1, 2):
        lo, hi = hydro2d.ppm_sweep(w, gamma, dt, dn, bc, d, linear=order == 1)
    else:
        lo, hi = hydro2d.faces_from_cells(w, w, bc)
    return np.moveaxis(lo, -1, ax), np.moveaxis(hi, -1, ax)


def _transverse(u, side, d, flux, e, n_d, bc_d, half_dtde):
    """u -= half dt/de * (F_e[hi] - F_e[lo]) at the cells on ``side`` (0 minus,
    1 plus) of direction d's faces, with F_e the stage-1 flux of direction e
    (Source/EvolveFunctions_Hydro.py:694-747)."""
    ax_d, ax_e = AXIS[d], AXIS[e]
    cells = wrap_index(np.arange(n_d + 1) - 1 + side, n_d, bc_d)
    fe = np.take(flux, cells, axis=ax_d)
    n_e = fe.shape[ax_e] - 1
    hi = np.take(fe, np.arange(1, n_e + 1), axis=ax_e)
    lo = np.take(fe, np.arange(0, n_e), axis=ax_e)
    u -= half_dtde * (hi - lo)


def cycle(prim, cons, dt, dx, dy, dz, bcx, bcy, bcz, gamma, min_d, min_p, min_e, order, efix, eps):
    """One cycle of evolve_3D_hydro (Source/EvolveFunctions_Hydro.py:607-792).

    Returns new (prim, cons); the inputs are not modified.
    """
    ny, nx, nz = prim.shape[1:]
    n = (nx, ny, nz)
    dn = (dx, dy, dz)
    bc = (bcx, bcy, bcz)
    half = tuple(0.5 * (dt / h) for h in dn)
    w = {}
    for d in range(3):
        lo, hi = edge_states(prim, d, gamma, dt, dn[d], bc[d], order)
        w[d] = [apply_floors_inplace(lo, min_d, min_p), apply_floors_inplace(hi, min_d, min_p)]
    u = {d: [hydro2d.prim_to_cons(s, gamma, d) for s in w[d]] for d in range(3)}
    f1 = {d: hydro2d.roe_flux(w[d][0], w[d][1], gamma, efix, eps, d) for d in range(3)}
    # each direction's states take the flux differences of the other two, in
    # ascending direction order (x: y then z; y: x then z; z: x then y)
    for d in range(3):
        for side in (0, 1):
            for e in range(3):
                if e != d:
                    _transverse(u[d][side], side, d, f1[e], e, n[d], bc[d], half[e])
    w = {d: [hydro2d.cons_to_prim(s, gamma, d) for s in u[d]] for d in range(3)}
    f2 = {d: hydro2d.roe_flux(w[d][0], w[d][1], gamma, efix, eps, d) for d in range(3)}
    nu = cons.copy()
    for d in range(3):
        ax = AXIS[d]
        m = f2[d].shape[ax] - 1
        nu -= (dt / dn[d]) * (np.take(f2[d], np.arange(1, m + 1), axis=ax) - np.take(f2[d], np.arange(0, m), axis=ax))
    nw = hydro2d.cons_to_prim(nu, gamma, 0)
    return nw, nu


def evolve(prim, cons, dx, dy, dz, bcx, bcy, bcz, t_start, t_end, start_cycle, max_cycles,
           gamma, cfl, min_d, min_p, min_e, order=0, efix=False, eps=0.5, dt_log=None):
    """The evolve_3D_hydro loop (Source/EvolveFunctions_Hydro.py:559-806); returns the
    reference's 7-tuple."""
    prim = np.array(prim, dtype=np.float64)
    cons = np.array(cons, dtype=np.float64)
    t = t_start
    cyc = start_cycle
    sl = (prim.copy(), cons.copy(), t_start)
    while t < t_end and cyc < max_cycles:
        sl = (prim.copy(), cons.copy(), t)
        dt = calc_dt(cons, gamma, cfl, dx, dy, dz)
        if t + dt > t_end:
            dt = t_end - t
        if dt_log is not None:
            dt_log.append(dt)
        prim, cons = cycle(prim, cons, dt, dx, dy, dz, bcx, bcy, bcz, gamma, min_d, min_p, min_e,
                           order, efix, eps)
        t += dt
        cyc += 1
    return (prim, cons, t, cyc) + sl
