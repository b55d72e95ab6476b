"""CPU oracle: one 2D CTU cycle of adiabatic hydrodynamics, restated in NumPy.

TEST INFRASTRUCTURE ONLY (see ``oracle/common.py``). State vectors are
[rho, vx, vy, vz, p] / [rho, mx, my, mz, E] in every sweep; the y- and
z-direction routines differ from the x ones in the order of a few sums and in
the order of their waves, which is kept here through the ``yaxis`` argument:
False / 0 is x, True / 1 is y and 2 is z (the z forms serve ``oracle/hydro3d.py``).
"""
from __future__ import annotations

import numpy as np

from .common import (FOUR_THIRDS, OUTFLOW, SMALL_VALUE, apply_floors_inplace,
                     take_x, take_y, wrap_index)


def prim_to_cons(w, gamma, yaxis=False):
    """primToCons_hydro_x / _y / _z (Source/PrimCons_HelperModule.py:46-114)."""
    u = np.empty_like(w)
    u[0] = w[0]
    u[1] = w[0] * w[1]
    u[2] = w[0] * w[2]
    u[3] = w[0] * w[3]
    if yaxis == 2:
        ke = np.square(w[3]) + np.square(w[1]) + np.square(w[2])
    elif yaxis:
        ke = np.square(w[2]) + np.square(w[3]) + np.square(w[1])
    else:
        ke = np.square(w[1]) + np.square(w[2]) + np.square(w[3])
    u[4] = (w[4] / (gamma - 1.0)) + 0.5 * w[0] * ke
    return u


def cons_to_prim(u, gamma, yaxis=False):
    """consToPrim_hydro_x / _y / _z (Source/PrimCons_HelperModule.py:135-196)."""
    w = np.empty_like(u)
    w[0] = u[0]
    inv_d = 1.0 / w[0]
    w[1] = u[1] * inv_d
    w[2] = u[2] * inv_d
    w[3] = u[3] * inv_d
    if yaxis == 2:
        m2 = np.square(u[3]) + np.square(u[1]) + np.square(u[2])
    elif yaxis:
        m2 = np.square(u[2]) + np.square(u[3]) + np.square(u[1])
    else:
        m2 = np.square(u[1]) + np.square(u[2]) + np.square(u[3])
    w[4] = u[4] - 0.5 * m2 * inv_d
    w[4] *= (gamma - 1.0)
    return w


def calc_dt(cons, gamma, cfl, dx, dy):
    """calcDt_2D_hydro (Source/TimestepCalculations_HelperModule.py:67-109)."""
    g1 = gamma - 1.0
    inv_d = 1.0 / cons[0]
    vx = cons[1] * inv_d
    vy = cons[2] * inv_d
    vz = cons[3] * inv_d
    vsq = vx * vx + vy * vy + vz * vz
    p = np.maximum(g1 * (cons[4] - 0.5 * cons[0] * vsq), SMALL_VALUE)
    a2 = gamma * p * inv_d
    max_x = np.max(np.abs(vx) + np.sqrt(a2))
    max_y = np.max(np.abs(vy) + np.sqrt(a2))
    dt_x = cfl / (max_x / dx)
    dt_y = cfl / (max_y / dy)
    return np.minimum(dt_x, dt_y)


def prim_eigensystem(w, gamma, yaxis=False):
    """getEigenmatricesX/Y/Z_hydro (Source/ReconstructionEigenmatrices_Hydro_HelperModule.py:25-151, :230-282).

    Wave order: x = (acoustic-, entropy, vy, vz, acoustic+),
                y = (acoustic-, vx, entropy, vz, acoustic+),
                z = (acoustic-, vx, vy, entropy, acoustic+).
    """
    n = 3 if yaxis == 2 else (2 if yaxis else 1)
    ent = n                       # the entropy wave sits at the normal velocity's index
    a2 = gamma * w[4] / w[0]
    a = np.sqrt(a2)
    vn = w[n]
    lam = [vn - a, vn, vn, vn, vn + a]
    R = {}
    R[0, 0] = np.ones_like(a)
    R[n, 0] = -a / w[0]
    R[4, 0] = a2
    R[0, ent] = np.ones_like(a)
    for k in (1, 2, 3):           # shear waves: wave k carries velocity slot k
        if k != ent:
            R[k, k] = np.ones_like(a)
    R[0, 4] = np.ones_like(a)
    R[n, 4] = -R[n, 0]
    R[4, 4] = a2
    L = {}
    L[0, n] = -0.5 * w[0] / a
    L[0, 4] = 0.5 / a2
    L[ent, 0] = np.ones_like(a)
    L[ent, 4] = -1.0 / a2
    for k in (1, 2, 3):
        if k != ent:
            L[k, k] = np.ones_like(a)
    L[4, n] = -L[0, n]
    L[4, 4] = L[0, 4]
    return lam, L, R


def _project(L, i, vec):
    acc = np.zeros_like(vec[0])
    for j in range(5):
        e = L.get((i, j))
        if e is not None:
            acc = acc + e * vec[j]
    return acc


def ppm_sweep(w, gamma, dt, dn, bc, yaxis, linear=False):
    """ppmReconstructX/Y_hydro (Source/Reconstruction_PPM_Hydro_HelperModule.py:86-371, :387-620)
    along the last axis of ``w`` (5, M, N); ``linear=True`` gives the PLM variant
    (no reference counterpart, see ``oracle.mhd2d.plm_edges``)."""
    N = w.shape[-1]
    g = wrap_index(np.arange(-2, N + 2), N, bc)
    we = take_x(w, g)
    wc = we[..., 1:-1]
    wl = we[..., :-2]
    wr = we[..., 2:]
    lam, L, R = prim_eigensystem(wc, gamma, yaxis)
    d_c = wr - wl
    d_l = wc - wl
    d_r = wr - wc
    weight = np.zeros_like(wc)
    wi = d_l * d_r > 0.0
    weight[wi] = (2.0 * d_l * d_r)[wi] / (d_l + d_r)[wi]
    sc = np.zeros_like(wc)
    for i in range(5):
        cc = _project(L, i, d_c)
        cl = _project(L, i, d_l)
        cr = _project(L, i, d_r)
        cw = _project(L, i, weight)
        ok = cl * cr > 0.0
        lim1 = np.minimum(np.abs(cl), np.abs(cr))
        lim2 = np.minimum(0.5 * np.abs(cc), np.abs(cw))
        s = np.sign(cc) * np.minimum(2.0 * lim1, lim2)
        sc[i][ok] = s[ok]
    slopes = np.zeros_like(wc)
    for i in range(5):
        acc = np.zeros_like(wc[0])
        for j in range(5):
            e = R.get((i, j))
            if e is not None:
                acc = acc + sc[j] * e
        slopes[i] = acc
    s_c = slopes[..., 1:-1]
    s_l = slopes[..., :-2]
    s_r = slopes[..., 2:]
    wc = wc[..., 1:-1]
    wl = wl[..., 1:-1]
    wr = wr[..., 1:-1]
    if linear:
        from .mhd2d import plm_edges
        lam = [x[..., 1:-1] for x in lam]
        L = {k: v[..., 1:-1] for k, v in L.items()}
        R = {k: v[..., 1:-1] for k, v in R.items()}
        lia, ria = plm_edges(wc, wl, wr, s_c, lam, L, R, dt / dn, tuple(range(5)), 5)
        return faces_from_cells(lia, ria, bc)
    lia = 0.5 * (wc + wl) - (s_c - s_l) / 6.0
    ria = 0.5 * (wr + wc) - (s_r - s_c) / 6.0
    dprod = (ria - wc) * (wc - lia)
    idiff = ria - lia
    idiff2 = np.square(idiff)
    adiff = 6.0 * (wc - 0.5 * (lia + ria))
    nz = dprod <= 0.0
    pz = ~nz
    lia[nz] = wc[nz]
    ria[nz] = wc[nz]
    cl_ = np.logical_and(pz, (idiff * adiff) > idiff2)
    lia[cl_] = ((6.0 * wc - 4.0 * ria) / 2.0)[cl_]
    cr_ = np.logical_and(pz, np.logical_and(~cl_, (idiff * adiff) < (-1.0 * idiff2)))
    ria[cr_] = ((6.0 * wc - 4.0 * lia) / 2.0)[cr_]
    lia = np.maximum(np.minimum(wc, wl), lia)
    lia = np.minimum(np.maximum(wc, wl), lia)
    ria = np.maximum(np.minimum(wc, wr), ria)
    ria = np.minimum(np.maximum(wc, wr), ria)
    lam = [x[..., 1:-1] for x in lam]
    L = {k: v[..., 1:-1] for k, v in L.items()}
    R = {k: v[..., 1:-1] for k, v in R.items()}
    dtdx = dt / dn
    c1 = ria - lia
    c2 = 6.0 * (wc - 0.5 * (lia + ria))
    c3 = 0.5 * np.maximum(lam[4], 0.0) * dtdx
    c4 = -0.5 * np.minimum(lam[0], 0.0) * dtdx
    lia = lia + c4 * (c1 + (1.0 - FOUR_THIRDS * c4) * c2)
    ria = ria - c3 * (c1 - (1.0 - FOUR_THIRDS * c3) * c2)
    for i in range(5):
        ind = lam[i] <= 0.0
        v1 = 0.5 * dtdx * lam[0]
        v2 = 0.5 * dtdx * lam[i]
        v3 = v1 - v2
        v4 = FOUR_THIRDS * (np.square(v1) - np.square(v2))
        fac = np.zeros_like(v1)
        for j in range(5):
            e = L.get((i, j))
            if e is not None:
                fac = fac + ind * e * (v3 * (c1[j] + c2[j]) + v4 * c2[j])
        for j in range(5):
            e = R.get((j, i))
            if e is not None:
                lia[j] = lia[j] + fac * e
    for i in range(5):
        ind = lam[i] >= 0.0
        v1 = 0.5 * dtdx * lam[4]
        v2 = 0.5 * dtdx * lam[i]
        v3 = v1 - v2
        v4 = FOUR_THIRDS * (np.square(v1) - np.square(v2))
        fac = np.zeros_like(v1)
        for j in range(5):
            e = L.get((i, j))
            if e is not None:
                fac = fac + ind * e * (v3 * (c1[j] - c2[j]) + v4 * c2[j])
        for j in range(5):
            e = R.get((j, i))
            if e is not None:
                ria[j] = ria[j] + fac * e
    return faces_from_cells(lia, ria, bc)


def faces_from_cells(lia, ria, bc):
    if bc == OUTFLOW:
        return (np.concatenate([lia[..., :1], ria], axis=-1),
                np.concatenate([lia, ria[..., -1:]], axis=-1))
    return (np.concatenate([ria[..., -1:], ria], axis=-1),
            np.concatenate([lia, lia[..., :1]], axis=-1))


def roe_flux(wl, wr, gamma, efix, eps, yaxis):
    """riemannSolverX/Y/Z_hydro_roe (Source/RiemannSolvers_Hydro_Roe_HelperModule.py:68-328, :342-596,
    :614-869)."""
    ul = prim_to_cons(wl, gamma, yaxis)
    ur = prim_to_cons(wr, gamma, yaxis)
    n = 3 if yaxis == 2 else (2 if yaxis else 1)
    sl = np.sqrt(wl[0])
    sr = np.sqrt(wr[0])
    isum = 1.0 / (sl + sr)
    v = {k: (sl * wl[k] + sr * wr[k]) * isum for k in (1, 2, 3)}
    if yaxis == 2:
        vsq = v[3] * v[3] + v[1] * v[1] + v[2] * v[2]
    elif yaxis:
        vsq = v[2] * v[2] + v[3] * v[3] + v[1] * v[1]
    else:
        vsq = v[1] * v[1] + v[2] * v[2] + v[3] * v[3]
    H = ((ul[4] + wl[4]) / sl + (ur[4] + wr[4]) / sr) * isum
    a2 = (gamma - 1.0) * np.maximum(H - 0.5 * vsq, SMALL_VALUE)
    a = np.sqrt(a2)
    vn = v[n]
    lam = [vn - a, vn, vn, vn, vn + a]
    if efix:
        lam = [x + np.sign(x) * (np.abs(x) < 2.0 * eps) * (eps + np.square(x) / (4.0 * eps)) for x in lam]
    one = np.ones_like(a)
    R = {}
    L = {}
    nf = 0.5 / a2
    g1 = gamma - 1.0
    gn = g1 / a2
    if yaxis == 2:
        # wave order (acoustic-, vy, entropy, vx, acoustic+) (:720-783)
        R[0, 0] = one
        R[1, 0] = v[1]
        R[2, 0] = v[2]
        R[3, 0] = v[3] - a
        R[4, 0] = H - v[3] * a
        R[2, 1] = one
        R[4, 1] = v[2]
        R[0, 2] = one
        R[1, 2] = v[1]
        R[2, 2] = v[2]
        R[3, 2] = v[3]
        R[4, 2] = 0.5 * vsq
        R[1, 3] = one
        R[4, 3] = v[1]
        R[0, 4] = one
        R[1, 4] = v[1]
        R[2, 4] = v[2]
        R[3, 4] = v[3] + a
        R[4, 4] = H + v[3] * a
        L[0, 0] = nf * (0.5 * g1 * vsq + v[3] * a)
        L[0, 1] = -nf * g1 * v[1]
        L[0, 2] = -nf * g1 * v[2]
        L[0, 3] = -nf * (g1 * v[3] + a)
        L[0, 4] = nf * g1
        L[1, 0] = -v[2]
        L[1, 2] = one
        L[2, 0] = 1.0 - nf * g1 * vsq
        L[2, 1] = gn * v[1]
        L[2, 2] = gn * v[2]
        L[2, 3] = gn * v[3]
        L[2, 4] = -gn
        L[3, 0] = -v[1]
        L[3, 1] = one
        L[4, 0] = nf * (0.5 * g1 * vsq - v[3] * a)
        L[4, 1] = L[0, 1]
        L[4, 2] = L[0, 2]
        L[4, 3] = -nf * (g1 * v[3] - a)
        L[4, 4] = L[0, 4]
    elif not yaxis:
        R[0, 0] = one
        R[1, 0] = v[1] - a
        R[2, 0] = v[2]
        R[3, 0] = v[3]
        R[4, 0] = H - v[1] * a
        R[2, 1] = one
        R[4, 1] = v[2]
        R[3, 2] = one
        R[4, 2] = v[3]
        R[0, 3] = one
        R[1, 3] = v[1]
        R[2, 3] = v[2]
        R[3, 3] = v[3]
        R[4, 3] = 0.5 * vsq
        R[0, 4] = one
        R[1, 4] = v[1] + a
        R[2, 4] = v[2]
        R[3, 4] = v[3]
        R[4, 4] = H + v[1] * a
        L[0, 0] = nf * (0.5 * g1 * vsq + v[1] * a)
        L[0, 1] = -nf * (g1 * v[1] + a)
        L[0, 2] = -nf * g1 * v[2]
        L[0, 3] = -nf * g1 * v[3]
        L[0, 4] = nf * g1
        L[1, 0] = -v[2]
        L[1, 2] = one
        L[2, 0] = -v[3]
        L[2, 3] = one
        L[3, 0] = 1.0 - nf * g1 * vsq
        L[3, 1] = gn * v[1]
        L[3, 2] = gn * v[2]
        L[3, 3] = gn * v[3]
        L[3, 4] = -gn
        L[4, 0] = nf * (0.5 * g1 * vsq - v[1] * a)
        L[4, 1] = -nf * (g1 * v[1] - a)
        L[4, 2] = L[0, 2]
        L[4, 3] = L[0, 3]
        L[4, 4] = L[0, 4]
    else:
        R[0, 0] = one
        R[1, 0] = v[1]
        R[2, 0] = v[2] - a
        R[3, 0] = v[3]
        R[4, 0] = H - v[2] * a
        R[0, 1] = one
        R[1, 1] = v[1]
        R[2, 1] = v[2]
        R[3, 1] = v[3]
        R[4, 1] = 0.5 * vsq
        R[3, 2] = one
        R[4, 2] = v[3]
        R[1, 3] = one
        R[4, 3] = v[1]
        R[0, 4] = one
        R[1, 4] = v[1]
        R[2, 4] = v[2] + a
        R[3, 4] = v[3]
        R[4, 4] = H + v[2] * a
        L[0, 0] = nf * (0.5 * g1 * vsq + v[2] * a)
        L[0, 1] = -nf * g1 * v[1]
        L[0, 2] = -nf * (g1 * v[2] + a)
        L[0, 3] = -nf * g1 * v[3]
        L[0, 4] = nf * g1
        L[1, 0] = 1.0 - nf * g1 * vsq
        L[1, 1] = gn * v[1]
        L[1, 2] = gn * v[2]
        L[1, 3] = gn * v[3]
        L[1, 4] = -gn
        L[2, 0] = -v[3]
        L[2, 3] = one
        L[3, 0] = -v[1]
        L[3, 1] = one
        L[4, 0] = nf * (0.5 * g1 * vsq - v[2] * a)
        L[4, 1] = L[0, 1]
        L[4, 2] = -nf * (g1 * v[2] - a)
        L[4, 3] = L[0, 3]
        L[4, 4] = L[0, 4]

    def cell_flux(w, u):
        def mom(k):  # the normal momentum flux carries the pressure
            return u[n] * w[k] + w[4] if k == n else u[n] * w[k]
        return np.array([u[n], mom(1), mom(2), mom(3),
                         (u[4] + w[4]) * w[n]])

    fl = cell_flux(wl, ul)
    fr = cell_flux(wr, ur)
    du = ur - ul
    amps = [0.5 * np.abs(lam[k]) * _project(L, k, du) for k in range(5)]
    flux = 0.5 * (fl + fr)
    for i in range(5):
        acc = flux[i]
        for j in range(5):
            e = R.get((i, j))
            if e is not None:
                acc = acc - amps[j] * e
        flux[i] = acc
    m0 = lam[0] >= 0.0
    flux[:, m0] = fl[:, m0]
    m4 = lam[4] <= 0.0
    flux[:, m4] = fr[:, m4]
    return flux


def swap_xy(a):
    return np.ascontiguousarray(np.swapaxes(a, -1, -2))


def cycle(prim, cons, dt, dx, dy, bcx, bcy, gamma, min_d, min_p, min_e, order, efix, eps):
    """One cycle of evolve_2D_hydro (Source/EvolveFunctions_Hydro.py:390-513).

    Returns new (prim, cons); the inputs are not modified.
    """
    Ny, Nx = prim.shape[1:]
    half_dtdx = 0.5 * (dt / dx)
    half_dtdy = 0.5 * (dt / dy)
    if order in (1, 2):
        lin = order == 1
        xl, xr = ppm_sweep(prim, gamma, dt, dx, bcx, False, linear=lin)
        tl, tr = ppm_sweep(swap_xy(prim), gamma, dt, dy, bcy, True, linear=lin)
    else:
        xl, xr = faces_from_cells(prim, prim, bcx)
        tl, tr = faces_from_cells(swap_xy(prim), swap_xy(prim), bcy)
    yl, yr = swap_xy(tl), swap_xy(tr)
    for a in (xl, xr, yl, yr):
        apply_floors_inplace(a, min_d, min_p)
    uxl = prim_to_cons(xl, gamma, False)
    uxr = prim_to_cons(xr, gamma, False)
    uyl = prim_to_cons(yl, gamma, True)
    uyr = prim_to_cons(yr, gamma, True)
    fx = roe_flux(xl, xr, gamma, efix, eps, False)
    fy = roe_flux(yl, yr, gamma, efix, eps, True)

    f = np.arange(Nx + 1)
    lfy = take_x(fy, wrap_index(f - 1, Nx, bcx))
    rfy = take_x(fy, wrap_index(f, Nx, bcx))
    g = np.arange(Ny + 1)
    tfx = take_y(fx, wrap_index(g - 1, Ny, bcy))
    bfx = take_y(fx, wrap_index(g, Ny, bcy))
    uxl -= half_dtdy * (lfy[:, 1:, :] - lfy[:, :-1, :])
    uxr -= half_dtdy * (rfy[:, 1:, :] - rfy[:, :-1, :])
    uyl -= half_dtdx * (tfx[:, :, 1:] - tfx[:, :, :-1])
    uyr -= half_dtdx * (bfx[:, :, 1:] - bfx[:, :, :-1])
    xl = cons_to_prim(uxl, gamma, False)
    xr = cons_to_prim(uxr, gamma, False)
    yl = cons_to_prim(uyl, gamma, True)
    yr = cons_to_prim(uyr, gamma, True)
    fx2 = roe_flux(xl, xr, gamma, efix, eps, False)
    fy2 = roe_flux(yl, yr, gamma, efix, eps, True)
    nu = cons - (dt / dx) * (fx2[:, :, 1:] - fx2[:, :, :-1])
    nu -= (dt / dy) * (fy2[:, 1:, :] - fy2[:, :-1, :])
    nw = cons_to_prim(nu, gamma, False)
    return nw, nu


def evolve(prim, cons, dx, dy, bcx, bcy, t_start, t_end, start_cycle, max_cycles,
           gamma, cfl, min_d, min_p, min_e, order=0, efix=False, eps=0.5, dt_log=None):
    """The evolve_2D_hydro loop; returns the reference's 7-tuple."""
    prim = np.array(prim, dtype=np.float64)
    cons = np.array(cons, dtype=np.float64)
    t = t_start
    cyc = start_cycle
    sl = (prim.copy(), cons.copy(), t_start)
    while t < t_end and cyc < max_cycles:
        sl = (prim.copy(), cons.copy(), t)
        dt = calc_dt(cons, gamma, cfl, dx, dy)
        if t + dt > t_end:
            dt = t_end - t
        if dt_log is not None:
            dt_log.append(dt)
        prim, cons = cycle(prim, cons, dt, dx, dy, bcx, bcy, gamma, min_d, min_p, min_e,
                           order, efix, eps)
        t += dt
        cyc += 1
    return (prim, cons, t, cyc) + sl
