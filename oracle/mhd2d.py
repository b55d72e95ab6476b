"""CPU oracle: one 2D CTU+CT cycle of ideal MHD, restated in NumPy.

TEST INFRASTRUCTURE ONLY (see ``oracle/common.py``). Every function below
cites the reference routine it restates and keeps that routine's operation
order, so that on the same inputs it returns the reference's bits.
"""
from __future__ import annotations

import numpy as np

from .common import (FOUR_THIRDS, FRAME_X, FRAME_Y, OUTFLOW,
                     SMALL_VALUE, Frame, apply_floors_inplace, np_sign_one,
                     take_x, take_y, wrap_index)


# ----------------------------------------------------------------------------
# prim <-> cons (Source/PrimCons_HelperModule.py)
# ----------------------------------------------------------------------------
def prim_to_cons7(w, bn, gamma):
    """primToCons_mhd (Source/PrimCons_HelperModule.py:208-229)."""
    u = np.empty_like(w)
    u[0] = w[0]
    u[1] = w[0] * w[1]
    u[2] = w[0] * w[2]
    u[3] = w[0] * w[3]
    u[4] = w[4]
    u[5] = w[5]
    u[6] = w[6] / (gamma - 1.0) + 0.5 * w[0] * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3])
    u[6] += 0.5 * (bn * bn + w[4] * w[4] + w[5] * w[5])
    return u


def cons_to_prim7(u, bn, gamma):
    """consToPrim_mhd (Source/PrimCons_HelperModule.py:358-380)."""
    w = np.empty_like(u)
    inv_d = 1.0 / u[0]
    w[0] = u[0]
    w[1] = u[1] * inv_d
    w[2] = u[2] * inv_d
    w[3] = u[3] * inv_d
    w[4] = u[4]
    w[5] = u[5]
    w[6] = u[6] - 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) * inv_d
    w[6] -= 0.5 * (bn * bn + w[4] * w[4] + w[5] * w[5])
    w[6] *= (gamma - 1.0)
    return w


def prim_to_cons8(p, gamma):
    """primToCons_mhd_allVars (Source/PrimCons_HelperModule.py:314-340)."""
    c = np.empty_like(p)
    c[0] = p[0]
    c[1] = p[0] * p[1]
    c[2] = p[0] * p[2]
    c[3] = p[0] * p[3]
    c[4] = p[4]
    c[5] = p[5]
    c[6] = p[6]
    c[7] = p[7] / (gamma - 1.0) + 0.5 * p[0] * (p[1] * p[1] + p[2] * p[2] + p[3] * p[3])
    c[7] += 0.5 * (p[4] * p[4] + p[5] * p[5] + p[6] * p[6])
    return c


# ----------------------------------------------------------------------------
# CFL timestep (Source/TimestepCalculations_HelperModule.py:239-289)
# ----------------------------------------------------------------------------
def calc_dt(cons, fbx, fby, gamma, cfl, dx, dy):
    g1 = gamma - 1.0
    inv_d = 1.0 / cons[0]
    vx = cons[1] * inv_d
    vy = cons[2] * inv_d
    vz = cons[3] * inv_d
    vsq = vx * vx + vy * vy + vz * vz
    bx = cons[4] + np.abs(fbx[:, :-1] - cons[4])
    by = cons[5] + np.abs(fby[:-1, :] - cons[5])
    bz = cons[6]
    bsq = bx * bx + by * by + bz * bz
    p = np.maximum(g1 * (cons[7] - 0.5 * cons[0] * vsq - 0.5 * bsq), SMALL_VALUE)
    a2 = gamma * p * inv_d
    ssum = bsq * inv_d + a2
    sdiff = bsq * inv_d - a2
    cfx2 = 0.5 * (ssum + np.sqrt(sdiff * sdiff + 4.0 * a2 * (by * by + bz * bz) * inv_d))
    cfy2 = 0.5 * (ssum + np.sqrt(sdiff * sdiff + 4.0 * a2 * (bx * bx + bz * bz) * inv_d))
    max_x = np.max(np.abs(vx) + np.sqrt(cfx2))
    max_y = np.max(np.abs(vy) + np.sqrt(cfy2))
    inv_dt = np.maximum(max_x / dx, max_y / dy)
    return cfl / inv_dt


# ----------------------------------------------------------------------------
# Cell-centred primitive eigensystem
# (Source/ReconstructionEigenmatrices_MHD_HelperModule.py:27-207 for x,
#  :220-396 for y; the y routine is the x routine in FRAME_Y)
# ----------------------------------------------------------------------------
def prim_eigensystem(w, bn, gamma, fr: Frame):
    n, t1, t2 = fr.n, fr.t1, fr.t2
    bt2 = np.square(w[4]) + np.square(w[5])
    bt = np.sqrt(bt2)
    gp = gamma * w[6]
    inv_d = 1.0 / w[0]
    sqrt_d = np.sqrt(w[0])
    red_bt2 = bt2 * inv_d
    a2 = gp * inv_d
    a = np.sqrt(a2)
    ca2 = bn * bn * inv_d
    ca = np.sqrt(ca2)
    ssum = ca2 + red_bt2 + a2
    sdiff = ca2 + red_bt2 - a2
    ssqrt = np.sqrt(sdiff * sdiff + 4.0 * a2 * red_bt2)
    cf2 = 0.5 * (ssum + ssqrt)
    cf = np.sqrt(cf2)
    cs2 = a2 * ca2 / cf2
    cs = np.sqrt(cs2)

    b1 = np.zeros_like(bt)
    b2 = np.zeros_like(bt)
    b1[bt == 0.0] = 1.0
    pos = bt > 0.0
    b1[pos] = w[4][pos] / bt[pos]
    b2[pos] = w[5][pos] / bt[pos]

    fa = np.zeros_like(bt)
    sa = np.zeros_like(bt)
    one_f = ssqrt == 0.0
    fa[one_f] = 1.0
    one_s = np.logical_and(~one_f, (a2 - cs2) <= 0.0)
    sa[one_s] = 1.0
    one_f2 = np.logical_and(~(one_f | one_s), (cf2 - a2) <= 0.0)
    fa[one_f2] = 1.0
    calc = ~(one_f | one_s | one_f2)
    fa[calc] = np.sqrt((a2 - cs2)[calc] / ssqrt[calc])
    sa[calc] = np.sqrt((cf2 - a2)[calc] / ssqrt[calc])

    sgn = np_sign_one(bn)
    qf = cf * fa * sgn
    qs = cs * sa * sgn
    af = a * fa * sqrt_d
    as_ = a * sa * sqrt_d

    vn = w[n]
    lam = [vn - cf, vn - ca, vn - cs, vn, vn + cs, vn + ca, vn + cf]

    R = {}
    R[0, 0] = w[0] * fa
    R[0, 2] = w[0] * sa
    R[0, 3] = np.ones_like(bt)
    R[0, 4] = R[0, 2]
    R[0, 6] = R[0, 0]
    R[n, 0] = -cf * fa
    R[n, 2] = -cs * sa
    R[n, 4] = -R[n, 2]
    R[n, 6] = -R[n, 0]
    R[t1, 0] = qs * b1
    R[t1, 1] = -b2
    R[t1, 2] = -qf * b1
    R[t1, 4] = -R[t1, 2]
    R[t1, 5] = b2
    R[t1, 6] = -R[t1, 0]
    R[t2, 0] = qs * b2
    R[t2, 1] = b1
    R[t2, 2] = -qf * b2
    R[t2, 4] = -R[t2, 2]
    R[t2, 5] = -b1
    R[t2, 6] = -R[t2, 0]
    R[6, 0] = w[0] * a2 * fa
    R[6, 2] = w[0] * a2 * sa
    R[6, 4] = R[6, 2]
    R[6, 6] = R[6, 0]
    R[4, 0] = as_ * b1
    R[4, 1] = -b2 * sgn * sqrt_d
    R[4, 2] = -af * b1
    R[4, 4] = R[4, 2]
    R[4, 5] = R[4, 1]
    R[4, 6] = R[4, 0]
    R[5, 0] = as_ * b2
    R[5, 1] = b1 * sgn * sqrt_d
    R[5, 2] = -af * b2
    R[5, 4] = R[5, 2]
    R[5, 5] = R[5, 1]
    R[5, 6] = R[5, 0]

    nf = 0.5 / a2
    qf_n = nf * qf
    qs_n = nf * qs
    afp = nf * af * inv_d
    asp = nf * as_ * inv_d
    L = {}
    L[0, n] = -nf * cf * fa
    L[0, t1] = qs_n * b1
    L[0, t2] = qs_n * b2
    L[0, 6] = nf * fa * inv_d
    L[0, 4] = asp * b1
    L[0, 5] = asp * b2
    L[1, t1] = -0.5 * b2
    L[1, t2] = 0.5 * b1
    L[1, 4] = -0.5 * b2 * sgn / sqrt_d
    L[1, 5] = 0.5 * b1 * sgn / sqrt_d
    L[2, n] = -nf * cs * sa
    L[2, t1] = -qf_n * b1
    L[2, t2] = -qf_n * b2
    L[2, 6] = nf * sa * inv_d
    L[2, 4] = -afp * b1
    L[2, 5] = -afp * b2
    L[3, 0] = np.ones_like(bt)
    L[3, 6] = -1.0 / a2
    L[4, n] = -L[2, n]
    L[4, t1] = -L[2, t1]
    L[4, t2] = -L[2, t2]
    L[4, 6] = L[2, 6]
    L[4, 4] = L[2, 4]
    L[4, 5] = L[2, 5]
    L[5, t1] = -L[1, t1]
    L[5, t2] = -L[1, t2]
    L[5, 4] = L[1, 4]
    L[5, 5] = L[1, 5]
    L[6, n] = -L[0, n]
    L[6, t1] = -L[0, t1]
    L[6, t2] = -L[0, t2]
    L[6, 6] = L[0, 6]
    L[6, 4] = L[0, 4]
    L[6, 5] = L[0, 5]
    return lam, L, R


def _project(L, i, vec, order):
    """Row i of L times vec, accumulated in the reference's order from +0."""
    acc = np.zeros_like(vec[0])
    for j in order:
        e = L.get((i, j))
        if e is not None:
            acc = acc + e * vec[j]
    return acc


# ----------------------------------------------------------------------------
# PPM reconstruction along the last axis
# (Source/Reconstruction_PPM_MHD_HelperModule.py:189-551 for x, :570-871 for y)
# ----------------------------------------------------------------------------
def ppm_sweep(w, bn_cell, gamma, dt, dn, bc, fr: Frame, linear=False):
    """Return (left_state, right_state) at the N+1 interfaces along the last axis.

    ``w`` is (7, M, N) sweep ordered, ``bn_cell`` (M, N) the cell-centred normal B.
    ``linear=True`` gives the PLM variant (no reference counterpart, see ``plm_edges``).
    """
    N = w.shape[-1]
    idx = np.arange(-2, N + 2)
    g = wrap_index(idx, N, bc)
    we = take_x(w, g)                     # (7, M, N+4): cells -2 .. N+1
    be = take_x(bn_cell, g)
    wc = we[..., 1:-1]                    # cells -1 .. N
    wl = we[..., :-2]
    wr = we[..., 2:]
    bc_c = be[..., 1:-1]
    lam, L, R = prim_eigensystem(wc, bc_c, gamma, fr)
    order = fr.proj_order

    d_c = wr - wl
    d_l = wc - wl
    d_r = wr - wc
    weight = np.zeros_like(wc)
    wi = d_l * d_r > 0.0
    weight[wi] = (2.0 * d_l * d_r)[wi] / (d_l + d_r)[wi]

    slopes_char = np.zeros_like(wc)
    for i in range(7):
        cc = _project(L, i, d_c, order)
        cl = _project(L, i, d_l, order)
        cr = _project(L, i, d_r, order)
        cw = _project(L, i, weight, order)
        ok = cl * cr > 0.0
        lim1 = np.minimum(np.abs(cl), np.abs(cr))
        lim2 = np.minimum(0.5 * np.abs(cc), np.abs(cw))
        s = np.sign(cc) * np.minimum(2.0 * lim1, lim2)
        slopes_char[i][ok] = s[ok]

    slopes = np.zeros_like(wc)
    for i in range(7):
        acc = np.zeros_like(wc[0])
        for j in range(7):
            e = R.get((i, j))
            if e is not None:
                acc = acc + slopes_char[j] * e
        slopes[i] = acc

    s_c = slopes[..., 1:-1]
    s_l = slopes[..., :-2]
    s_r = slopes[..., 2:]
    wc = wc[..., 1:-1]
    wl = wl[..., 1:-1]
    wr = wr[..., 1:-1]
    if linear:
        lam = [x[..., 1:-1] for x in lam]
        L = {k: v[..., 1:-1] for k, v in L.items()}
        R = {k: v[..., 1:-1] for k, v in R.items()}
        lia, ria = plm_edges(wc, wl, wr, s_c, lam, L, R, dt / dn, order, 7)
        return _faces_from_cells(lia, ria, bc)

    lia = 0.5 * (wc + wl) - (s_c - s_l) / 6.0
    ria = 0.5 * (wr + wc) - (s_r - s_c) / 6.0
    dprod = (ria - wc) * (wc - lia)
    idiff = ria - lia
    adiff = 6.0 * (wc - 0.5 * (lia + ria))
    nz = dprod <= 0.0
    pz = ~nz
    lia[nz] = wc[nz]
    ria[nz] = wc[nz]
    cl_ = np.logical_and(pz, (idiff * adiff) > np.square(idiff))
    lia[cl_] = ((6.0 * wc - 4.0 * ria) / 2.0)[cl_]
    cr_ = np.logical_and(np.logical_and(pz, ~cl_), (idiff * adiff) < (-1.0 * np.square(idiff)))
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
    c3 = 0.5 * np.maximum(lam[6], 0.0) * dtdx
    c4 = -0.5 * np.minimum(lam[0], 0.0) * dtdx
    lia = lia + c4 * (c1 + (1.0 - FOUR_THIRDS * c4) * c2)
    ria = ria - c3 * (c1 - (1.0 - FOUR_THIRDS * c3) * c2)

    for i in range(7):
        ind = lam[i] <= 0.0
        v1 = 0.5 * dtdx * lam[0]
        v2 = 0.5 * dtdx * lam[i]
        v3 = v1 - v2
        v4 = FOUR_THIRDS * (np.square(v1) - np.square(v2))
        fac = np.zeros_like(v1)
        for j in order:
            e = L.get((i, j))
            if e is not None:
                fac = fac + ind * e * (v3 * (c1[j] + c2[j]) + v4 * c2[j])
        for j in range(7):
            e = R.get((j, i))
            if e is not None:
                lia[j] = lia[j] + fac * e
    for i in range(7):
        ind = lam[i] >= 0.0
        v1 = 0.5 * dtdx * lam[6]
        v2 = 0.5 * dtdx * lam[i]
        v3 = v1 - v2
        v4 = FOUR_THIRDS * (np.square(v1) - np.square(v2))
        fac = np.zeros_like(v1)
        for j in order:
            e = L.get((i, j))
            if e is not None:
                fac = fac + ind * e * (v3 * (c1[j] - c2[j]) + v4 * c2[j])
        for j in range(7):
            e = R.get((j, i))
            if e is not None:
                ria[j] = ria[j] + fac * e

    return _faces_from_cells(lia, ria, bc)


def plm_edges(wc, wl, wr, s, lam, L, R, dtdx, order, nv):
    """PLM edge states of each cell with dt/2 characteristic tracing.

    No counterpart in the reference (its PLM branches are commented out,
    Source/EvolveFunctions_MHD.py:487-488).  The limited slope ``s`` is the
    reference's characteristic-limited slope (primMonSlopes,
    Source/Reconstruction_PPM_MHD_HelperModule.py:317-389); the edge values are
    W -/+ s/2 kept between the neighbours, and the tracing is the reference's
    own (:460-524) applied to the linear profile, i.e. with the parabolic
    coefficient zero -- the PLM tracing of Stone et al. (2008) eqs. 38-42 with the
    reference's <= / >= wave tests.
    """
    lia = wc - 0.5 * s
    ria = wc + 0.5 * s
    lia = np.maximum(np.minimum(wc, wl), lia)
    lia = np.minimum(np.maximum(wc, wl), lia)
    ria = np.maximum(np.minimum(wc, wr), ria)
    ria = np.minimum(np.maximum(wc, wr), ria)
    c1 = ria - lia
    c3 = 0.5 * np.maximum(lam[nv - 1], 0.0) * dtdx
    c4 = -0.5 * np.minimum(lam[0], 0.0) * dtdx
    lia = lia + c4 * c1
    ria = ria - c3 * c1
    for i in range(nv):
        ind = lam[i] <= 0.0
        v3 = 0.5 * dtdx * lam[0] - 0.5 * dtdx * lam[i]
        fac = np.zeros_like(v3)
        for j in order:
            e = L.get((i, j))
            if e is not None:
                fac = fac + ind * e * (v3 * c1[j])
        for j in range(nv):
            e = R.get((j, i))
            if e is not None:
                lia[j] = lia[j] + fac * e
    for i in range(nv):
        ind = lam[i] >= 0.0
        v3 = 0.5 * dtdx * lam[nv - 1] - 0.5 * dtdx * lam[i]
        fac = np.zeros_like(v3)
        for j in order:
            e = L.get((i, j))
            if e is not None:
                fac = fac + ind * e * (v3 * c1[j])
        for j in range(nv):
            e = R.get((j, i))
            if e is not None:
                ria[j] = ria[j] + fac * e
    return lia, ria


def _faces_from_cells(lia, ria, bc):
    """Interface states from per-cell edge values (reference :529-548)."""
    if bc == OUTFLOW:
        left = np.concatenate([lia[..., :1], ria], axis=-1)
        right = np.concatenate([lia, ria[..., -1:]], axis=-1)
    else:
        left = np.concatenate([ria[..., -1:], ria], axis=-1)
        right = np.concatenate([lia, lia[..., :1]], axis=-1)
    return left, right


def first_order_sweep(w, bc):
    """reconstructOrder=0 face states (Source/EvolveFunctions_MHD.py:489-511)."""
    return _faces_from_cells(w, w, bc)


def swap_xy(a):
    return np.ascontiguousarray(np.swapaxes(a, -1, -2))


# ----------------------------------------------------------------------------
# Reconstruction source terms for the transverse in-plane B
# (Source/Reconstruction_PPM_MHD_HelperModule.py:1193-1239)
# ----------------------------------------------------------------------------
def by_source_terms(vy, fbx, dt, dx, bcx):
    """getByReconSourceTerms_2D: (2, Ny, Nx+1) corrections for x-face By."""
    inv_dx = 1.0 / dx
    half_dt = 0.5 * dt
    N = vy.shape[1]
    f = np.arange(N + 1)
    lv = take_x(vy, wrap_index(f - 1, N, bcx))
    rv = take_x(vy, wrap_index(f, N, bcx))
    if bcx == OUTFLOW:
        lf_idx = np.clip(f - 1, 0, N)
        rf_idx = np.clip(f + 1, 0, N)
    else:
        lf_idx = np.where(f == 0, N - 1, f - 1)
        rf_idx = np.where(f == N, 1, f + 1)
    lfb = take_x(fbx, lf_idx)
    rfb = take_x(fbx, rf_idx)
    out = np.empty((2,) + fbx.shape)
    out[0] = half_dt * lv * ((fbx - lfb) * inv_dx)
    out[1] = half_dt * rv * ((rfb - fbx) * inv_dx)
    return out


def bx_source_terms(vx, fby, dt, dy, bcy):
    """getBxReconSourceTerms_2D: (2, Ny+1, Nx) corrections for y-face Bx."""
    t = by_source_terms(swap_xy(vx), swap_xy(fby), dt, dy, bcy)
    return np.swapaxes(t, -1, -2).copy()


# ----------------------------------------------------------------------------
# Roe solver (Source/RiemannSolvers_MHD_Roe_HelperModule.py:74-576 for x,
# :595-1071 for y)
# ----------------------------------------------------------------------------
def roe_flux(wl, wr, ul, ur, bn, gamma, efix, eps, fr: Frame):
    n, t1, t2 = fr.n, fr.t1, fr.t2
    sl = np.sqrt(wl[0])
    sr = np.sqrt(wr[0])
    isum = 1.0 / (sl + sr)
    rd = sl * sr
    v = {}
    for k in (1, 2, 3):
        v[k] = (sl * wl[k] + sr * wr[k]) * isum
    vsq = v[n] * v[n] + v[t1] * v[t1] + v[t2] * v[t2]
    b1 = (sr * wl[4] + sl * wr[4]) * isum
    b2 = (sr * wl[5] + sl * wr[5]) * isum
    hbl = 0.5 * (np.square(bn) + np.square(wl[4]) + np.square(wl[5]))
    hbr = 0.5 * (np.square(bn) + np.square(wr[4]) + np.square(wr[5]))
    pl = wl[6]
    pr = wr[6]
    H = ((ul[6] + pl + hbl) / sl + (ur[6] + pr + hbr) / sr) * isum

    ird = 1.0 / rd
    btc = 0.5 * (np.square(wl[4] - wr[4]) + np.square(wl[5] - wr[5])) / (np.square(sl + sr))
    rc = 0.5 * (wl[0] + wr[0]) / rd
    bt2 = b1 * b1 + b2 * b2
    bt = np.sqrt(bt2)
    bts2 = ((gamma - 1.0) - (gamma - 2.0) * rc) * bt2
    bts = np.sqrt(bts2)
    rbts2 = bts2 * ird
    ca2 = bn * bn * ird
    ca = np.sqrt(ca2)
    hmb = H - (ca2 + bt2 * ird)
    a2 = np.maximum((gamma - 1.0) * (hmb - 0.5 * vsq) - (gamma - 2.0) * btc, SMALL_VALUE)
    a = np.sqrt(a2)
    ssum = ca2 + rbts2 + a2
    sdiff = ca2 + rbts2 - a2
    ssqrt = np.sqrt(sdiff * sdiff + 4.0 * a2 * rbts2)
    cf2 = 0.5 * (ssum + ssqrt)
    cf = np.sqrt(cf2)
    cs2 = a2 * ca2 / cf2
    cs = np.sqrt(cs2)

    vn = v[n]
    lam = [vn - cf, vn - ca, vn - cs, vn, vn + cs, vn + ca, vn + cf]
    if efix:
        lam = [x + np.sign(x) * (np.abs(x) < 2.0 * eps) * (eps + np.square(x) / (4.0 * eps)) for x in lam]

    fa = np.zeros_like(cf)
    sa = np.zeros_like(cf)
    one_f = cf2 - cs2 == 0.0
    fa[one_f] = 1.0
    one_s = np.logical_and(~one_f, a2 - cs2 <= 0.0)
    sa[one_s] = 1.0
    one_f2 = np.logical_and(~(one_f | one_s), cf2 - a2 <= 0.0)
    fa[one_f2] = 1.0
    calc = ~((cf2 - cs2 == 0.0) | (a2 - cs2 <= 0.0) | (cf2 - a2 <= 0.0))
    fa[calc] = np.sqrt((a2 - cs2)[calc] / (cf2 - cs2)[calc])
    sa[calc] = np.sqrt((cf2 - a2)[calc] / (cf2 - cs2)[calc])

    sgn = np_sign_one(bn)
    srd = np.sqrt(rd)
    isrd = 1.0 / srd
    qf = cf * fa * sgn
    qs = cs * sa * sgn
    afp = a * fa * isrd
    asp = a * sa * isrd

    bh1 = np.zeros_like(bt)
    bh2 = np.zeros_like(bt)
    bh1[bt == 0.0] = 1.0
    pos = bt > 0.0
    bh1[pos] = b1[pos] / bt[pos]
    bh2[pos] = b2[pos] / bt[pos]
    den = np.sqrt((gamma - 1.0) - (gamma - 2.0) * rc)
    b1s = bh1 / den
    b2s = bh2 / den
    vb = v[t1] * b1s + v[t2] * b2s
    bs2 = b1s * b1s + b2s * b2s
    afb = afp * bts * bs2
    asb = asp * bts * bs2

    R = {}
    R[0, 0] = fa
    R[0, 2] = sa
    R[0, 3] = np.ones_like(fa)
    R[0, 4] = sa
    R[0, 6] = fa
    R[n, 0] = fa * lam[0]
    R[n, 2] = sa * lam[2]
    R[n, 3] = vn
    R[n, 4] = sa * lam[4]
    R[n, 6] = fa * lam[6]
    for tk, bsk, bhk, bho, sgn_o in ((t1, b1s, bh1, bh2, -1.0), (t2, b2s, bh2, bh1, 1.0)):
        fv = fa * v[tk]
        sv = sa * v[tk]
        qsb = qs * bsk
        qfb = qf * bsk
        R[tk, 0] = fv + qsb
        R[tk, 1] = -bho if sgn_o < 0 else bho
        R[tk, 2] = sv - qfb
        R[tk, 3] = v[tk]
        R[tk, 4] = sv + qfb
        R[tk, 5] = bho if sgn_o < 0 else -bho
        R[tk, 6] = fv - qsb
    R[6, 0] = fa * (hmb - vn * cf) + qs * vb + asb
    R[6, 1] = -(v[t1] * bh2 - v[t2] * bh1)
    R[6, 2] = sa * (hmb - vn * cs) - qf * vb - afb
    R[6, 3] = 0.5 * vsq + (gamma - 2.0) * btc / (gamma - 1.0)
    R[6, 4] = sa * (hmb + vn * cs) + qf * vb - afb
    R[6, 5] = -R[6, 1]
    R[6, 6] = fa * (hmb + vn * cf) - qs * vb + asb
    R[4, 0] = asp * b1s
    R[4, 1] = -bh2 * sgn * isrd
    R[4, 2] = -afp * b1s
    R[4, 4] = R[4, 2]
    R[4, 5] = R[4, 1]
    R[4, 6] = R[4, 0]
    R[5, 0] = asp * b2s
    R[5, 1] = bh1 * sgn * isrd
    R[5, 2] = -afp * b2s
    R[5, 4] = R[5, 2]
    R[5, 5] = R[5, 1]
    R[5, 6] = R[5, 0]

    nf = 0.5 / a2
    cff = nf * fa * cf
    css = nf * sa * cs
    qf = qf * nf
    qs = qs * nf
    af = nf * afp * rd
    as_ = nf * asp * rd
    afb = nf * afp * bts
    asb = nf * asp * bts
    nf = nf * (gamma - 1.0)
    fa = fa * nf
    sa = sa * nf
    b1c = b1s / bs2
    b2c = b2s / bs2
    vbs = v[t1] * b1c + v[t2] * b2c
    nf = nf * 2.0

    L = {}
    L[0, 0] = fa * (vsq - hmb) + cff * (cf + vn) - qs * vbs - asb
    L[0, n] = -1.0 * fa * vn - cff
    L[0, t1] = -1.0 * fa * v[t1] + qs * b1c
    L[0, t2] = -1.0 * fa * v[t2] + qs * b2c
    L[0, 6] = fa
    L[0, 4] = as_ * b1c - fa * b1
    L[0, 5] = as_ * b2c - fa * b2
    L[1, 0] = 0.5 * (v[t1] * bh2 - v[t2] * bh1)
    L[1, t1] = -0.5 * bh2
    L[1, t2] = 0.5 * bh1
    L[1, 4] = -0.5 * srd * bh2 * sgn
    L[1, 5] = 0.5 * srd * bh1 * sgn
    L[2, 0] = sa * (vsq - hmb) + css * (cs + vn) + qf * vbs + afb
    L[2, n] = -sa * vn - css
    L[2, t1] = -sa * v[t1] - qf * b1c
    L[2, t2] = -sa * v[t2] - qf * b2c
    L[2, 6] = sa
    L[2, 4] = -af * b1c - sa * b1
    L[2, 5] = -af * b2c - sa * b2
    L[3, 0] = 1.0 - nf * (0.5 * vsq - (gamma - 2.0) * btc / (gamma - 1.0))
    for k in (1, 2, 3):
        L[3, k] = nf * v[k]
    L[3, 6] = -1.0 * nf
    L[3, 4] = nf * b1
    L[3, 5] = nf * b2
    L[4, 0] = sa * (vsq - hmb) + css * (cs - vn) - qf * vbs + afb
    L[4, n] = -sa * vn + css
    L[4, t1] = -sa * v[t1] + qf * b1c
    L[4, t2] = -sa * v[t2] + qf * b2c
    L[4, 6] = sa
    L[4, 4] = L[2, 4]
    L[4, 5] = L[2, 5]
    L[5, 0] = -L[1, 0]
    L[5, t1] = -L[1, t1]
    L[5, t2] = -L[1, t2]
    L[5, 4] = L[1, 4]
    L[5, 5] = L[1, 5]
    L[6, 0] = fa * (vsq - hmb) + cff * (cf - vn) + qs * vbs - asb
    L[6, n] = -fa * vn + cff
    L[6, t1] = -fa * v[t1] - qs * b1c
    L[6, t2] = -fa * v[t2] - qs * b2c
    L[6, 6] = fa
    L[6, 4] = L[0, 4]
    L[6, 5] = L[0, 5]

    fl = _cell_flux(wl, ul, bn, hbl, fr)
    fr_ = _cell_flux(wr, ur, bn, hbr, fr)
    du = ur - ul
    order = fr.proj_order
    amps = [0.5 * np.abs(lam[k]) * _project(L, k, du, order) for k in range(7)]
    flux = 0.5 * (fl + fr_)
    for i in range(7):
        acc = flux[i]
        for j in range(7):
            e = R.get((i, j))
            if e is not None:
                acc = acc - amps[j] * e
        flux[i] = acc
    m0 = lam[0] >= 0.0
    flux[:, m0] = fl[:, m0]
    m6 = lam[6] <= 0.0
    flux[:, m6] = fr_[:, m6]
    return flux


def _cell_flux(w, u, bn, hb, fr: Frame):
    n, t1, t2 = fr.n, fr.t1, fr.t2
    p = w[6]
    F = np.empty_like(u)
    F[0] = u[n]
    for k in (1, 2, 3):
        F[k] = u[n] * w[k]
    F[n] = F[n] + p
    F[6] = (u[6] + p) * w[n]
    F[n] = F[n] - 0.5 * (bn * bn - np.square(w[4]) - np.square(w[5]))
    F[t1] = F[t1] - bn * w[4]
    F[t2] = F[t2] - bn * w[5]
    F[6] = F[6] + (hb * w[n] - bn * (bn * w[n] + w[4] * w[t1] + w[5] * w[t2]))
    F[4] = w[4] * w[n] - bn * w[t1]
    F[5] = w[5] * w[n] - bn * w[t2]
    return F


# ----------------------------------------------------------------------------
# Corner EMF (Source/CornerEMF_HelperModule.py:440-529)
# ----------------------------------------------------------------------------
def corner_emf(fx, fy, ez, bcx, bcy):
    """Ez at the (Ny+1, Nx+1) cell corners from the x/y face fluxes and cell Ez."""
    Ny, Nx = ez.shape
    jj = np.arange(Ny + 1)
    ii = np.arange(Nx + 1)
    # y-face fluxes at row j, columns i (right of the corner) and i-1 (left)
    top = take_x(fy, wrap_index(ii, Nx, bcx))
    ltop = take_x(fy, wrap_index(ii - 1, Nx, bcx))
    # x-face fluxes at column i, rows j (below the corner) and j-1 (above)
    left = take_y(fx, wrap_index(jj, Ny, bcy))
    uleft = take_y(fx, wrap_index(jj - 1, Ny, bcy))
    rj = wrap_index(jj, Ny, bcy)
    rjm = wrap_index(jj - 1, Ny, bcy)
    ci = wrap_index(ii, Nx, bcx)
    cim = wrap_index(ii - 1, Nx, bcx)
    e_c = ez[np.ix_(rj, ci)]
    e_l = ez[np.ix_(rj, cim)]
    e_u = ez[np.ix_(rjm, ci)]
    e_ul = ez[np.ix_(rjm, cim)]

    shape = (Ny + 1, Nx + 1)
    x1 = np.zeros(shape)
    s = ltop[0]
    m = s > 0.0
    x1[m] = (ltop[5] - uleft[4] - e_ul)[m]
    m = s < 0.0
    x1[m] = (ltop[5] - left[4] - e_l)[m]
    m = s == 0.0
    x1[m] = (ltop[5] - 0.5 * (left[4] + uleft[4] + e_l + e_ul))[m]

    x2 = np.zeros(shape)
    s = top[0]
    m = s > 0.0
    x2[m] = (top[5] - uleft[4] - e_u)[m]
    m = s < 0.0
    x2[m] = (top[5] - left[4] - e_c)[m]
    m = s == 0.0
    x2[m] = (top[5] - 0.5 * (left[4] + uleft[4] + e_c + e_u))[m]

    y1 = np.zeros(shape)
    s = uleft[0]
    m = s > 0.0
    y1[m] = (-uleft[4] + ltop[5] - e_ul)[m]
    m = s < 0.0
    y1[m] = (-uleft[4] + top[5] - e_u)[m]
    m = s == 0.0
    y1[m] = (-uleft[4] + 0.5 * (ltop[5] + top[5] - e_ul - e_u))[m]

    y2 = np.zeros(shape)
    s = left[0]
    m = s > 0.0
    y2[m] = (-left[4] + ltop[5] - e_l)[m]
    m = s < 0.0
    y2[m] = (-left[4] + top[5] - e_c)[m]
    m = s == 0.0
    y2[m] = (-left[4] + 0.5 * (ltop[5] + top[5] - e_l - e_c))[m]

    return 0.25 * (x1 + x2 + y1 + y2)


# ----------------------------------------------------------------------------
# CTU transverse corrections (Source/CTU_HelperModule.py:282-360, :366-444)
# ----------------------------------------------------------------------------
def x_transverse(wx, wy, fy, fbx, dt, dx, dy, bcx):
    """(2, 7, Ny, Nx+1) corrections for the left/right x-face cons states."""
    inv_dx = 1.0 / dx
    half_dtdy = 0.5 * (dt / dy)
    half_dt = 0.5 * dt
    Ny, Nx = wx.shape[1:]
    k = np.arange(Nx + 2)                       # padded cells -1 .. Nx
    cell = wrap_index(k - 1, Nx, bcx)
    if bcx == OUTFLOW:
        lb = take_x(fbx, np.clip(k - 1, 0, Nx))
        rb = take_x(fbx, np.clip(k, 0, Nx))
    else:
        lb = take_x(fbx, np.where(k == 0, Nx - 1, k - 1))
        rb = take_x(fbx, np.where(k == Nx + 1, 1, k))
    dB = rb - lb
    cbx = take_x(wy[5], cell)
    cby = take_x(wx[4], cell)
    cbz = take_x(wx[5], cell)
    cvz = take_x(wx[3], cell)
    zeros = np.zeros_like(cbx)
    src = np.array([zeros,
                    cbx * dB * inv_dx,
                    cby * dB * inv_dx,
                    cbz * dB * inv_dx,
                    zeros,
                    cvz * dB * inv_dx,
                    cbz * cvz * dB * inv_dx])
    tf = fy[:, :-1, :]
    bf = fy[:, 1:, :]
    f = np.arange(Nx + 1)
    out = np.empty((2, 7, Ny, Nx + 1))
    for side, cidx in ((0, wrap_index(f - 1, Nx, bcx)), (1, wrap_index(f, Nx, bcx))):
        t = take_x(tf, cidx).copy()
        b = take_x(bf, cidx).copy()
        t[5] = t[4]
        t[4] = 0.0
        b[5] = b[4]
        b[4] = 0.0
        s = src[..., side:side + Nx + 1]
        out[side] = -half_dtdy * (b - t) + half_dt * s
    return out


def y_transverse(wx, wy, fx, fby, dt, dx, dy, bcy):
    """(2, 7, Ny+1, Nx) corrections for the top/bottom y-face cons states."""
    inv_dy = 1.0 / dy
    half_dtdx = 0.5 * (dt / dx)
    half_dt = 0.5 * dt
    Ny, Nx = wx.shape[1:]
    k = np.arange(Ny + 2)
    if bcy == OUTFLOW:
        # the reference pads the top with row 1, not row 0 (CTU_HelperModule.py:378-387)
        cell = np.where(k == 0, 1 if Ny > 1 else 0, np.clip(k - 1, 0, Ny - 1))
        tb = take_y(fby, np.where(k == 0, 1, k - 1))
        bb = take_y(fby, np.where(k == Ny + 1, Ny - 1, k))
    else:
        cell = wrap_index(k - 1, Ny, bcy)
        tb = take_y(fby, np.where(k == 0, Ny - 1, k - 1))
        bb = take_y(fby, np.where(k == Ny + 1, 1, k))
    dB = bb - tb
    cbx = take_y(wy[5], cell)
    cby = take_y(wx[4], cell)
    cbz = take_y(wx[5], cell)
    cvz = take_y(wx[3], cell)
    zeros = np.zeros_like(cbx)
    src = np.array([zeros,
                    cbx * dB * inv_dy,
                    cby * dB * inv_dy,
                    cbz * dB * inv_dy,
                    cvz * dB * inv_dy,
                    zeros,
                    (cbz * cvz) * dB * inv_dy])
    lf = fx[:, :, :-1]
    rf = fx[:, :, 1:]
    f = np.arange(Ny + 1)
    out = np.empty((2, 7, Ny + 1, Nx))
    for side, cidx in ((0, wrap_index(f - 1, Ny, bcy)), (1, wrap_index(f, Ny, bcy))):
        l_ = take_y(lf, cidx).copy()
        r_ = take_y(rf, cidx).copy()
        l_[4] = l_[5]
        l_[5] = 0.0
        r_[4] = r_[5]
        r_[5] = 0.0
        s = src[:, side:side + Ny + 1, :]
        out[side] = -half_dtdx * (r_ - l_) + half_dt * s
    return out


# ----------------------------------------------------------------------------
# One cycle and the evolve loop (Source/EvolveFunctions_MHD.py:393-697)
# ----------------------------------------------------------------------------
def cycle(prim, cons, fbx, fby, dt, dx, dy, bcx, bcy, gamma, min_d, min_p, min_e,
          order, efix, eps, trace=None):
    """Advance (prim, cons, faceBx, faceBy) by one cycle of size dt.

    order: 0 first order, 1 PLM (no reference counterpart), 2 PPM.
    Returns new (prim8, cons8, faceBx, faceBy); inputs are not modified.
    ``trace`` (a dict) receives the stage intermediates when given.
    """
    wx = np.array([prim[0], prim[1], prim[2], prim[3], prim[5], prim[6], prim[7]])
    wy = np.array([prim[0], prim[1], prim[2], prim[3], prim[6], prim[4], prim[7]])
    ux = np.array([cons[0], cons[1], cons[2], cons[3], cons[5], cons[6], cons[7]])
    half_dtdx = 0.5 * (dt / dx)
    half_dtdy = 0.5 * (dt / dy)

    if order in (1, 2):
        lin = order == 1
        xl, xr = ppm_sweep(wx, wy[5], gamma, dt, dx, bcx, FRAME_X, linear=lin)
        tl, tr = ppm_sweep(swap_xy(wy), swap_xy(wx[4]), gamma, dt, dy, bcy, FRAME_Y, linear=lin)
        yl, yr = swap_xy(tl), swap_xy(tr)
    else:
        xl, xr = first_order_sweep(wx, bcx)
        tl, tr = first_order_sweep(swap_xy(wy), bcy)
        yl, yr = swap_xy(tl), swap_xy(tr)
    for a in (xl, xr, yl, yr):
        apply_floors_inplace(a, min_d, min_p)

    byc = by_source_terms(wx[2], fbx, dt, dx, bcx)
    xl[4] += byc[0]
    xr[4] += byc[1]
    uxl = prim_to_cons7(xl, fbx, gamma)
    uxr = prim_to_cons7(xr, fbx, gamma)
    bxc = bx_source_terms(wx[1], fby, dt, dy, bcy)
    yl[5] += bxc[0]
    yr[5] += bxc[1]
    uyl = prim_to_cons7(yl, fby, gamma)
    uyr = prim_to_cons7(yr, fby, gamma)
    if trace is not None:
        trace.update(xl=xl.copy(), xr=xr.copy(), yl=yl.copy(), yr=yr.copy())

    ez = wx[2] * wy[5] - wx[1] * wx[4]
    fx = roe_flux(xl, xr, uxl, uxr, fbx, gamma, efix, eps, FRAME_X)
    fy = roe_flux(yl, yr, uyl, uyr, fby, gamma, efix, eps, FRAME_Y)
    emf = corner_emf(fx, fy, ez, bcx, bcy)
    if trace is not None:
        trace.update(fx1=fx.copy(), fy1=fy.copy(), emf1=emf.copy())

    hx = x_transverse(wx, wy, fy, fbx, dt, dx, dy, bcx)
    uxl += hx[0]
    uxr += hx[1]
    apply_floors_inplace(uxl, min_d, min_e)
    apply_floors_inplace(uxr, min_d, min_e)
    hy = y_transverse(wx, wy, fx, fby, dt, dx, dy, bcy)
    uyl += hy[0]
    uyr += hy[1]
    apply_floors_inplace(uyl, min_d, min_e)
    apply_floors_inplace(uyr, min_d, min_e)

    nfbx = fbx - half_dtdy * (emf[1:, :] - emf[:-1, :])
    nfby = fby + half_dtdx * (emf[:, 1:] - emf[:, :-1])
    xl = cons_to_prim7(uxl, nfbx, gamma)
    xr = cons_to_prim7(uxr, nfbx, gamma)
    yl = cons_to_prim7(uyl, nfby, gamma)
    yr = cons_to_prim7(uyr, nfby, gamma)

    # half-step cell state (only rho, mx, my are used downstream)
    fxr = fx.copy()
    fyr = fy.copy()
    fyr[5] = fyr[4]
    fyr[4] = 0.0
    fxr[4] = 0.0
    hu = ux - half_dtdx * (fxr[:, :, 1:] - fxr[:, :, :-1])
    hu -= half_dtdy * (fyr[:, 1:, :] - fyr[:, :-1, :])
    hbx = (nfbx[:, :-1] + nfbx[:, 1:]) / 2.0
    hby = (nfby[:-1, :] + nfby[1:, :]) / 2.0
    hvx = hu[1] / hu[0]
    hvy = hu[2] / hu[0]
    hez = hvy * hbx - hvx * hby
    if trace is not None:
        trace.update(uxl=uxl.copy(), uxr=uxr.copy(), uyl=uyl.copy(), uyr=uyr.copy(),
                     nfbx=nfbx.copy(), nfby=nfby.copy(), hez=hez.copy())

    fx2 = roe_flux(xl, xr, uxl, uxr, nfbx, gamma, efix, eps, FRAME_X)
    fy2 = roe_flux(yl, yr, uyl, uyr, nfby, gamma, efix, eps, FRAME_Y)
    emf2 = corner_emf(fx2, fy2, hez, bcx, bcy)
    if trace is not None:
        trace.update(fx2=fx2.copy(), fy2=fy2.copy(), emf2=emf2.copy())

    ofbx = fbx - (dt / dy) * (emf2[1:, :] - emf2[:-1, :])
    ofby = fby + (dt / dx) * (emf2[:, 1:] - emf2[:, :-1])
    cbx = (ofbx[:, :-1] + ofbx[:, 1:]) / 2.0
    cby = (ofby[:-1, :] + ofby[1:, :]) / 2.0
    lfl = fx2[:, :, :-1]
    rfl = fx2[:, :, 1:]
    tfl = fy2[:, :-1, :]
    bfl = fy2[:, 1:, :]
    new_bz = ux[5] - (dt / dx) * (rfl[5] - lfl[5]) - (dt / dy) * (bfl[4] - tfl[4])
    nu = ux - (dt / dx) * (rfl - lfl)
    nu -= (dt / dy) * (bfl - tfl)
    nu[5] = new_bz
    nu[4] = cby
    nw = cons_to_prim7(nu, cbx, gamma)
    prim_out = np.array([nw[0], nw[1], nw[2], nw[3], cbx, nw[4], nw[5], nw[6]])
    cons_out = np.array([nu[0], nu[1], nu[2], nu[3], cbx, nu[4], nu[5], nu[6]])
    return prim_out, cons_out, ofbx, ofby


def evolve(prim, cons, fbx, fby, dx, dy, bcx, bcy, t_start, t_end, start_cycle, max_cycles,
           gamma, cfl, min_d, min_p, min_e, order=0, efix=False, eps=0.5, dt_log=None):
    """The evolve_2D_mhd loop (Source/EvolveFunctions_MHD.py:464-697), same 11-tuple."""
    prim = np.asarray(prim, dtype=np.float64)
    cons = np.asarray(cons, dtype=np.float64)
    fbx = np.array(fbx, dtype=np.float64)
    fby = np.array(fby, dtype=np.float64)
    t = t_start
    cyc = start_cycle
    sl = (prim.copy(), cons.copy(), fbx.copy(), fby.copy(), t_start)
    while t < t_end and cyc < max_cycles:
        sl = (prim.copy(), cons.copy(), fbx.copy(), fby.copy(), t)
        dt = calc_dt(cons, fbx, fby, gamma, cfl, dx, dy)
        if t + dt > t_end:
            dt = t_end - t
        if dt_log is not None:
            dt_log.append(dt)
        prim, cons, fbx, fby = cycle(prim, cons, fbx, fby, dt, dx, dy, bcx, bcy, gamma,
                                     min_d, min_p, min_e, order, efix, eps)
        t += dt
        cyc += 1
    return (prim, cons, fbx, fby, t, cyc) + sl
