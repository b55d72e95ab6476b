"""CPU oracle: one 3D CTU+CT cycle of ideal MHD (evolve_3D_mhd), restated in NumPy.

TEST INFRASTRUCTURE ONLY (see ``oracle/common.py``).  Arrays have the reference's
3D layout: prim/cons (8, ny, nx, nz), faceBx (ny, nx+1, nz), faceBy (ny+1, nx, nz),
faceBz (ny, nx, nz+1); z is the fastest axis.

The cycle follows Source/EvolveFunctions_MHD.py:750-1157:
* sweep vectors [rho, v, B_t1, B_t2, p] per direction (x: By, Bz; y: Bz, Bx;
  z: Bx, By); the reconstruction, eigensystem and Roe solver in z are the x
  routines relabelled to the frame (vz, vx, vy), so ``oracle.mhd2d``'s
  frame-generic routines serve all three directions;
* the reconstructed transverse B gets the 3D source corrections
  (Source/Reconstruction_PPM_MHD_HelperModule.py:1351-1824);
* face states convert with direction-ordered kinetic sums (Source/PrimCons_HelperModule.py:232-468);
* three edge EMF components (Source/CornerEMF_HelperModule.py:546-951), the 3D
  transverse predictor (Source/CTU_HelperModule.py:451-1078), a half-step CT
  update of the three face-B arrays and of the cell E field, stage-2 fluxes and
  EMFs, the full CT update and the conservative update.

Where the reference computes in ``np.longdouble`` (the y terms of the x
predictor, Source/CTU_HelperModule.py:455) this restatement does too, so it
reproduces the reference on the machine it runs on.  The reference's own quirks
are kept: the first-order z padding and the z B corrections use BcX
(Source/EvolveFunctions_MHD.py:867, :921-922); the y B correction zeroes the z term
when dBz == 0 (:1606-1615).
"""
from __future__ import annotations

import numpy as np

from . import mhd2d
from .common import OUTFLOW, SMALL_VALUE, Frame, apply_floors_inplace, wrap_index

FRAMES = {0: Frame(1, 2, 3), 1: Frame(2, 3, 1), 2: Frame(3, 1, 2)}
# prim8 slots of each direction's sweep vector
SWEEP = {0: [0, 1, 2, 3, 5, 6, 7], 1: [0, 1, 2, 3, 6, 4, 7], 2: [0, 1, 2, 3, 4, 5, 7]}
# axis of direction d in a (ny, nx, nz) field, and in an (nvars, ny, nx, nz) stack
FAX = {0: 1, 1: 0, 2: 2}
VAX = {0: 2, 1: 1, 2: 3}


def _take(a, ax, idx):
    return np.take(a, idx, axis=ax)


def calc_dt(cons, fbx, fby, fbz, gamma, cfl, dx, dy, dz):
    """calcDt_3D_mhd (Source/TimestepCalculations_HelperModule.py:305-361)."""
    g1 = gamma - 1.0
    inv_d = 1.0 / cons[0]
    vx = cons[1] * inv_d
    vy = cons[2] * inv_d
    vz = cons[3] * inv_d
    vsq = vx * vx + vy * vy + vz * vz
    bx = cons[4] + np.abs(fbx[:, :-1, :] - cons[4])
    by = cons[5] + np.abs(fby[:-1, :, :] - cons[5])
    bz = cons[6] + np.abs(fbz[:, :, :-1] - cons[6])
    bsq = bx * bx + by * by + bz * bz
    p = np.maximum(g1 * (cons[7] - 0.5 * cons[0] * vsq - 0.5 * bsq), SMALL_VALUE)
    a2 = gamma * p * inv_d
    ssum = bsq * inv_d + a2
    sdiff = bsq * inv_d - a2
    cfx = 0.5 * (ssum + np.sqrt(sdiff * sdiff + 4.0 * a2 * (by * by + bz * bz) * inv_d))
    cfy = 0.5 * (ssum + np.sqrt(sdiff * sdiff + 4.0 * a2 * (bx * bx + bz * bz) * inv_d))
    cfz = 0.5 * (ssum + np.sqrt(sdiff * sdiff + 4.0 * a2 * (bx * bx + by * by) * inv_d))
    mx = np.max(np.abs(vx) + np.sqrt(cfx))
    my = np.max(np.abs(vy) + np.sqrt(cfy))
    mz = np.max(np.abs(vz) + np.sqrt(cfz))
    inv = np.maximum(mx / dx, np.maximum(my / dy, mz / dz))
    return cfl / inv


def prim_to_cons_dir(w, bn, gamma, fr):
    """primToCons_mhd_x / _y / _z: the kinetic sum in the order (n, t1, t2)."""
    u = np.empty_like(w)
    u[0] = w[0]
    u[1] = w[0] * w[1]
    u[2] = w[0] * w[2]
    u[3] = w[0] * w[3]
    u[4] = w[4]
    u[5] = w[5]
    u[6] = w[6] / (gamma - 1.0) + 0.5 * w[0] * (w[fr.n] * w[fr.n] + w[fr.t1] * w[fr.t1] + w[fr.t2] * w[fr.t2])
    u[6] += 0.5 * (bn * bn + w[4] * w[4] + w[5] * w[5])
    return u


def cons_to_prim_dir(u, bn, gamma, fr):
    """consToPrim_mhd_x / _y / _z."""
    w = np.empty_like(u)
    inv_d = 1.0 / u[0]
    w[0] = u[0]
    w[1] = u[1] * inv_d
    w[2] = u[2] * inv_d
    w[3] = u[3] * inv_d
    w[4] = u[4]
    w[5] = u[5]
    w[6] = u[6] - 0.5 * (u[fr.n] * u[fr.n] + u[fr.t1] * u[fr.t1] + u[fr.t2] * u[fr.t2]) * inv_d
    w[6] -= 0.5 * (bn * bn + w[4] * w[4] + w[5] * w[5])
    w[6] *= (gamma - 1.0)
    return w


def edge_states(w, bn, gamma, dt, dn, bc, d, order):
    """Face states along direction d of the sweep vector ``w`` (7, ny, nx, nz):
    PPM for order 2 (Source/Reconstruction_PPM_MHD_HelperModule.py:189-1177), PLM for
    the added order 1, else the first-order copy (Source/EvolveFunctions_MHD.py:846-884)."""
    ax = VAX[d]
    wm = np.ascontiguousarray(np.moveaxis(w, ax, -1))
    if order in (1, 2):
        bm = np.ascontiguousarray(np.moveaxis(bn, FAX[d], -1))
        lo, hi = mhd2d.ppm_sweep(wm, bm, gamma, dt, dn, bc, FRAMES[d], linear=order == 1)
    else:
        lo, hi = mhd2d.first_order_sweep(wm, bc)
    return np.moveaxis(lo, -1, ax), np.moveaxis(hi, -1, ax)


def _normal_ghost_change(fb, d, n, bc, inv):
    """(fb[c+1] - fb[c]) * inv over the sweep-extended cells c = -1..n of direction d,
    with the reference's ghost faces: outflow repeats the end faces (a zero change),
    periodic takes faces n-1 and 1."""
    ax = FAX[d]
    if bc == OUTFLOW:
        idx = np.concatenate([[0], np.arange(n + 1), [n]])
    else:
        idx = np.concatenate([[n - 1], np.arange(n + 1), [1]])
    e = _take(fb, ax, idx)
    return (_take(e, ax, np.arange(1, n + 3)) - _take(e, ax, np.arange(0, n + 2))) * inv


def _ext_cells(a, d, n, bc):
    """A cell field over the sweep-extended cells -1..n of direction d."""
    return _take(a, FAX[d], wrap_index(np.arange(-1, n + 1), n, bc))


def _own_change(fb, e, h, divide):
    """(fb[hi] - fb[lo]) along direction e of a face array, per cell, times ``h``
    (an inverse spacing) or, with ``divide``, divided by ``h`` (a spacing)."""
    ax = FAX[e]
    m = fb.shape[ax] - 1
    diff = _take(fb, ax, np.arange(1, m + 1)) - _take(fb, ax, np.arange(0, m))
    return diff / h if divide else diff * h


def _limit(nch, tch, zero_when_t_zero=False):
    """The B-correction change term: ``nch`` the normal change, ``tch`` a transverse one
    (Source/Reconstruction_PPM_MHD_HelperModule.py:1405-1425)."""
    r = np.zeros_like(nch)
    pos = nch >= 0.0
    neg = ~pos
    less = nch < -tch
    more = nch > -tch
    m = pos & less
    r[m] = nch[m]
    m = pos & ~less
    r[m] = -tch[m]
    if zero_when_t_zero:
        r[m & (tch == 0.0)] = 0.0
    r[pos & (r < 0.0)] = 0.0
    m = neg & more
    r[m] = nch[m]
    m = neg & ~more
    r[m] = -tch[m]
    if zero_when_t_zero:
        r[m & (tch == 0.0)] = 0.0
    r[neg & (r > 0.0)] = 0.0
    return r


def b_corrections(d, prim, cons, fb, dt, dn, bc):
    """The half-dt corrections of the reconstructed transverse B of direction d
    (getReconBCorrectionsX/Y/Z_3D, Source/Reconstruction_PPM_MHD_HelperModule.py:1351-1434,
    :1543-1628, :1743-1824).  Returns [[slot-4 minus, slot-4 plus], [slot-5 minus,
    slot-5 plus]] at the faces of direction d."""
    n = {0: prim.shape[2], 1: prim.shape[1], 2: prim.shape[3]}
    fr = FRAMES[d]
    inv = [1.0 / h for h in dn]
    nch = _normal_ghost_change(fb[d], d, n[d], bc, inv[d])
    out = []
    for slot, e in ((4, fr.t1 - 1), (5, fr.t2 - 1)):
        tch = _ext_cells(_own_change(fb[e], e, inv[e], False), d, n[d], bc)
        v = _ext_cells(cons[1 + e] / prim[0], d, n[d], bc)
        term = _limit(nch, tch, zero_when_t_zero=(d == 1 and slot == 4))
        src = 0.5 * dt * (v * term)
        ax = FAX[d]
        out.append([_take(src, ax, np.arange(0, n[d] + 1)), _take(src, ax, np.arange(1, n[d] + 2))])
    return out


def _upwind(s, pos, neg, zero):
    r = np.zeros_like(s)
    m = s > 0.0
    r[m] = pos[m]
    m = s < 0.0
    r[m] = neg[m]
    m = s == 0.0
    r[m] = zero[m]
    return r


def _gather(a, axes_idx):
    """a[..., idx_y, idx_x, idx_z] by successive takes over the given (axis, index) pairs."""
    for ax, idx in axes_idx:
        a = np.take(a, idx, axis=ax)
    return a


def corner_emfs(fx, fy, fz, ex, ey, ez, n, bcs):
    """The three edge EMF components on the (ny+1, nx+1, nz+1) edge grid
    (getXCornerEMF_3D / getYCornerEMF_3D / getZCornerEMF_3D,
    Source/CornerEMF_HelperModule.py:546-951).  Fluxes are 7-vectors (7, ...) in
    their sweep order; ex/ey/ez cell fields; n = (nx, ny, nz); bcs = (bcx, bcy, bcz)."""
    nx, ny, nz = n
    bx_, by_, bz_ = bcs
    I, J, K = np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1)
    wI, wI1 = wrap_index(I, nx, bx_), wrap_index(I - 1, nx, bx_)
    wJ, wJ1 = wrap_index(J, ny, by_), wrap_index(J - 1, ny, by_)
    wK, wK1 = wrap_index(K, nz, bz_), wrap_index(K - 1, nz, bz_)

    # z component: edges at (y-corner J, x-corner I, z-cell K)
    tF = _gather(fy, [(2, wI), (3, wK)])
    ltF = _gather(fy, [(2, wI1), (3, wK)])
    lF = _gather(fx, [(1, wJ), (3, wK)])
    ulF = _gather(fx, [(1, wJ1), (3, wK)])
    cE = _gather(ez, [(0, wJ), (1, wI), (2, wK)])
    lE = _gather(ez, [(0, wJ), (1, wI1), (2, wK)])
    uE = _gather(ez, [(0, wJ1), (1, wI), (2, wK)])
    ulE = _gather(ez, [(0, wJ1), (1, wI1), (2, wK)])
    x1 = _upwind(ltF[0], -ulF[4] - ulE, -lF[4] - lE, -0.5 * (lF[4] + ulF[4] + lE + ulE))
    x2 = _upwind(tF[0], -ulF[4] - uE, -lF[4] - cE, -0.5 * (lF[4] + ulF[4] + cE + uE))
    y1 = _upwind(ulF[0], ltF[5] - ulE, tF[5] - uE, 0.5 * (ltF[5] + tF[5] - ulE - uE))
    y2 = _upwind(lF[0], ltF[5] - lE, tF[5] - cE, 0.5 * (ltF[5] + tF[5] - lE - cE))
    emf_z = 0.25 * (ltF[5] + tF[5] - ulF[4] - lF[4] + x1 + x2 + y1 + y2)

    # x component: edges at (y-corner J, x-cell I, z-corner K)
    bF = _gather(fz, [(2, wI), (1, wJ)])
    ubF = _gather(fz, [(2, wI), (1, wJ1)])
    tF = _gather(fy, [(2, wI), (3, wK)])
    btF = _gather(fy, [(2, wI), (3, wK1)])
    cE = _gather(ex, [(0, wJ), (1, wI), (2, wK)])
    bE = _gather(ex, [(0, wJ), (1, wI), (2, wK1)])
    uE = _gather(ex, [(0, wJ1), (1, wI), (2, wK)])
    ubE = _gather(ex, [(0, wJ1), (1, wI), (2, wK1)])
    z1 = _upwind(btF[0], ubF[5] - ubE, bF[5] - bE, 0.5 * (ubF[5] + bF[5] - ubE - bE))
    z2 = _upwind(tF[0], ubF[5] - uE, bF[5] - cE, 0.5 * (ubF[5] + bF[5] - uE - cE))
    y1 = _upwind(ubF[0], -btF[4] - ubE, -tF[4] - uE, 0.5 * (-btF[4] - tF[4] - ubE - uE))
    y2 = _upwind(bF[0], -btF[4] - bE, -tF[4] - cE, 0.5 * (-btF[4] - tF[4] - bE - cE))
    emf_x = 0.25 * (bF[5] + ubF[5] - tF[4] - btF[4] + y1 + y2 + z1 + z2)

    # y component: edges at (y-cell J, x-corner I, z-corner K)
    bF = _gather(fz, [(1, wJ), (2, wI)])
    lbF = _gather(fz, [(1, wJ), (2, wI1)])
    lF = _gather(fx, [(1, wJ), (3, wK)])
    blF = _gather(fx, [(1, wJ), (3, wK1)])
    cE = _gather(ey, [(0, wJ), (1, wI), (2, wK)])
    bE = _gather(ey, [(0, wJ), (1, wI), (2, wK1)])
    lE = _gather(ey, [(0, wJ), (1, wI1), (2, wK)])
    blE = _gather(ey, [(0, wJ), (1, wI1), (2, wK1)])
    z1 = _upwind(blF[0], -lbF[4] - blE, -bF[4] - bE, 0.5 * (-lbF[4] - bF[4] - blE - bE))
    z2 = _upwind(lF[0], -lbF[4] - lE, -bF[4] - cE, 0.5 * (-lbF[4] - bF[4] - lE - cE))
    x1 = _upwind(lbF[0], blF[5] - blE, lF[5] - lE, 0.5 * (blF[5] + lF[5] - blE - lE))
    x2 = _upwind(bF[0], blF[5] - bE, lF[5] - cE, 0.5 * (blF[5] + lF[5] - bE - cE))
    emf_y = 0.25 * (lF[5] + blF[5] - bF[4] - lbF[4] + x1 + x2 + z1 + z2)
    return emf_x, emf_y, emf_z


def _minmod(nch, tch):
    """The predictor's source-term limiter (Source/CTU_HelperModule.py:624-651)."""
    r = np.zeros_like(nch)
    for m, val in (((nch > 0.0) & (tch < 0.0) & (tch > -nch), tch), ((nch > 0.0) & (tch < 0.0) & (tch <= -nch), -nch),
                   ((nch < 0.0) & (tch > 0.0) & (tch < -nch), tch), ((nch < 0.0) & (tch > 0.0) & (tch >= -nch), -nch)):
        r[m] = val[m]
    return r


# predictor steps of each direction: (transverse direction, B slot its EMF term
# updates, sign of that update); the x predictor's y terms are in np.longdouble
STEPS = {0: ((1, 5, 1.0), (2, 4, -1.0)), 1: ((0, 4, -1.0), (2, 5, 1.0)), 2: ((0, 5, 1.0), (1, 4, -1.0))}


def transverse(d, u_sides, prim, fluxes, fb, emf, dt, dn, bc, long_double=True):
    """getXTransverseUpdates_3D / Y / Z (Source/CTU_HelperModule.py:451-1078): the
    face states of direction d (conserved, [minus, plus]) take, per transverse
    direction, the half-dt flux difference at their cell (B slots zeroed) and the
    EMF term of the edge EMF parallel to d, then the source vector of their
    (sweep-extended) cell.  Returns new [minus, plus].  ``long_double=False`` computes
    the x predictor's y terms in float64, as the CUDA step does."""
    n = {0: prim.shape[2], 1: prim.shape[1], 2: prim.shape[3]}
    L = n[d]
    ax = FAX[d]
    out = []
    for side, u in enumerate(u_sides):
        u = u.copy()
        cells = wrap_index(np.arange(L + 1) - 1 + side, L, bc)
        for e, slot, sign in STEPS[d]:
            o = 3 - d - e
            fe = np.take(fluxes[e], cells, axis=VAX[d]).copy()
            fe[4] = 0.0
            fe[5] = 0.0
            m = fe.shape[VAX[e]] - 1
            diff = np.take(fe, np.arange(1, m + 1), axis=VAX[e]) - np.take(fe, np.arange(0, m), axis=VAX[e])
            half = 0.5 * (dt / dn[e])
            ed = np.take(emf, cells, axis=ax)
            ne, no = ed.shape[FAX[e]] - 1, ed.shape[FAX[o]] - 1

            def at(eh, oh):
                a = np.take(ed, np.arange(eh, ne + eh), axis=FAX[e])
                return np.take(a, np.arange(oh, no + oh), axis=FAX[o])
            delta = ((at(1, 0) - at(0, 0)) + at(1, 1)) - at(0, 1)
            if d == 0 and e == 1 and long_double:
                half_ld = 0.5 * (np.longdouble(dt) / np.longdouble(dn[e]))
                u = (u.astype(np.longdouble) - half_ld * diff).astype(np.float64)
                upd = (half_ld * 0.5) * delta
                u[slot] = (u[slot].astype(np.longdouble) + sign * upd).astype(np.float64) if sign > 0 else \
                    (u[slot].astype(np.longdouble) - upd).astype(np.float64)
            else:
                u = u - half * diff
                upd = (half * 0.5) * delta
                u[slot] = u[slot] + upd if sign > 0 else u[slot] - upd
        out.append(u)
    # source vector over the sweep-extended cells (x: products with 1/dn; y, z: quotients by dn)
    divide = d != 0
    fr = FRAMES[d]
    a, b = fr.t1 - 1, fr.t2 - 1
    if divide:
        # the z predictor's outflow ghost above the last cell takes face nz-1
        # (Source/CTU_HelperModule.py:918-920 index faceBz with faceBy's z extent)
        nch = _normal_ghost_div(fb[d], d, L, bc, dn[d], hi_face=L - 1 if d == 2 else L)
    else:
        nch = _normal_ghost_change(fb[d], d, L, bc, 1.0 / dn[d])
    ta = _ext_cells(_own_change(fb[a], a, dn[a] if divide else 1.0 / dn[a], divide), d, L, bc)
    tb = _ext_cells(_own_change(fb[b], b, dn[b] if divide else 1.0 / dn[b], divide), d, L, bc)
    cell = {k: _ext_cells(prim[k], d, L, bc) for k in range(1, 7)}
    hdt = 0.5 * dt
    mmb, mma = _minmod(nch, tb), _minmod(nch, ta)
    va, vb = cell[1 + a], cell[1 + b]
    ba, bb = cell[4 + a], cell[4 + b]
    src = [np.zeros_like(nch), hdt * cell[4] * nch, hdt * cell[5] * nch, hdt * cell[6] * nch,
           hdt * va * (-mmb), hdt * vb * (-mma), hdt * (ba * va * (-mmb) + bb * vb * (-mma))]
    src = np.array(src)
    lo = np.take(src, np.arange(0, L + 1), axis=VAX[d])
    hi = np.take(src, np.arange(1, L + 2), axis=VAX[d])
    return [out[0] + lo, out[1] + hi]


def _normal_ghost_div(fb, d, n, bc, h, hi_face):
    """_normal_ghost_change with the difference divided by the spacing ``h``; the
    outflow ghost above the last cell takes face ``hi_face``."""
    ax = FAX[d]
    if bc == OUTFLOW:
        idx = np.concatenate([[0], np.arange(n + 1), [hi_face]])
    else:
        idx = np.concatenate([[n - 1], np.arange(n + 1), [1]])
    e = _take(fb, ax, idx)
    return (_take(e, ax, np.arange(1, n + 3)) - _take(e, ax, np.arange(0, n + 2))) / h


def cycle(prim, cons, fbx, fby, fbz, dt, dx, dy, dz, bcx, bcy, bcz, gamma, min_d, min_p, min_e, order, efix, eps,
          long_double=True):
    """One cycle of evolve_3D_mhd (Source/EvolveFunctions_MHD.py:819-1152).
    Returns new (prim, cons, faceBx, faceBy, faceBz); the inputs are not modified."""
    ny, nx, nz = prim.shape[1:]
    fb = (fbx, fby, fbz)
    dn = (dx, dy, dz)
    bcs = (bcx, bcy, bcz)
    bn_cell = {0: prim[4], 1: prim[5], 2: prim[6]}
    rec_bc = {0: bcx, 1: bcy, 2: bcz if order in (1, 2) else bcx}
    corr_bc = {0: bcx, 1: bcy, 2: bcx}
    wf = {}
    for d in range(3):
        lo, hi = edge_states(prim[SWEEP[d]], bn_cell[d], gamma, dt, dn[d], rec_bc[d], d, order)
        wf[d] = [apply_floors_inplace(np.array(lo), min_d, min_p), apply_floors_inplace(np.array(hi), min_d, min_p)]
    uf = {}
    for d in range(3):
        c = b_corrections(d, prim, cons, fb, dt, dn, corr_bc[d])
        for side in range(2):
            wf[d][side][4] += c[0][side]
            wf[d][side][5] += c[1][side]
        uf[d] = [prim_to_cons_dir(s, fb[d], gamma, FRAMES[d]) for s in wf[d]]
    ex = (prim[5] * cons[3] - prim[6] * cons[2]) / cons[0]
    ey = (prim[6] * cons[1] - prim[4] * cons[3]) / cons[0]
    ez = (prim[4] * cons[2] - prim[5] * cons[1]) / cons[0]
    f1 = [mhd2d.roe_flux(wf[d][0], wf[d][1], uf[d][0], uf[d][1], fb[d], gamma, efix, eps, FRAMES[d]) for d in range(3)]
    e1 = corner_emfs(f1[0], f1[1], f1[2], ex, ey, ez, (nx, ny, nz), bcs)
    for d in range(3):
        uf[d] = transverse(d, uf[d], prim, f1, fb, e1[d], dt, dn, bcs[d], long_double)
    h = [0.5 * (dt / v) for v in dn]
    nfb = _ct(fb, e1, h, ny, nx, nz)
    wf = {d: [cons_to_prim_dir(s, nfb[d], gamma, FRAMES[d]) for s in uf[d]] for d in range(3)}
    # half-step cell state for the stage-2 cell E field (Source/EvolveFunctions_MHD.py:1038-1058)
    half = []
    for k in range(4):
        v = cons[k] - h[0] * (f1[0][k][:, 1:, :] - f1[0][k][:, :-1, :])
        v = v - h[1] * (f1[1][k][1:, :, :] - f1[1][k][:-1, :, :])
        v = v - h[2] * (f1[2][k][:, :, 1:] - f1[2][k][:, :, :-1])
        half.append(v)
    nbx = 0.5 * (nfb[0][:, :-1, :] + nfb[0][:, 1:, :])
    nby = 0.5 * (nfb[1][:-1, :, :] + nfb[1][1:, :, :])
    nbz = 0.5 * (nfb[2][:, :, :-1] + nfb[2][:, :, 1:])
    nex = (nby * half[3] - nbz * half[2]) / half[0]
    ney = (nbz * half[1] - nbx * half[3]) / half[0]
    nez = (nbx * half[2] - nby * half[1]) / half[0]
    f2 = [mhd2d.roe_flux(wf[d][0], wf[d][1], uf[d][0], uf[d][1], nfb[d], gamma, efix, eps, FRAMES[d]) for d in range(3)]
    e2 = corner_emfs(f2[0], f2[1], f2[2], nex, ney, nez, (nx, ny, nz), bcs)
    full = [dt / v for v in dn]
    ofb = _ct(fb, e2, full, ny, nx, nz)
    ux = cons[SWEEP[0]].copy()
    ux -= full[0] * (f2[0][:, :, 1:, :] - f2[0][:, :, :-1, :])
    ux -= full[1] * (f2[1][:, 1:, :, :] - f2[1][:, :-1, :, :])
    ux -= full[2] * (f2[2][:, :, :, 1:] - f2[2][:, :, :, :-1])
    cbx = 0.5 * (ofb[0][:, :-1, :] + ofb[0][:, 1:, :])
    cby = 0.5 * (ofb[1][:-1, :, :] + ofb[1][1:, :, :])
    cbz = 0.5 * (ofb[2][:, :, :-1] + ofb[2][:, :, 1:])
    ux[4] = cby
    ux[5] = cbz
    px = mhd2d.cons_to_prim7(ux, cbx, gamma)
    nprim = np.array([px[0], px[1], px[2], px[3], cbx, px[4], px[5], px[6]])
    ncons = np.array([ux[0], ux[1], ux[2], ux[3], cbx, ux[4], ux[5], ux[6]])
    return nprim, ncons, ofb[0], ofb[1], ofb[2]


def _ct(fb, emf, h, ny, nx, nz):
    """Face B after a CT update with step factors h = (dt/dx, dt/dy, dt/dz) (halved
    for the half step) from the edge EMFs (Source/EvolveFunctions_MHD.py:1005-1029)."""
    ex, ey, ez = emf
    bx = fb[0] + (h[2] * (ey[0:ny, :, 1:] - ey[0:ny, :, :-1]) - h[1] * (ez[1:, :, 0:nz] - ez[:-1, :, 0:nz]))
    by = fb[1] + (h[0] * (ez[:, 1:, 0:nz] - ez[:, :-1, 0:nz]) - h[2] * (ex[:, 0:nx, 1:] - ex[:, 0:nx, :-1]))
    bz = fb[2] + (h[1] * (ex[1:, 0:nx, :] - ex[:-1, 0:nx, :]) - h[0] * (ey[0:ny, 1:, :] - ey[0:ny, :-1, :]))
    return bx, by, bz


def evolve(prim, cons, fbx, fby, fbz, dx, dy, dz, bcx, bcy, bcz, t_start, t_end, start_cycle, max_cycles, gamma,
           cfl, min_d, min_p, min_e, order=0, efix=True, eps=0.5, dt_log=None, long_double=True):
    """The evolve_3D_mhd loop (Source/EvolveFunctions_MHD.py:750-1157); returns the
    reference's 13-tuple (prim, cons, faceBx, faceBy, faceBz, time, cycle and the
    second-last prim, cons, faceBx, faceBy, faceBz and time).  ``long_double=False``
    gives the FP64 predictor of the CUDA step (see ``transverse``)."""
    st = [np.array(a, dtype=np.float64) for a in (prim, cons, fbx, fby, fbz)]
    t = t_start
    cyc = start_cycle
    sl = tuple(a.copy() for a in st) + (t_start,)
    while t < t_end and cyc < max_cycles:
        sl = tuple(a.copy() for a in st) + (t,)
        dt = calc_dt(st[1], st[2], st[3], st[4], gamma, cfl, dx, dy, dz)
        if t_end - t < dt:
            dt = t_end - t
        if dt_log is not None:
            dt_log.append(dt)
        st = list(cycle(*st, dt, dx, dy, dz, bcx, bcy, bcz, gamma, min_d, min_p, min_e, order, efix, eps,
                        long_double))
        t += dt
        cyc += 1
    return tuple(st) + (t, cyc) + sl
