"""The pointwise functions of one MHD CTU+CT cycle, written in the SSA language
of ``dsl.py`` for reverse-mode differentiation.

Each function is the per-item computation of one forward kernel body in
``csrc/godunov2d_kernels.cuh`` / ``csrc/mhd_math.cuh`` (which cite the reference
lines), with the same operation order, so its generated forward code rounds
exactly like the forward kernels; branches are ``select``s.  Inputs and
outputs are flat lists; the stencil (which cell or face feeds which input) is
the caller's business.

Sweep vectors are in the x/y sweep orderings [rho, vx, vy, vz, B1, B2, p]
with the normal/transverse velocity slots (N, T1, T2) = (1, 2, 3) for x and
(2, 3, 1) for y.
"""
from __future__ import annotations

from .dsl import dmax, dmin, fabs, select, sqrt

SMALL_VALUE = 0.000000000001
FOUR_THIRDS = 1.333333333333333
FRAMES = {0: (1, 2, 3), 1: (2, 3, 1)}


def _sum_first(terms):
    """Sum in order starting from the first term (no leading +0)."""
    acc = terms[0]
    for t in terms[1:]:
        acc = acc + t
    return acc


def sign_one(x):
    return select(x < 0.0, -1.0, 1.0)


def signed_mag(x, m):
    return select(x > 0.0, m, select(x < 0.0, -m, 0.0))


# ---------------------------------------------------------------------------
# primitive eigensystem (mhd_math.cuh: prim_eigensystem)
# ---------------------------------------------------------------------------
EIG_BASE = 16   # words of eig_base


def eig_base(w, bn, gamma):
    """The costly part of the primitive eigensystem of one cell state: its square
    roots, divisions and signs, as the list [a2, a, ca, cf, cs, fa, sa, b1, b2, sgn,
    sqrt_d, inv_d, nf, l14, l15, l36].  ``eig_from_base`` builds lam, L and R from
    them with multiplies only, so a stage can take them as inputs from the stage that
    formed them instead of recomputing them."""
    bt2 = w[4] * w[4] + w[5] * w[5]
    bt = sqrt(bt2)
    gp = gamma * w[6]
    inv_d = 1.0 / w[0]
    sqrt_d = sqrt(w[0])
    red_bt2 = bt2 * inv_d
    a2 = gp * inv_d
    a = sqrt(a2)
    ca2 = bn * bn * inv_d
    ca = sqrt(ca2)
    ssum = ca2 + red_bt2 + a2
    sdiff = ca2 + red_bt2 - a2
    ssqrt = sqrt(sdiff * sdiff + 4.0 * a2 * red_bt2)
    cf2 = 0.5 * (ssum + ssqrt)
    cf = sqrt(cf2)
    cs2 = a2 * ca2 / cf2
    cs = sqrt(cs2)
    b1 = select(bt > 0.0, w[4] / bt, select(bt.eq(0.0), 1.0, 0.0))
    b2 = select(bt > 0.0, w[5] / bt, 0.0)
    c_f1 = ssqrt.eq(0.0)
    c_s1 = (a2 - cs2) <= 0.0
    c_f2 = (cf2 - a2) <= 0.0
    fa = select(c_f1, 1.0, select(c_s1, 0.0, select(c_f2, 1.0, sqrt((a2 - cs2) / ssqrt))))
    sa = select(c_f1, 0.0, select(c_s1, 1.0, select(c_f2, 0.0, sqrt((cf2 - a2) / ssqrt))))
    sgn = sign_one(bn)
    nf = 0.5 / a2
    l14 = -0.5 * b2 * sgn / sqrt_d
    l15 = 0.5 * b1 * sgn / sqrt_d
    l36 = -1.0 / a2
    return [a2, a, ca, cf, cs, fa, sa, b1, b2, sgn, sqrt_d, inv_d, nf, l14, l15, l36]


def eig_from_base(base, w, axis):
    """lam, L and R (mhd_math.cuh: prim_eigensystem) of the cell state w from its
    ``eig_base`` words, in the same operation order."""
    N, T1, T2 = FRAMES[axis]
    a2, a, ca, cf, cs, fa, sa, b1, b2, sgn, sqrt_d, inv_d, nf, l14, l15, l36 = base
    qf = cf * fa * sgn
    qs = cs * sa * sgn
    af = a * fa * sqrt_d
    as_ = a * sa * sqrt_d
    vn = w[N]
    lam = [vn - cf, vn - ca, vn - cs, vn, vn + cs, vn + ca, vn + cf]
    R = {}
    r00 = w[0] * fa
    r02 = w[0] * sa
    R[0, 0] = r00; R[0, 2] = r02; R[0, 3] = 1.0; R[0, 4] = r02; R[0, 6] = r00
    rn0 = -cf * fa
    rn2 = -cs * sa
    R[N, 0] = rn0; R[N, 2] = rn2; R[N, 4] = -rn2; R[N, 6] = -rn0
    qsb1 = qs * b1; qfb1 = qf * b1; qsb2 = qs * b2; qfb2 = qf * b2
    R[T1, 0] = qsb1; R[T1, 1] = -b2; R[T1, 2] = -qfb1; R[T1, 4] = qfb1; R[T1, 5] = b2; R[T1, 6] = -qsb1
    R[T2, 0] = qsb2; R[T2, 1] = b1; R[T2, 2] = -qfb2; R[T2, 4] = qfb2; R[T2, 5] = -b1; R[T2, 6] = -qsb2
    r60 = w[0] * a2 * fa
    r62 = w[0] * a2 * sa
    R[6, 0] = r60; R[6, 2] = r62; R[6, 4] = r62; R[6, 6] = r60
    r40 = as_ * b1; r41 = -b2 * sgn * sqrt_d; r42 = -af * b1
    R[4, 0] = r40; R[4, 1] = r41; R[4, 2] = r42; R[4, 4] = r42; R[4, 5] = r41; R[4, 6] = r40
    r50 = as_ * b2; r51 = b1 * sgn * sqrt_d; r52 = -af * b2
    R[5, 0] = r50; R[5, 1] = r51; R[5, 2] = r52; R[5, 4] = r52; R[5, 5] = r51; R[5, 6] = r50
    qf_n = nf * qf
    qs_n = nf * qs
    afp = nf * af * inv_d
    asp = nf * as_ * inv_d
    L = {}
    l0n = -nf * cf * fa; l0t1 = qs_n * b1; l0t2 = qs_n * b2; l06 = nf * fa * inv_d
    l04 = asp * b1; l05 = asp * b2
    L[0, N] = l0n; L[0, T1] = l0t1; L[0, T2] = l0t2; L[0, 6] = l06; L[0, 4] = l04; L[0, 5] = l05
    L[6, N] = -l0n; L[6, T1] = -l0t1; L[6, T2] = -l0t2; L[6, 6] = l06; L[6, 4] = l04; L[6, 5] = l05
    l1t1 = -0.5 * b2; l1t2 = 0.5 * b1
    L[1, T1] = l1t1; L[1, T2] = l1t2; L[1, 4] = l14; L[1, 5] = l15
    L[5, T1] = -l1t1; L[5, T2] = -l1t2; L[5, 4] = l14; L[5, 5] = l15
    l2n = -nf * cs * sa; l2t1 = -qf_n * b1; l2t2 = -qf_n * b2; l26 = nf * sa * inv_d
    l24 = -afp * b1; l25 = -afp * b2
    L[2, N] = l2n; L[2, T1] = l2t1; L[2, T2] = l2t2; L[2, 6] = l26; L[2, 4] = l24; L[2, 5] = l25
    L[4, N] = -l2n; L[4, T1] = -l2t1; L[4, T2] = -l2t2; L[4, 6] = l26; L[4, 4] = l24; L[4, 5] = l25
    L[3, 0] = 1.0
    L[3, 6] = l36
    return lam, L, R


def _order(axis):
    N, T1, T2 = FRAMES[axis]
    return (0, N, T1, T2, 6, 4, 5)


def _project(L, i, v, order):
    return _sum_first([L[i, j] * v[j] for j in order if (i, j) in L])


def char_slopes(wl, wc, wr, bn, gamma, axis):
    """The reference's limited slope of one cell (k_ppm_slopes), its eigensystem and
    the eigensystem's base words."""
    base = eig_base(wc, bn, gamma)
    lam, L, R = eig_from_base(base, wc, axis)
    order = _order(axis)
    dc = [wr[k] - wl[k] for k in range(7)]
    dl = [wc[k] - wl[k] for k in range(7)]
    dr = [wr[k] - wc[k] for k in range(7)]
    wt = [select(dl[k] * dr[k] > 0.0, (2.0 * dl[k] * dr[k]) / (dl[k] + dr[k]), 0.0) for k in range(7)]
    sc = []
    for i in range(7):
        cc = _project(L, i, dc, order)
        cl = _project(L, i, dl, order)
        cr = _project(L, i, dr, order)
        cw = _project(L, i, wt, order)
        lim1 = dmin(fabs(cl), fabs(cr))
        lim2 = dmin(0.5 * fabs(cc), fabs(cw))
        sc.append(select(cl * cr > 0.0, signed_mag(cc, dmin(2.0 * lim1, lim2)), 0.0))
    s = [_sum_first([sc[j] * R[i, j] for j in range(7) if (i, j) in R]) for i in range(7)]
    return s, lam, L, R, base


def plm_cell(ins, pars, axis):
    """PLM edge states of one cell (k_faces MODE 1), slope and eigensystem included:
    one fused stage (splitting it like PPM measured slower).

    ins = wl(7) + wc(7) + wr(7) + bn ; pars = [gamma, dtdx] -> lia(7) + ria(7)
    """
    wl, wc, wr, bn = ins[0:7], ins[7:14], ins[14:21], ins[21]
    gamma, dtdx = pars
    s, lam, L, R, _ = char_slopes(wl, wc, wr, bn, gamma, axis)
    order = _order(axis)
    lia, ria = [], []
    for k in range(7):
        a = wc[k] - 0.5 * s[k]
        b = wc[k] + 0.5 * s[k]
        a = dmax(dmin(wc[k], wl[k]), a)
        a = dmin(dmax(wc[k], wl[k]), a)
        b = dmax(dmin(wc[k], wr[k]), b)
        b = dmin(dmax(wc[k], wr[k]), b)
        lia.append(a)
        ria.append(b)
    c1 = [ria[k] - lia[k] for k in range(7)]
    c3 = 0.5 * dmax(lam[6], 0.0) * dtdx
    c4 = -0.5 * dmin(lam[0], 0.0) * dtdx
    lia = [lia[k] + c4 * c1[k] for k in range(7)]
    ria = [ria[k] - c3 * c1[k] for k in range(7)]
    for side in (0, 1):
        edge = lia if side == 0 else ria
        for i in range(7):
            active = (lam[i] <= 0.0) if side == 0 else (lam[i] >= 0.0)
            v3 = 0.5 * dtdx * lam[0 if side == 0 else 6] - 0.5 * dtdx * lam[i]
            fac = _sum_first([L[i, j] * (v3 * c1[j]) for j in order if (i, j) in L])
            for j in range(7):
                if (j, i) in R:
                    edge[j] = select(active, edge[j] + fac * R[j, i], edge[j])
    return lia + ria


def ppm_slope(ins, pars, axis):
    """Characteristic-limited primitive slope of one (sweep-extended) cell (k_ppm_slopes)
    and the base words of its eigensystem, which the PPM edge stage reads.

    ins = wl(7) + wc(7) + wr(7) + bn ; pars = [gamma] -> s(7) + base(EIG_BASE)
    """
    wl, wc, wr, bn = ins[0:7], ins[7:14], ins[14:21], ins[21]
    s, _, _, _, base = char_slopes(wl, wc, wr, bn, pars[0], axis)
    return s + base


def ppm_iface(ins, pars, axis):
    """PPM interface values of one cell with the monotonicity tests and the clamps to
    the neighbours (k_faces MODE 2, first half; oracle.mhd2d.ppm_sweep).

    ins = wl(7) + wc(7) + wr(7) + sl(7) + sc(7) + sr(7) ; pars = [gamma] -> a(7) + b(7)
    """
    wl, wc, wr = ins[0:7], ins[7:14], ins[14:21]
    sl, sc, sr = ins[21:28], ins[28:35], ins[35:42]
    lia, ria = [], []
    for k in range(7):
        a = 0.5 * (wc[k] + wl[k]) - (sc[k] - sl[k]) / 6.0
        b = 0.5 * (wr[k] + wc[k]) - (sr[k] - sc[k]) / 6.0
        dprod = (b - wc[k]) * (wc[k] - a)
        idiff = b - a
        adiff = 6.0 * (wc[k] - 0.5 * (a + b))
        nzc = dprod <= 0.0
        sq = idiff * idiff
        cl_ = ~nzc & ((idiff * adiff) > sq)
        cr_ = ~nzc & ~cl_ & ((idiff * adiff) < (-1.0 * sq))
        a2 = select(nzc, wc[k], select(cl_, (6.0 * wc[k] - 4.0 * b) / 2.0, a))
        b2 = select(nzc, wc[k], select(cr_, (6.0 * wc[k] - 4.0 * a) / 2.0, b))
        a2 = dmax(dmin(wc[k], wl[k]), a2)
        a2 = dmin(dmax(wc[k], wl[k]), a2)
        b2 = dmax(dmin(wc[k], wr[k]), b2)
        b2 = dmin(dmax(wc[k], wr[k]), b2)
        lia.append(a2)
        ria.append(b2)
    return lia + ria


def ppm_trace(ins, pars, axis):
    """dt/2 characteristic tracing of one cell's PPM edge values (k_faces MODE 2, second
    half), with the eigensystem built from the slope stage's base words.

    ins = wc(7) + a(7) + b(7) + base(EIG_BASE) ; pars = [gamma, dtdx] -> lia(7) + ria(7)
    """
    wc, lia, ria = ins[0:7], list(ins[7:14]), list(ins[14:21])
    base = ins[21:21 + EIG_BASE]
    dtdx = pars[1]
    lam, L, R = eig_from_base(base, wc, axis)
    order = _order(axis)
    c1 = [ria[k] - lia[k] for k in range(7)]
    c2 = [6.0 * (wc[k] - 0.5 * (lia[k] + ria[k])) for k in range(7)]
    c3 = 0.5 * dmax(lam[6], 0.0) * dtdx
    c4 = -0.5 * dmin(lam[0], 0.0) * dtdx
    lia = [lia[k] + c4 * (c1[k] + (1.0 - FOUR_THIRDS * c4) * c2[k]) for k in range(7)]
    ria = [ria[k] - c3 * (c1[k] - (1.0 - FOUR_THIRDS * c3) * c2[k]) for k in range(7)]
    for side in (0, 1):
        edge = lia if side == 0 else ria
        for i in range(7):
            active = (lam[i] <= 0.0) if side == 0 else (lam[i] >= 0.0)
            v1 = 0.5 * dtdx * lam[0 if side == 0 else 6]
            v2 = 0.5 * dtdx * lam[i]
            v3 = v1 - v2
            v4 = FOUR_THIRDS * (v1 * v1 - v2 * v2)
            if side == 0:
                terms = [L[i, j] * (v3 * (c1[j] + c2[j]) + v4 * c2[j]) for j in order if (i, j) in L]
            else:
                terms = [L[i, j] * (v3 * (c1[j] - c2[j]) + v4 * c2[j]) for j in order if (i, j) in L]
            fac = _sum_first(terms)
            for j in range(7):
                if (j, i) in R:
                    edge[j] = select(active, edge[j] + fac * R[j, i], edge[j])
    return lia + ria


def face_state(ins, pars, sb):
    """Floors and the transverse-B source of one reconstructed face state (put_face).

    ins = edge(7) + [vt, fb1, fb2] ; pars = [min_d, min_p, half_dt, inv_dn] -> state(7)
    """
    e = ins[0:7]
    vt, fb1, fb2 = ins[7], ins[8], ins[9]
    min_d, min_p, half_dt, inv_dn = pars
    out = []
    for k in range(7):
        x = e[k]
        if k == 0:
            x = select(x < min_d, min_d, x)
        if k == 6:
            x = select(x < min_p, min_p, x)
        if k == sb:
            x = x + half_dt * vt * ((fb2 - fb1) * inv_dn)
        out.append(x)
    return out


def prim_to_cons7(w, bn, gamma):
    u = [w[0], w[0] * w[1], w[0] * w[2], w[0] * w[3], w[4], w[5]]
    e = w[6] / (gamma - 1.0) + 0.5 * w[0] * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3])
    e = e + 0.5 * (bn * bn + w[4] * w[4] + w[5] * w[5])
    return u + [e]


def cons_to_prim7(u, bn, gamma):
    inv_d = 1.0 / u[0]
    w = [u[0], u[1] * inv_d, u[2] * inv_d, u[3] * inv_d, u[4], u[5]]
    p = u[6] - 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) * inv_d
    p = p - 0.5 * (bn * bn + w[4] * w[4] + w[5] * w[5])
    return w + [p * (gamma - 1.0)]


def _cell_flux(w, u, bn, hb, axis):
    N, T1, T2 = FRAMES[axis]
    p = w[6]
    F = [None] * 7
    F[0] = u[N]
    for k in (1, 2, 3):
        F[k] = u[N] * w[k]
    F[N] = F[N] + p
    F[6] = (u[6] + p) * w[N]
    F[N] = F[N] - 0.5 * (bn * bn - w[4] * w[4] - w[5] * w[5])
    F[T1] = F[T1] - bn * w[4]
    F[T2] = F[T2] - bn * w[5]
    F[6] = F[6] + (hb * w[N] - bn * (bn * w[N] + w[4] * w[T1] + w[5] * w[T2]))
    F[4] = w[4] * w[N] - bn * w[T1]
    F[5] = w[5] * w[N] - bn * w[T2]
    return F


def roe_flux(wl, wr, ul, ur, bn, gamma, eps, efix, axis):
    """mhd_math.cuh: roe_flux (Roe average, 7-wave L/R, entropy fix, upwind switch)."""
    N, T1, T2 = FRAMES[axis]
    sl = sqrt(wl[0])
    sr = sqrt(wr[0])
    isum = 1.0 / (sl + sr)
    rd = sl * sr
    v = {k: (sl * wl[k] + sr * wr[k]) * isum for k in (1, 2, 3)}
    vsq = v[N] * v[N] + v[T1] * v[T1] + v[T2] * v[T2]
    b1 = (sr * wl[4] + sl * wr[4]) * isum
    b2 = (sr * wl[5] + sl * wr[5]) * isum
    hbl = 0.5 * (bn * bn + wl[4] * wl[4] + wl[5] * wl[5])
    hbr = 0.5 * (bn * bn + wr[4] * wr[4] + wr[5] * wr[5])
    H = ((ul[6] + wl[6] + hbl) / sl + (ur[6] + wr[6] + hbr) / sr) * isum
    ird = 1.0 / rd
    dB1 = wl[4] - wr[4]
    dB2 = wl[5] - wr[5]
    ssl = sl + sr
    btc = 0.5 * (dB1 * dB1 + dB2 * dB2) / (ssl * ssl)
    rc = 0.5 * (wl[0] + wr[0]) / rd
    bt2 = b1 * b1 + b2 * b2
    bt = sqrt(bt2)
    bts2 = ((gamma - 1.0) - (gamma - 2.0) * rc) * bt2
    bts = sqrt(bts2)
    rbts2 = bts2 * ird
    ca2 = bn * bn * ird
    ca = sqrt(ca2)
    hmb = H - (ca2 + bt2 * ird)
    a2 = dmax((gamma - 1.0) * (hmb - 0.5 * vsq) - (gamma - 2.0) * btc, SMALL_VALUE)
    a = sqrt(a2)
    ssum = ca2 + rbts2 + a2
    sdiff = ca2 + rbts2 - a2
    ssqrt = sqrt(sdiff * sdiff + 4.0 * a2 * rbts2)
    cf2 = 0.5 * (ssum + ssqrt)
    cf = sqrt(cf2)
    cs2 = a2 * ca2 / cf2
    cs = sqrt(cs2)
    vn = v[N]
    lam = [vn - cf, vn - ca, vn - cs, vn, vn + cs, vn + ca, vn + cf]
    if efix:
        for k in range(7):
            x = lam[k]
            corr = eps + (x * x) / (4.0 * eps)
            fixed = select(x > 0.0, x + corr, x - corr)
            lam[k] = select((fabs(x) < 2.0 * eps) & ~x.eq(0.0), fixed, x)
    c_f1 = (cf2 - cs2).eq(0.0)
    c_s1 = (a2 - cs2) <= 0.0
    c_f2 = (cf2 - a2) <= 0.0
    fa = select(c_f1, 1.0, select(c_s1, 0.0, select(c_f2, 1.0, sqrt((a2 - cs2) / (cf2 - cs2)))))
    sa = select(c_f1, 0.0, select(c_s1, 1.0, select(c_f2, 0.0, sqrt((cf2 - a2) / (cf2 - cs2)))))
    sgn = sign_one(bn)
    srd = sqrt(rd)
    isrd = 1.0 / srd
    qf = cf * fa * sgn
    qs = cs * sa * sgn
    afp = a * fa * isrd
    asp = a * sa * isrd
    bh1 = select(bt > 0.0, b1 / bt, select(bt.eq(0.0), 1.0, 0.0))
    bh2 = select(bt > 0.0, b2 / bt, 0.0)
    den = sqrt((gamma - 1.0) - (gamma - 2.0) * rc)
    b1s = bh1 / den
    b2s = bh2 / den
    vb = v[T1] * b1s + v[T2] * b2s
    bs2 = b1s * b1s + b2s * b2s
    afb = afp * bts * bs2
    asb = asp * bts * bs2
    nf = 0.5 / a2
    cff = nf * fa * cf
    css = nf * sa * cs
    qfn = qf * nf
    qsn = qs * nf
    af_ = nf * afp * rd
    as_ = nf * asp * rd
    afb2 = nf * afp * bts
    asb2 = nf * asp * bts
    nf = nf * (gamma - 1.0)
    fan = fa * nf
    san = sa * nf
    b1c = b1s / bs2
    b2c = b2s / bs2
    vbs = v[T1] * b1c + v[T2] * b2c
    nf = nf * 2.0
    fl = _cell_flux(wl, ul, bn, hbl, axis)
    fr = _cell_flux(wr, ur, bn, hbr, axis)
    du = [ur[i] - ul[i] for i in range(7)]
    order = _order(axis)
    # L row by row, each wave amplitude right after its row (the same values; the
    # reverse sweep then holds few of L's adjoints at a time)
    amps = []
    L = {}
    L[0, 0] = fan * (vsq - hmb) + cff * (cf + vn) - qsn * vbs - asb2
    L[0, N] = -1.0 * fan * vn - cff
    L[0, T1] = -1.0 * fan * v[T1] + qsn * b1c
    L[0, T2] = -1.0 * fan * v[T2] + qsn * b2c
    L[0, 6] = fan
    L[0, 4] = as_ * b1c - fan * b1
    L[0, 5] = as_ * b2c - fan * b2
    amps.append(0.5 * fabs(lam[0]) * _project(L, 0, du, order))
    L[1, 0] = 0.5 * (v[T1] * bh2 - v[T2] * bh1)
    L[1, T1] = -0.5 * bh2
    L[1, T2] = 0.5 * bh1
    L[1, 4] = -0.5 * srd * bh2 * sgn
    L[1, 5] = 0.5 * srd * bh1 * sgn
    amps.append(0.5 * fabs(lam[1]) * _project(L, 1, du, order))
    L[2, 0] = san * (vsq - hmb) + css * (cs + vn) + qfn * vbs + afb2
    L[2, N] = -san * vn - css
    L[2, T1] = -san * v[T1] - qfn * b1c
    L[2, T2] = -san * v[T2] - qfn * b2c
    L[2, 6] = san
    L[2, 4] = -af_ * b1c - san * b1
    L[2, 5] = -af_ * b2c - san * b2
    amps.append(0.5 * fabs(lam[2]) * _project(L, 2, du, order))
    L[3, 0] = 1.0 - nf * (0.5 * vsq - (gamma - 2.0) * btc / (gamma - 1.0))
    L[3, 1] = nf * v[1]
    L[3, 2] = nf * v[2]
    L[3, 3] = nf * v[3]
    L[3, 6] = -1.0 * nf
    L[3, 4] = nf * b1
    L[3, 5] = nf * b2
    amps.append(0.5 * fabs(lam[3]) * _project(L, 3, du, order))
    L[4, 0] = san * (vsq - hmb) + css * (cs - vn) - qfn * vbs + afb2
    L[4, N] = -san * vn + css
    L[4, T1] = -san * v[T1] + qfn * b1c
    L[4, T2] = -san * v[T2] + qfn * b2c
    L[4, 6] = san
    L[4, 4] = L[2, 4]
    L[4, 5] = L[2, 5]
    amps.append(0.5 * fabs(lam[4]) * _project(L, 4, du, order))
    L[5, 0] = -L[1, 0]
    L[5, T1] = -L[1, T1]
    L[5, T2] = -L[1, T2]
    L[5, 4] = L[1, 4]
    L[5, 5] = L[1, 5]
    amps.append(0.5 * fabs(lam[5]) * _project(L, 5, du, order))
    L[6, 0] = fan * (vsq - hmb) + cff * (cf - vn) + qsn * vbs - asb2
    L[6, N] = -fan * vn + cff
    L[6, T1] = -fan * v[T1] - qsn * b1c
    L[6, T2] = -fan * v[T2] - qsn * b2c
    L[6, 6] = fan
    L[6, 4] = L[0, 4]
    L[6, 5] = L[0, 5]
    amps.append(0.5 * fabs(lam[6]) * _project(L, 6, du, order))
    # R where it is used (after L and the amplitudes): the same values, with its
    # entries' adjoints held only across the flux rows in the reverse sweep
    R = {}
    R[0, 0] = fa; R[0, 2] = sa; R[0, 3] = 1.0; R[0, 4] = sa; R[0, 6] = fa
    R[N, 0] = fa * lam[0]; R[N, 2] = sa * lam[2]; R[N, 3] = vn; R[N, 4] = sa * lam[4]; R[N, 6] = fa * lam[6]
    fv = fa * v[T1]; sv = sa * v[T1]; qsb = qs * b1s; qfb = qf * b1s
    R[T1, 0] = fv + qsb; R[T1, 1] = -bh2; R[T1, 2] = sv - qfb; R[T1, 3] = v[T1]
    R[T1, 4] = sv + qfb; R[T1, 5] = bh2; R[T1, 6] = fv - qsb
    fv = fa * v[T2]; sv = sa * v[T2]; qsb = qs * b2s; qfb = qf * b2s
    R[T2, 0] = fv + qsb; R[T2, 1] = bh1; R[T2, 2] = sv - qfb; R[T2, 3] = v[T2]
    R[T2, 4] = sv + qfb; R[T2, 5] = -bh1; R[T2, 6] = fv - qsb
    R[6, 0] = fa * (hmb - vn * cf) + qs * vb + asb
    R[6, 1] = -(v[T1] * bh2 - v[T2] * bh1)
    R[6, 2] = sa * (hmb - vn * cs) - qf * vb - afb
    R[6, 3] = 0.5 * vsq + (gamma - 2.0) * btc / (gamma - 1.0)
    R[6, 4] = sa * (hmb + vn * cs) + qf * vb - afb
    R[6, 5] = -R[6, 1]
    R[6, 6] = fa * (hmb + vn * cf) - qs * vb + asb
    R[4, 0] = asp * b1s; R[4, 1] = -bh2 * sgn * isrd; R[4, 2] = -afp * b1s
    R[4, 4] = R[4, 2]; R[4, 5] = R[4, 1]; R[4, 6] = R[4, 0]
    R[5, 0] = asp * b2s; R[5, 1] = bh1 * sgn * isrd; R[5, 2] = -afp * b2s
    R[5, 4] = R[5, 2]; R[5, 5] = R[5, 1]; R[5, 6] = R[5, 0]
    flux = []
    for i in range(7):
        acc = 0.5 * (fl[i] + fr[i])
        for j in range(7):
            if (i, j) in R:
                acc = acc - amps[j] * R[i, j]
        acc = select(lam[0] >= 0.0, fl[i], acc)
        acc = select(lam[6] <= 0.0, fr[i], acc)
        flux.append(acc)
    return flux


def roe1(ins, pars, axis, efix):
    """Stage-1 Roe flux (k_roe_mhd STAGE 1): ins = wl(7) + wr(7) + bn ; pars = [gamma, eps]."""
    wl, wr, bn = ins[0:7], ins[7:14], ins[14]
    gamma, eps = pars
    return roe_flux(wl, wr, prim_to_cons7(wl, bn, gamma), prim_to_cons7(wr, bn, gamma), bn, gamma, eps, efix, axis)


def roe2(ins, pars, axis, efix):
    """Stage-2 Roe flux (k_roe_mhd STAGE 2): ins = wl(7) + wr(7) + ul(7) + ur(7) + bn."""
    wl, wr, ul, ur, bn = ins[0:7], ins[7:14], ins[14:21], ins[21:28], ins[28]
    gamma, eps = pars
    return roe_flux(wl, wr, ul, ur, bn, gamma, eps, efix, axis)


def cell_ez(ins, pars):
    """Cell Ez = vy*Bx - vx*By: ins = [vy, Bx, vx, By]."""
    vy, bx, vx, by = ins
    return [vy * bx - vx * by]


def emf_corner(ins, pars):
    """k_emf: ins = [lt0, lt5, top0, top5, l0, l4, ul0, ul4, ec, el, eu, eul]."""
    lt0, lt5, top0, top5, l0, l4, ul0, ul4, ec, el, eu, eul = ins

    def three(s, pos, neg, zero):
        return select(s > 0.0, pos, select(s < 0.0, neg, select(s.eq(0.0), zero, 0.0)))
    x1 = three(lt0, lt5 - ul4 - eul, lt5 - l4 - el, lt5 - 0.5 * (l4 + ul4 + el + eul))
    x2 = three(top0, top5 - ul4 - eu, top5 - l4 - ec, top5 - 0.5 * (l4 + ul4 + ec + eu))
    y1 = three(ul0, -ul4 + lt5 - eul, -ul4 + top5 - eu, -ul4 + 0.5 * (lt5 + top5 - eul - eu))
    y2 = three(l0, -l4 + lt5 - el, -l4 + top5 - ec, -l4 + 0.5 * (lt5 + top5 - el - ec))
    return [0.25 * (x1 + x2 + y1 + y2)]


def ctu_side(ins, pars, axis):
    """One side of k_ctu_mhd.

    ins = w(7) + [bn] + fh(7) + flo(7) (raw transverse fluxes, before the remap)
          + [cbx, cby, cbz, cvz, lb, rb]
    pars = [gamma, half_dt, inv_dn, half_dtdt, min_d, min_e, nb]
    -> u(7) + w2(7)
    The half-step face B ``nb`` enters only cons->prim; it is a parameter here and
    differentiated separately (nfb_face).
    """
    w, bn = ins[0:7], ins[7]
    fh, flo = list(ins[8:15]), list(ins[15:22])
    cbx, cby, cbz, cvz, lb, rb = ins[22:28]
    gamma, half_dt, inv_dn, half_dtdt, min_d, min_e = pars[:6]
    nb = ins[28]
    u = prim_to_cons7(w, bn, gamma)
    dB = rb - lb
    src = [None, cbx * dB * inv_dn, cby * dB * inv_dn, cbz * dB * inv_dn,
           (cvz * dB * inv_dn) if axis == 1 else None, (cvz * dB * inv_dn) if axis == 0 else None,
           (cbz * cvz) * dB * inv_dn]
    if axis == 0:
        fh[5], fh[4] = fh[4], None
        flo[5], flo[4] = flo[4], None
    else:
        fh[4], fh[5] = fh[5], None
        flo[4], flo[5] = flo[5], None
    out_u = []
    for k in range(7):
        zero_src = (k == 0) or (k == (4 if axis == 0 else 5))
        if zero_src:
            if fh[k] is None:
                corr = None
            else:
                corr = -half_dtdt * (fh[k] - flo[k])
        else:
            corr = -half_dtdt * (fh[k] - flo[k]) + half_dt * src[k]
        out_u.append(u[k] if corr is None else u[k] + corr)
    out_u[0] = select(out_u[0] < min_d, min_d, out_u[0])
    out_u[6] = select(out_u[6] < min_e, min_e, out_u[6])
    w2 = cons_to_prim7(out_u, nb, gamma)
    return out_u + w2


def half_ez(ins, pars):
    """k_half_ez: ins = c(3) + fxl(3) + fxr(3) + fyt(3) + fyb(3) + [bxl, bxr, byt, byb]."""
    c = ins[0:3]
    fxl, fxr, fyt, fyb = ins[3:6], ins[6:9], ins[9:12], ins[12:15]
    bxl, bxr, byt, byb = ins[15:19]
    hx, hy = pars
    hu = []
    for k in range(3):
        u = c[k] - hx * (fxr[k] - fxl[k])
        u = u - hy * (fyb[k] - fyt[k])
        hu.append(u)
    hbx = (bxl + bxr) / 2.0
    hby = (byt + byb) / 2.0
    hvx = hu[1] / hu[0]
    hvy = hu[2] / hu[0]
    return [hvy * hbx - hvx * hby]


def final_cell(ins, pars):
    """k_final_mhd: new prim8 + cons8 of one cell.

    ins = [fbx_l, fbx_r, fby_t, fby_b, E00, E10, E01, E11] (E_ji at corners (j, i), (j+1, i),
          (j, i+1), (j+1, i+1)) + u(7) (x-sweep cons) + fxl(7) + fxr(7) + fyt(7) + fyb(7)
    pars = [dtdx, dtdy, gamma]
    """
    fbl, fbr, fbt, fbb, e00, e10, e01, e11 = ins[0:8]
    u = list(ins[8:15])
    fxl, fxr, fyt, fyb = ins[15:22], ins[22:29], ins[29:36], ins[36:43]
    dtdx, dtdy, gamma = pars
    bxl = fbl - dtdy * (e10 - e00)
    bxr = fbr - dtdy * (e11 - e01)
    byt = fbt + dtdx * (e01 - e00)
    byb = fbb + dtdx * (e11 - e10)
    cbx = (bxl + bxr) / 2.0
    cby = (byt + byb) / 2.0
    bz = u[5] - dtdx * (fxr[5] - fxl[5]) - dtdy * (fyb[4] - fyt[4])
    for k in (0, 1, 2, 3, 6):
        v = u[k] - dtdx * (fxr[k] - fxl[k])
        u[k] = v - dtdy * (fyb[k] - fyt[k])
    u[5] = bz
    u[4] = cby
    w = cons_to_prim7(u, cbx, gamma)
    prim = [w[0], w[1], w[2], w[3], cbx, w[4], w[5], w[6]]
    cons = [u[0], u[1], u[2], u[3], cbx, u[4], u[5], u[6]]
    return prim + cons


def face_half_x(ins, pars):
    """Half-step x-face B: nb = fbx - half_dtdy*(E_lo - E_up). ins = [fbx, E_lo, E_up]."""
    fb, lo, up = ins
    return [fb - pars[0] * (lo - up)]


def face_half_y(ins, pars):
    """Half-step y-face B: nb = fby + half_dtdx*(E_r - E_l). ins = [fby, E_r, E_l]."""
    fb, r, l_ = ins
    return [fb + pars[0] * (r - l_)]
