"""One MHD CTU+CT cycle and its reverse sweep, assembled in NumPy from the SSA
stage functions (``stages.py``).

This is the CPU form of the adjoint: the same pointwise functions the GPU
adjoint kernels are generated from, glued by the same stencil (gathers in the
forward sweep, scatter-adds in the reverse sweep).  Its forward cycle must equal
the forward step bit for bit, and its reverse sweep is checked against finite
differences; the GPU adjoint is then checked against it.

dt is an input of a cycle (frozen): the forward pass records it, the reverse
sweep does not differentiate it.  Reconstruction: first order (0), PLM (1) and PPM (2).
"""
from __future__ import annotations

import functools

import numpy as np

from . import dsl, stages

OUTFLOW, PERIODIC = 0, 1


@functools.lru_cache(maxsize=None)
def _fn(name, efix=False, backend="numpy", device=None):
    spec = {
        "plm0": (stages.plm_cell, 22, 2, dict(axis=0)),
        "plm1": (stages.plm_cell, 22, 2, dict(axis=1)),
        "pslope0": (stages.ppm_slope, 22, 1, dict(axis=0)),
        "pslope1": (stages.ppm_slope, 22, 1, dict(axis=1)),
        "ppmi0": (stages.ppm_iface, 42, 1, dict(axis=0)),
        "ppmi1": (stages.ppm_iface, 42, 1, dict(axis=1)),
        "ppmt0": (stages.ppm_trace, 21 + stages.EIG_BASE, 2, dict(axis=0)),
        "ppmt1": (stages.ppm_trace, 21 + stages.EIG_BASE, 2, dict(axis=1)),
        "face0": (stages.face_state, 10, 4, dict(sb=4)),
        "face1": (stages.face_state, 10, 4, dict(sb=5)),
        "roe1_0": (stages.roe1, 15, 2, dict(axis=0, efix=efix)),
        "roe1_1": (stages.roe1, 15, 2, dict(axis=1, efix=efix)),
        "roe2_0": (stages.roe2, 29, 2, dict(axis=0, efix=efix)),
        "roe2_1": (stages.roe2, 29, 2, dict(axis=1, efix=efix)),
        "ez": (stages.cell_ez, 4, 0, {}),
        "emf": (stages.emf_corner, 12, 0, {}),
        "ctu0": (stages.ctu_side, 29, 6, dict(axis=0)),
        "ctu1": (stages.ctu_side, 29, 6, dict(axis=1)),
        "half": (stages.half_ez, 19, 2, {}),
        "final": (stages.final_cell, 43, 3, {}),
        "fhx": (stages.face_half_x, 3, 1, {}),
        "fhy": (stages.face_half_y, 3, 1, {}),
    }[name]
    fn, nin, npar, kw = spec
    t = dsl.trace(name.replace("-", "_") + ("_efix" if efix else ""), fn, nin, npar, **kw)
    if backend == "torch":
        return dsl.compile_torch(t, device), None
    return dsl.compile_numpy(t, reverse=True)


def _wrap(i, n, bc):
    return np.mod(i, n) if bc == PERIODIC else np.clip(i, 0, n - 1)


class _Arr:
    """An array of the cycle with its adjoint accumulator (NumPy form only)."""

    def __init__(self, data):
        self.v = data
        self.b = np.zeros_like(data) if isinstance(data, np.ndarray) else None


def _stage(tape, name, efix, ins, pars, backend="numpy", device=None):
    """Run a stage forward on gathered inputs; remember it for the reverse sweep.

    ins: list of (arr, slot, idx) -- slot None for a 2D array; idx a tuple of index arrays.
    """
    fwd, rev = _fn(name, efix, backend, device)
    x = [a.v[idx] if slot is None else a.v[slot][idx] for (a, slot, idx) in ins]
    y = fwd(x, pars)
    tape.append((rev, ins, pars, x))
    return y


def _reverse(tape_entry, ybar):
    rev, ins, pars, x = tape_entry
    xb = rev(x, pars, ybar)
    for (a, slot, idx), g in zip(ins, xb):
        if isinstance(g, float) and g == 0.0:
            continue
        tgt = a.b if slot is None else a.b[slot]
        np.add.at(tgt, idx, np.broadcast_to(g, np.broadcast(*idx).shape))


X_SLOTS = (0, 1, 2, 3, 5, 6, 7)      # prim8/cons8 slots of the x-sweep vector
Y_SLOTS = (0, 1, 2, 3, 6, 4, 7)


class Cycle:
    """Forward sweep of one cycle that records what the reverse sweep needs.

    ``backend="torch"`` runs the same stencil on torch float64 tensors with the
    stage functions emitted as torch code (forward only): a plain PyTorch
    transcription of the step that torch's own automatic differentiation can
    differentiate, as an independent check of the hand-written reverse sweeps.
    """

    def __init__(self, prim, cons, fbx, fby, dt, dx, dy, bcx, bcy, gamma, min_d, min_p, min_e, order, efix, eps,
                 backend="numpy"):
        assert order in (0, 1, 2)
        self.backend = backend
        if backend == "torch":
            import torch
            self._torch = torch
            self.P, self.C, self.FX, self.FY = (_Arr(t) for t in (prim, cons, fbx, fby))
        else:
            self.P, self.C = _Arr(np.array(prim, dtype=float)), _Arr(np.array(cons, dtype=float))
            self.FX, self.FY = _Arr(np.array(fbx, dtype=float)), _Arr(np.array(fby, dtype=float))
        self.dt, self.dx, self.dy = dt, dx, dy
        self.bc = (bcx, bcy)
        self.gamma, self.min_d, self.min_p, self.min_e = gamma, min_d, min_p, min_e
        self.order, self.efix, self.eps = order, bool(efix), eps
        self.tape = []          # (entry, outputs: list of (arr, slot, idx))
        self._run()

    def _zeros(self, shape):
        if self.backend == "torch":
            return _Arr(self._torch.zeros(shape, dtype=self._torch.float64, device=self.P.v.device))
        return _Arr(np.zeros(shape))

    # -- helpers -------------------------------------------------------------
    def _rec(self, name, ins, pars, outs):
        if self.backend == "torch":
            ins = [(a, slot, self._tix(idx)) for (a, slot, idx) in ins]
            outs = [(a, slot, self._tix(idx)) for (a, slot, idx) in outs]
        dev = str(self.P.v.device) if self.backend == "torch" else None
        y = _stage(self._t, name, self.efix if name.startswith("roe") else False, ins, pars, self.backend, dev)
        entry = self._t.pop()
        for (a, slot, idx), val in zip(outs, y):
            tgt = a.v if slot is None else a.v[slot]
            tgt[idx] = val
        self.tape.append((entry, outs))
        return y

    def _run(self):
        self._t = []
        P, C, FX, FY = self.P, self.C, self.FX, self.FY
        ny, nx = P.v.shape[1:]
        self.ny, self.nx = ny, nx
        g = self.gamma
        dt, dx, dy = self.dt, self.dx, self.dy
        J, I = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
        # ---- reconstruction + face states, x and y
        self.XL, self.XR = self._zeros((7, ny, nx + 1)), self._zeros((7, ny, nx + 1))
        self.YL, self.YR = self._zeros((7, ny + 1, nx)), self._zeros((7, ny + 1, nx))
        for ax in (0, 1):
            slots = X_SLOTS if ax == 0 else Y_SLOTS
            L = nx if ax == 0 else ny
            bc = self.bc[ax]
            dn = dx if ax == 0 else dy
            E = self._zeros((14, ny, nx))      # lia(7) + ria(7) per cell
            def cell(off):
                if ax == 0:
                    return (J, _wrap(I + off, nx, bc))
                return (_wrap(J + off, ny, bc), I)
            bslot = 4 if ax == 0 else 5
            if self.order == 1:
                ins = [(P, s, cell(off)) for off in (-1, 0, 1) for s in slots]
                ins.append((P, bslot, cell(0)))
                self._rec(f"plm{ax}", ins, [g, dt / dn], [(E, k, (J, I)) for k in range(14)])
            elif self.order == 2:
                # slopes of the sweep-extended cells -1 .. L (extended index e = cell + 1),
                # each with its eigensystem's base words (planes 7 ..)
                ns = 7 + stages.EIG_BASE
                if ax == 0:
                    SJ, SE = np.meshgrid(np.arange(ny), np.arange(nx + 2), indexing="ij")
                    S = self._zeros((ns, ny, nx + 2))

                    def ecell(off):
                        return (SJ, _wrap(SE - 1 + off, nx, bc))
                else:
                    SE, SJ = np.meshgrid(np.arange(ny + 2), np.arange(nx), indexing="ij")
                    S = self._zeros((ns, ny + 2, nx))

                    def ecell(off):
                        return (_wrap(SE - 1 + off, ny, bc), SJ)
                ins = [(P, s, ecell(off)) for off in (-1, 0, 1) for s in slots]
                ins.append((P, bslot, ecell(0)))
                self._rec(f"pslope{ax}", ins, [g], [(S, k, (SJ, SE) if ax == 0 else (SE, SJ)) for k in range(ns)])
                # interface values with monotonicity (E0), then the characteristic tracing
                E0 = self._zeros((14, ny, nx))
                ins = [(P, s, cell(off)) for off in (-1, 0, 1) for s in slots]
                for off in (0, 1, 2):
                    sidx = (J, I + off) if ax == 0 else (J + off, I)
                    ins += [(S, k, sidx) for k in range(7)]
                self._rec(f"ppmi{ax}", ins, [g], [(E0, k, (J, I)) for k in range(14)])
                own = (J, I + 1) if ax == 0 else (J + 1, I)
                ins = [(P, s, cell(0)) for s in slots] + [(E0, k, (J, I)) for k in range(14)]
                ins += [(S, 7 + k, own) for k in range(stages.EIG_BASE)]
                self._rec(f"ppmt{ax}", ins, [g, dt / dn], [(E, k, (J, I)) for k in range(14)])
            else:
                for k, s in enumerate(slots):
                    self._rec_copy(P, s, E, k)
                    self._rec_copy(P, s, E, 7 + k)
            # face states
            nf = L + 1
            if ax == 0:
                FJ, FF = np.meshgrid(np.arange(ny), np.arange(nf), indexing="ij")
            else:
                FF, FJ = np.meshgrid(np.arange(nf), np.arange(nx), indexing="ij")
            f = FF
            # left state: ria of cell f-1 (f>=1); f=0: outflow lia of cell 0, periodic ria of cell L-1
            if bc == OUTFLOW:
                l_cell = np.where(f == 0, 0, f - 1)
                l_side = np.where(f == 0, 0, 7)
                l_vc, l_f1, l_f2 = np.where(f == 0, 0, f - 1), np.where(f == 0, 0, f - 1), np.where(f == 0, 0, f)
                r_cell = np.where(f == L, L - 1, f)
                r_side = np.where(f == L, 7, 0)
                r_vc, r_f1, r_f2 = np.where(f == L, L - 1, f), np.where(f == L, L, f), np.where(f == L, L, f + 1)
            else:
                l_cell = np.where(f == 0, L - 1, f - 1)
                l_side = np.full_like(f, 7)
                l_vc, l_f1, l_f2 = l_cell, np.where(f == 0, L - 1, f - 1), f
                r_cell = np.where(f == L, 0, f)
                r_side = np.zeros_like(f)
                r_vc, r_f1, r_f2 = r_cell, np.where(f == L, L, f), np.where(f == L, 1, f + 1)
            fb = FX if ax == 0 else FY
            vslot = 2 if ax == 0 else 1
            for side, (cel, sd, vc, f1, f2) in enumerate(((l_cell, l_side, l_vc, l_f1, l_f2),
                                                          (r_cell, r_side, r_vc, r_f1, r_f2))):
                out = (self.XL if side == 0 else self.XR) if ax == 0 else (self.YL if side == 0 else self.YR)
                if ax == 0:
                    cidx = (FJ, cel)
                    vidx = (FJ, vc)
                    f1i, f2i = (FJ, f1), (FJ, f2)
                else:
                    cidx = (cel, FJ)
                    vidx = (vc, FJ)
                    f1i, f2i = (f1, FJ), (f2, FJ)
                # the edge slot (lia or ria) differs per face: gather from E with a per-face slot
                ins = []
                for k in range(7):
                    ins.append((E, None, (sd + k, ) + cidx))
                ins += [(P, vslot, vidx), (fb, None, f1i), (fb, None, f2i)]
                self._rec(f"face{ax}", ins, [self.min_d, self.min_p, 0.5 * dt, 1.0 / dn],
                          [(out, k, (FJ, FF) if ax == 0 else (FF, FJ)) for k in range(7)])
        # ---- stage-1 Roe
        self.F1X, self.F1Y = self._zeros((7, ny, nx + 1)), self._zeros((7, ny + 1, nx))
        self._roe(1, self.XL, self.XR, None, None, self.FX, self.F1X, 0)
        self._roe(1, self.YL, self.YR, None, None, self.FY, self.F1Y, 1)
        # ---- cell Ez and corner EMF
        self.EZ = self._zeros((ny, nx))
        self._rec("ez", [(P, 2, (J, I)), (P, 4, (J, I)), (P, 1, (J, I)), (P, 5, (J, I))], [],
                  [(self.EZ, None, (J, I))])
        self.E1 = self._zeros((ny + 1, nx + 1))
        self._emf(self.F1X, self.F1Y, self.EZ, self.E1)
        # ---- half-step faces
        self.NBX, self.NBY = self._zeros((ny, nx + 1)), self._zeros((ny + 1, nx))
        hj, hi = np.meshgrid(np.arange(ny), np.arange(nx + 1), indexing="ij")
        self._rec("fhx", [(FX, None, (hj, hi)), (self.E1, None, (hj + 1, hi)), (self.E1, None, (hj, hi))],
                  [0.5 * (dt / dy)], [(self.NBX, None, (hj, hi))])
        vj, vi = np.meshgrid(np.arange(ny + 1), np.arange(nx), indexing="ij")
        self._rec("fhy", [(FY, None, (vj, vi)), (self.E1, None, (vj, vi + 1)), (self.E1, None, (vj, vi))],
                  [0.5 * (dt / dx)], [(self.NBY, None, (vj, vi))])
        # ---- CTU
        self.UXL, self.UXR = self._zeros((7, ny, nx + 1)), self._zeros((7, ny, nx + 1))
        self.UYL, self.UYR = self._zeros((7, ny + 1, nx)), self._zeros((7, ny + 1, nx))
        self.WXL, self.WXR = self._zeros((7, ny, nx + 1)), self._zeros((7, ny, nx + 1))
        self.WYL, self.WYR = self._zeros((7, ny + 1, nx)), self._zeros((7, ny + 1, nx))
        self._ctu(0)
        self._ctu(1)
        # ---- half-step cell Ez
        self.HEZ = self._zeros((ny, nx))
        ins = [(C, k, (J, I)) for k in range(3)]
        ins += [(self.F1X, k, (J, I)) for k in range(3)] + [(self.F1X, k, (J, I + 1)) for k in range(3)]
        ins += [(self.F1Y, k, (J, I)) for k in range(3)] + [(self.F1Y, k, (J + 1, I)) for k in range(3)]
        ins += [(self.NBX, None, (J, I)), (self.NBX, None, (J, I + 1)), (self.NBY, None, (J, I)),
                (self.NBY, None, (J + 1, I))]
        self._rec("half", ins, [0.5 * (dt / dx), 0.5 * (dt / dy)], [(self.HEZ, None, (J, I))])
        # ---- stage-2 Roe and EMF
        self.F2X, self.F2Y = self._zeros((7, ny, nx + 1)), self._zeros((7, ny + 1, nx))
        self._roe(2, self.WXL, self.WXR, self.UXL, self.UXR, self.NBX, self.F2X, 0)
        self._roe(2, self.WYL, self.WYR, self.UYL, self.UYR, self.NBY, self.F2Y, 1)
        self.E2 = self._zeros((ny + 1, nx + 1))
        self._emf(self.F2X, self.F2Y, self.HEZ, self.E2)
        # ---- final update
        self.NP, self.NC = self._zeros(tuple(P.v.shape)), self._zeros(tuple(C.v.shape))
        E2 = self.E2
        ins = [(FX, None, (J, I)), (FX, None, (J, I + 1)), (FY, None, (J, I)), (FY, None, (J + 1, I)),
               (E2, None, (J, I)), (E2, None, (J + 1, I)), (E2, None, (J, I + 1)), (E2, None, (J + 1, I + 1))]
        ins += [(C, s, (J, I)) for s in X_SLOTS]
        ins += [(self.F2X, k, (J, I)) for k in range(7)] + [(self.F2X, k, (J, I + 1)) for k in range(7)]
        ins += [(self.F2Y, k, (J, I)) for k in range(7)] + [(self.F2Y, k, (J + 1, I)) for k in range(7)]
        outs = [(self.NP, k, (J, I)) for k in range(8)] + [(self.NC, k, (J, I)) for k in range(8)]
        self._rec("final", ins, [dt / dx, dt / dy, g], outs)
        self.NFX, self.NFY = self._zeros(tuple(FX.v.shape)), self._zeros(tuple(FY.v.shape))
        self._rec("fhx", [(FX, None, (hj, hi)), (E2, None, (hj + 1, hi)), (E2, None, (hj, hi))],
                  [dt / dy], [(self.NFX, None, (hj, hi))])
        self._rec("fhy", [(FY, None, (vj, vi)), (E2, None, (vj, vi + 1)), (E2, None, (vj, vi))],
                  [dt / dx], [(self.NFY, None, (vj, vi))])

    def _tix(self, idx):
        return tuple(self._torch.as_tensor(np.asarray(i), device=self.P.v.device) for i in idx)

    def _rec_copy(self, src, s, dst, k):
        """dst[k] = src[s] (first-order edges), recorded as an identity stage."""
        dst.v[k] = src.v[s]
        self.tape.append((("copy", src, s, dst, k), None))

    def _roe(self, stage, WL, WR, UL, UR, BN, F, ax):
        shape = WL.v.shape[1:]
        A, B = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
        idx = (A, B)
        ins = [(WL, k, idx) for k in range(7)] + [(WR, k, idx) for k in range(7)]
        if stage == 2:
            ins += [(UL, k, idx) for k in range(7)] + [(UR, k, idx) for k in range(7)]
        ins.append((BN, None, idx))
        self._rec(f"roe{stage}_{ax}", ins, [self.gamma, self.eps], [(F, k, idx) for k in range(7)])

    def _emf(self, FXa, FYa, EZ, OUT):
        ny, nx = self.ny, self.nx
        bcx, bcy = self.bc
        JJ, II = np.meshgrid(np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
        ic, im = _wrap(II, nx, bcx), _wrap(II - 1, nx, bcx)
        jc, jm = _wrap(JJ, ny, bcy), _wrap(JJ - 1, ny, bcy)
        ins = [(FYa, 0, (JJ, im)), (FYa, 5, (JJ, im)), (FYa, 0, (JJ, ic)), (FYa, 5, (JJ, ic)),
               (FXa, 0, (jc, II)), (FXa, 4, (jc, II)), (FXa, 0, (jm, II)), (FXa, 4, (jm, II)),
               (EZ, None, (jc, ic)), (EZ, None, (jc, im)), (EZ, None, (jm, ic)), (EZ, None, (jm, im))]
        self._rec("emf", ins, [], [(OUT, None, (JJ, II))])

    def _ctu(self, ax):
        ny, nx = self.ny, self.nx
        bc = self.bc[ax]
        dt, dx, dy, g = self.dt, self.dx, self.dy, self.gamma
        L = nx if ax == 0 else ny
        if ax == 0:
            T, Fi = np.meshgrid(np.arange(ny), np.arange(nx + 1), indexing="ij")
        else:
            Fi, T = np.meshgrid(np.arange(ny + 1), np.arange(nx), indexing="ij")
        fb = self.FX if ax == 0 else self.FY
        fidx = (T, Fi) if ax == 0 else (Fi, T)
        inv_dn = 1.0 / (dx if ax == 0 else dy)
        half_dtdt = 0.5 * (dt / (dy if ax == 0 else dx))
        for side in (0, 1):
            W = (self.XL if side == 0 else self.XR) if ax == 0 else (self.YL if side == 0 else self.YR)
            U = (self.UXL if side == 0 else self.UXR) if ax == 0 else (self.UYL if side == 0 else self.UYR)
            W2 = (self.WXL if side == 0 else self.WXR) if ax == 0 else (self.WYL if side == 0 else self.WYR)
            kpad = Fi + side
            if ax == 0:
                scell = _wrap(kpad - 1, L, bc)
                if bc == OUTFLOW:
                    lb, rb = np.clip(kpad - 1, 0, L), np.minimum(kpad, L)
                else:
                    lb, rb = np.where(kpad == 0, L - 1, kpad - 1), np.where(kpad == L + 1, 1, kpad)
            else:
                if bc == OUTFLOW:
                    scell = np.where(kpad == 0, 1, np.minimum(kpad - 1, L - 1))
                    lb, rb = np.where(kpad == 0, 1, kpad - 1), np.where(kpad == L + 1, L - 1, kpad)
                else:
                    scell = _wrap(kpad - 1, L, bc)
                    lb, rb = np.where(kpad == 0, L - 1, kpad - 1), np.where(kpad == L + 1, 1, kpad)
            fc = _wrap(Fi - 1 + side, L, bc)
            if ax == 0:
                Ft = self.F1Y
                hi_idx, lo_idx = (T + 1, fc), (T, fc)
                sidx = (T, scell)
                lbi, rbi = (T, lb), (T, rb)
            else:
                Ft = self.F1X
                hi_idx, lo_idx = (fc, T + 1), (fc, T)
                sidx = (scell, T)
                lbi, rbi = (lb, T), (rb, T)
            P = self.P
            ins = [(W, k, fidx) for k in range(7)] + [(fb, None, fidx)]
            ins += [(Ft, k, hi_idx) for k in range(7)] + [(Ft, k, lo_idx) for k in range(7)]
            ins += [(P, 4, sidx), (P, 5, sidx), (P, 6, sidx), (P, 3, sidx), (fb, None, lbi), (fb, None, rbi)]
            ins.append(((self.NBX if ax == 0 else self.NBY), None, fidx))
            outs = [(U, k, fidx) for k in range(7)] + [(W2, k, fidx) for k in range(7)]
            self._rec(f"ctu{ax}", ins, [g, 0.5 * dt, inv_dn, half_dtdt, self.min_d, self.min_e], outs)

    # -- results -------------------------------------------------------------
    def outputs(self):
        return self.NP.v, self.NC.v, self.NFX.v, self.NFY.v

    def reverse(self, prim_bar, cons_bar, fbx_bar, fby_bar):
        """Adjoint of the cycle: returns (prim_bar, cons_bar, fbx_bar, fby_bar) of its inputs."""
        self.NP.b[...] = prim_bar
        self.NC.b[...] = cons_bar
        self.NFX.b[...] = fbx_bar
        self.NFY.b[...] = fby_bar
        for entry, outs in reversed(self.tape):
            if entry[0] == "copy":
                _, src, s, dst, k = entry
                src.b[s] += dst.b[k]
                continue
            ybar = [(a.b if slot is None else a.b[slot])[idx] for (a, slot, idx) in outs]
            _reverse(entry, ybar)
        return self.P.b, self.C.b, self.FX.b, self.FY.b
