"""Gradients through many independent MHD grids at once (the batched adjoint).

The forward pass advances every instance together on the batched step (one
persistent-kernel launch per stage over a work list of row tiles, per-instance
CFL dt; ``mhdb_*`` in the C ABI), one cycle per call from t = 0 so each
instance's returned time is its cycle's dt exactly.  Every ``every`` cycles
(default ceil(sqrt(steps)), less for an instance whose segment of resident
cycles would not fit the memory budget) each instance's state is packed into
one device arena that holds the checkpoints of all instances.  The backward pass then
runs instance by instance, largest first, on one adjoint handle re-targeted to
each grid in turn (its device memory allocated once), from that instance's
checkpoints and recorded dts: a segment stays resident when it fits the
budget, otherwise it is recomputed cycle by cycle.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from .. import _lib
from ..solver import Batch2D
from .device import Adjoint2D, _dptr


def state_words(nx, ny):
    return 16 * nx * ny + ny * (nx + 1) + (ny + 1) * nx


class BatchAdjoint:
    """Forward and backward passes over independent MHD grids.

    ``grids``: dicts with nx, ny, dx, dy, gamma and optionally bcx, bcy (default
    periodic).  ``recon`` 0, 1 or 2 (PPM).  ``budget`` bytes the backward pass may
    use to keep a segment resident (0: 85% of free memory at that time).
    """

    def __init__(self, grids, recon=2, entropy_fix=False, eps=0.5, min_d=1e-12, min_p=1e-12, min_e=1e-12,
                 budget=0, device=None):
        self.lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.grids = [dict(g) for g in grids]
        for g in self.grids:
            g.setdefault("bcx", 1)
            g.setdefault("bcy", 1)
        self.recon, self.efix, self.eps = int(recon), bool(entropy_fix), float(eps)
        self.floors = (float(min_d), float(min_p), float(min_e))
        self.budget = int(budget)
        self.words = [state_words(g["nx"], g["ny"]) for g in self.grids]
        self.steps = 0
        self.every = 0
        self.dts = None
        self.arena = None
        self.offsets = None

    def unpack(self, k, vec):
        g = self.grids[k]
        ny, nx = g["ny"], g["nx"]
        a = 8 * ny * nx
        b = ny * (nx + 1)
        return (vec[:a].view(8, ny, nx), vec[a:2 * a].view(8, ny, nx), vec[2 * a:2 * a + b].view(ny, nx + 1),
                vec[2 * a + b:].view(ny + 1, nx))

    def forward(self, states, steps, cfl=0.4, every=0):
        """Advance every instance ``steps`` cycles from its packed device state; returns
        the final packed states and records dts and checkpoints for :meth:`backward`."""
        n = len(self.grids)
        steps = int(steps)
        base = int(every) if every > 0 else int(np.ceil(np.sqrt(steps)))
        base = min(base, steps)
        self.arena = None
        torch.cuda.empty_cache()     # hand a previous arena back to the driver before sizing
        b = Batch2D(self.grids, mhd=True, recon=self.recon, entropy_fix=self.efix, eps=self.eps,
                    min_d=self.floors[0], min_p=self.floors[1], min_e=self.floors[2], arith="exact")
        everies = self._intervals(steps, base, b.info()["device_bytes"])
        ncks = [-(-steps // e) for e in everies]
        self.offsets = np.concatenate([[0], np.cumsum([c * w for c, w in zip(ncks, self.words)])])
        self.arena = torch.empty(int(self.offsets[-1]), dtype=torch.float64, device=self.device)
        torch.cuda.current_stream(self.device).synchronize()
        for k, st in enumerate(states):
            p, c, bx, by = self.unpack(k, st)
            _lib.check(self.lib.mhdb_upload_device(b._h, k, _dptr(p), _dptr(c), _dptr(bx), _dptr(by)),
                       "mhdb_upload_device")
        dts = np.zeros((n, steps))
        zeros = np.zeros(n)
        big = np.full(n, 1e300)
        for c in range(steps):
            for k in range(n):
                if c % everies[k] == 0:
                    dst = self.arena[int(self.offsets[k]) + (c // everies[k]) * self.words[k]:]
                    _lib.check(self.lib.mhdb_pack_state(b._h, k, _dptr(dst)), "mhdb_pack_state")
            t_out, c_out = b.advance(zeros, big, c, c + 1, cfl)
            if not np.all(c_out == c + 1):
                raise RuntimeError("batched step did not advance every instance by one cycle")
            dts[:, c] = t_out
        outs = []
        for k in range(n):
            o = torch.empty(self.words[k], dtype=torch.float64, device=self.device)
            _lib.check(self.lib.mhdb_pack_state(b._h, k, _dptr(o)), "mhdb_pack_state")
            outs.append(o)
        b.close()
        # the step has no positivity fix: a state can turn non-finite (negative
        # pressure under a square root) while dt stays finite; no gradient exists then
        bad = [k for k, o in enumerate(outs) if not bool(torch.isfinite(o).all())]
        if bad:
            raise FloatingPointError(f"non-finite final state in instance(s) {bad}")
        self.steps, self.every, self.dts = steps, everies, dts
        return outs

    def _intervals(self, steps, base, solver_bytes):
        """Checkpoint interval of each instance: ``base`` (sqrt(steps) by default), cut
        down where a segment of that many resident cycles (arrays and tapes) would not
        fit the segment budget, so that the backward pass recomputes every cycle once.
        The budget is half the memory left for the backward pass (free now, plus the
        batched step's, released before it, minus the checkpoint arena), and the arena
        itself is kept below 70% of the memory free now."""
        cyc = []
        for g in self.grids:
            nb = ctypes.c_size_t()
            _lib.check(self.lib.mhd2d_adj_cycle_bytes(g["ny"], g["nx"], self.recon, 1 if self.efix else 0,
                                                      ctypes.byref(nb)), "mhd2d_adj_cycle_bytes")
            cyc.append(nb.value)
        free, _ = torch.cuda.mem_get_info(self.device)

        def arena(ev):
            return 8 * sum(-(-steps // e) * w for e, w in zip(ev, self.words))

        everies = [base] * len(self.grids)
        for _ in range(3):
            budget = self.budget or int(0.5 * max(free + solver_bytes - arena(everies), 0))
            trial = [max(1, min(base, budget // c)) for c in cyc]
            if arena(trial) > 0.7 * free:
                break
            everies = trial
        if arena(everies) > 0.7 * free:
            raise MemoryError("the checkpoints of this batch do not fit the device memory")
        return everies

    def backward(self, bars):
        """Adjoints of the initial states from the adjoints of the final states
        (dt frozen at the recorded values), instance by instance."""
        if self.arena is None:
            raise RuntimeError("backward before forward")
        out = [None] * len(self.grids)
        self.backward_seconds = [0.0] * len(self.grids)
        # one handle for all instances, largest first: its device memory is allocated
        # once and reused by every smaller instance
        order = sorted(range(len(self.grids)), key=lambda k: -self.grids[k]["nx"] * self.grids[k]["ny"])
        # memory torch has cached but not returned would otherwise look used to the
        # handle's resident-segment decision (cudaMemGetInfo)
        torch.cuda.empty_cache()
        a = None
        for k in order:
            g = self.grids[k]
            t0 = time.perf_counter()
            if a is None:
                a = Adjoint2D(g["ny"], g["nx"], g["dx"], g["dy"], g["bcx"], g["bcy"], g["gamma"], recon=self.recon,
                              entropy_fix=self.efix, eps=self.eps, min_d=self.floors[0], min_p=self.floors[1],
                              min_e=self.floors[2], device=self.device)
                a.configure(self.budget)
            else:
                a.reshape(g["ny"], g["nx"], g["dx"], g["dy"], g["bcx"], g["bcy"], g["gamma"])
            ck = self.arena[int(self.offsets[k]):int(self.offsets[k + 1])]
            a.restore(ck, self.steps, self.every[k], self.dts[k])
            out[k] = a.backward(bars[k].contiguous())
            self.backward_seconds[k] = time.perf_counter() - t0
        if a is not None:
            a.close()
        return out
