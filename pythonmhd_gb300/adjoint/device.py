"""Host-side handle of the GPU adjoint of the MHD step (``mhd2d_adj_*`` in the C ABI).

States live on the device as one packed float64 vector
``prim (8,ny,nx) | cons (8,ny,nx) | faceBx (ny,nx+1) | faceBy (ny+1,nx)``; an
adjoint ("bar") vector has the same layout.  Torch tensors carry the device
memory; the arithmetic is the library's.  dt is frozen: :meth:`Adjoint2D.forward`
records each cycle's CFL dt and :meth:`Adjoint2D.backward` treats it as a
constant (the choice the reference leaves open, since it has no adjoint).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib

OUTFLOW, PERIODIC = 0, 1


def _dptr(t):
    if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise ValueError("expected a contiguous float64 CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


class Adjoint2D:
    """Forward and reverse sweeps of the MHD CTU+CT step on one ny x nx grid.

    ``recon`` 0 (first order), 1 (PLM) or 2 (PPM).  Parameters mirror
    :class:`pythonmhd_gb300.solver.Grid2D` (MHD only).
    """

    def __init__(self, ny, nx, dx, dy, bcx=PERIODIC, bcy=PERIODIC, gamma=5.0 / 3.0, recon=1,
                 entropy_fix=False, eps=0.5, min_d=1e-12, min_p=1e-12, min_e=1e-12, device=None):
        self.lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.ny, self.nx = int(ny), int(nx)
        self.dx, self.dy = float(dx), float(dy)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.mhd2d_adj_create(self.ny, self.nx, self.dx, self.dy, int(bcx), int(bcy),
                                                 float(gamma), int(recon), 1 if entropy_fix else 0, float(eps),
                                                 float(min_d), float(min_p), float(min_e), ctypes.byref(h)),
                       "mhd2d_adj_create")
        self._h = h
        self.state_words = self.info()["state_words"]
        self.dts = None

    def info(self):
        """state_words, device_bytes (held now) and segment_sets (cycles kept resident per
        checkpoint segment by the last forward; 1 = recompute mode)."""
        words, nbytes, sets = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_int()
        _lib.check(self.lib.mhd2d_adj_info(self._h, ctypes.byref(words), ctypes.byref(nbytes), ctypes.byref(sets)),
                   "mhd2d_adj_info")
        return dict(state_words=words.value, device_bytes=nbytes.value, segment_sets=sets.value)

    def reshape(self, ny, nx, dx, dy, bcx=PERIODIC, bcy=PERIODIC, gamma=5.0 / 3.0):
        """Re-target this handle to another grid (same reconstruction and floors),
        reusing its device memory where it is large enough; drops the forward record."""
        _lib.check(self.lib.mhd2d_adj_reshape(self._h, int(ny), int(nx), float(dx), float(dy), int(bcx), int(bcy),
                                              float(gamma)), "mhd2d_adj_reshape")
        self.ny, self.nx = int(ny), int(nx)
        self.dx, self.dy = float(dx), float(dy)
        self.state_words = self.info()["state_words"]
        self.dts = None
        self._ckpt_ref = None

    def configure(self, segment_bytes=0, tail=None):
        """Memory the backward pass may use to keep a checkpoint segment resident (0 =
        automatic); ``tail``: cycles at the end of a forward pass run with tapes and left
        resident for the backward pass (-1 as many as fit, 0 none; None leaves it)."""
        _lib.check(self.lib.mhd2d_adj_configure(self._h, int(segment_bytes)), "mhd2d_adj_configure")
        if tail is not None:
            _lib.check(self.lib.mhd2d_adj_set_tail(self._h, int(tail)), "mhd2d_adj_set_tail")

    def record(self):
        """The last forward record: steps, checkpoint interval and tail cycles."""
        v = [ctypes.c_int() for _ in range(3)]
        _lib.check(self.lib.mhd2d_adj_record(self._h, *[ctypes.byref(x) for x in v]), "mhd2d_adj_record")
        return dict(steps=v[0].value, every=v[1].value, tail=v[2].value)

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.lib.mhd2d_adj_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- packing ----------------------------------------------------------
    def sizes(self):
        ny, nx = self.ny, self.nx
        return (8 * ny * nx, 8 * ny * nx, ny * (nx + 1), (ny + 1) * nx)

    def pack(self, prim, cons, fbx, fby):
        """Packed device vector from the four state arrays (NumPy or torch)."""
        parts = [torch.as_tensor(np.ascontiguousarray(a) if isinstance(a, np.ndarray) else a,
                                 dtype=torch.float64).reshape(-1) for a in (prim, cons, fbx, fby)]
        for p, n in zip(parts, self.sizes()):
            if p.numel() != n:
                raise ValueError(f"state part has {p.numel()} values, expected {n}")
        return torch.cat([p.to(self.device) for p in parts]).contiguous()

    def unpack(self, vec):
        """(prim, cons, faceBx, faceBy) views of a packed vector."""
        ny, nx = self.ny, self.nx
        a, b, c, _ = self.sizes()
        return (vec[:a].view(8, ny, nx), vec[a:a + b].view(8, ny, nx),
                vec[a + b:a + b + c].view(ny, nx + 1), vec[a + b + c:].view(ny + 1, nx))

    def _new(self):
        return torch.empty(self.state_words, dtype=torch.float64, device=self.device)

    def _sync(self):
        torch.cuda.current_stream(self.device).synchronize()

    # -- one cycle --------------------------------------------------------
    def cycle(self, state, dt):
        out = self._new()
        self._sync()
        _lib.check(self.lib.mhd2d_adj_cycle(self._h, float(dt), _dptr(state), _dptr(out)), "mhd2d_adj_cycle")
        return out

    def cycle_vjp(self, state, dt, bar_out):
        """Adjoint of one cycle at ``state``: d(<bar_out, cycle(state)>)/d(state)."""
        bar_in = self._new()
        self._sync()
        _lib.check(self.lib.mhd2d_adj_cycle_reverse(self._h, float(dt), _dptr(state), _dptr(bar_out),
                                                    _dptr(bar_in)), "mhd2d_adj_cycle_reverse")
        return bar_in

    # -- many cycles with checkpoints ---------------------------------------
    def forward(self, state, steps, cfl=0.4, dts=None, every=0):
        """``steps`` cycles; returns the final packed state.  ``self.dts`` holds the dts used."""
        steps = int(steps)
        out = self._new()
        log = np.zeros(steps, dtype=np.float64)
        fixed = None
        if dts is not None:
            fixed_arr = np.ascontiguousarray(dts, dtype=np.float64)
            if fixed_arr.shape != (steps,):
                raise ValueError("dts must hold one dt per step")
            fixed = fixed_arr.ctypes.data_as(_lib.c_double_p)
        self._sync()
        _lib.check(self.lib.mhd2d_adj_forward(self._h, _dptr(state), steps, float(cfl), fixed, int(every),
                                              _dptr(out), log.ctypes.data_as(_lib.c_double_p)),
                   "mhd2d_adj_forward")
        self.dts = log
        return out

    def restore(self, checkpoints, steps, every, dts):
        """Install a forward record made elsewhere: ``checkpoints`` a contiguous device
        tensor of ceil(steps/every) packed states (at cycles 0, every, ...; kept alive
        by the caller until the backward pass has run) and the host ``dts``."""
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        if dts.shape != (int(steps),):
            raise ValueError("dts must hold one dt per step")
        nck = -(-int(steps) // int(every))
        if checkpoints.numel() < nck * self.state_words:
            raise ValueError("checkpoints hold fewer states than the record needs")
        self._sync()
        _lib.check(self.lib.mhd2d_adj_restore(self._h, _dptr(checkpoints), int(steps), int(every),
                                              dts.ctypes.data_as(_lib.c_double_p)), "mhd2d_adj_restore")
        self._ckpt_ref = checkpoints
        self.dts = dts.copy()

    def branches(self, mode, state, dts):
        """``len(dts)`` cycles from ``state`` with the given dts, recording ("record") or
        replaying ("replay") every branch decision (``mhd2d_adj_branches``); returns the
        final packed state.  Replaying from nearby states evaluates the piece of the
        step the recorded run was on, which is what the backward pass differentiates."""
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        out = self._new()
        self._sync()
        _lib.check(self.lib.mhd2d_adj_branches(self._h, {"record": 1, "replay": 2}[mode], _dptr(state), len(dts),
                                               dts.ctypes.data_as(_lib.c_double_p), _dptr(out)),
                   "mhd2d_adj_branches")
        return out

    def backward(self, bar_final):
        """Adjoint of the last :meth:`forward` with respect to its initial state."""
        bar0 = self._new()
        self._sync()
        _lib.check(self.lib.mhd2d_adj_backward(self._h, _dptr(bar_final), _dptr(bar0)), "mhd2d_adj_backward")
        return bar0


class EvolveFunction(torch.autograd.Function):
    """``steps`` MHD cycles as a differentiable torch op on a packed state.

    Forward: the checkpointed forward pass; backward: the hand-written reverse
    sweep (dt frozen at the forward pass's values).
    """

    @staticmethod
    def forward(ctx, state, adj, steps, cfl, every):
        out = adj.forward(state.detach().contiguous(), steps, cfl=cfl, every=every)
        ctx.adj = adj
        return out

    @staticmethod
    def backward(ctx, grad_out):
        return ctx.adj.backward(grad_out.contiguous()), None, None, None, None


def evolve(state, adj, steps, cfl=0.4, every=0):
    """Differentiable ``steps``-cycle evolution of a packed state (see :class:`EvolveFunction`)."""
    return EvolveFunction.apply(state, adj, int(steps), float(cfl), int(every))
