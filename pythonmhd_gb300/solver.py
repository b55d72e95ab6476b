"""Host-side handle of one 2D grid on the GPU (thin wrapper over the C ABI)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib

ARITH = {"exact": 0, "fast": 1, "checked": 2}


def default_arith() -> str:
    """Arithmetic mode used when none is given: ``PYTHONMHD_GB300_ARITH`` or "exact"."""
    mode = os.environ.get("PYTHONMHD_GB300_ARITH", "exact").lower()
    if mode not in ARITH:
        raise ValueError(f"PYTHONMHD_GB300_ARITH must be one of {sorted(ARITH)}, got {mode!r}")
    return mode


def _ptr(a):
    return a.ctypes.data_as(_lib.c_double_p) if a is not None else None


def _as_f64c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Grid2D:
    """One ny x nx grid (hydro or MHD) resident on the current CUDA device.

    The state is uploaded with :meth:`upload`, advanced on the device with
    :meth:`advance` (the reference's evolve loop) and copied back with
    :meth:`download`.  ``arith="exact"`` reproduces the reference's float64
    arithmetic bit for bit; ``"fast"`` allows fused multiply-adds.
    """

    def __init__(self, ny, nx, dx, dy, bcx, bcy, gamma, mhd=True, recon=2, entropy_fix=False,
                 eps=0.5, min_d=1e-12, min_p=1e-12, min_e=1e-12, arith=None):
        self.lib = _lib.load()
        self.ny, self.nx = int(ny), int(nx)
        self.mhd = bool(mhd)
        self.nvars = 8 if self.mhd else 5
        self.arith = arith or default_arith()
        h = ctypes.c_void_p()
        _lib.check(self.lib.mhd2d_create(self.ny, self.nx, float(dx), float(dy), int(bcx), int(bcy),
                                         float(gamma), 1 if self.mhd else 0, int(recon),
                                         1 if entropy_fix else 0, float(eps), float(min_d),
                                         float(min_p), float(min_e), ARITH[self.arith], ctypes.byref(h)),
                   "mhd2d_create")
        self._h = h
        self.last_cycles = 0

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.lib.mhd2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- shapes -----------------------------------------------------------
    def cell_shape(self):
        return (self.nvars, self.ny, self.nx)

    def check_shapes(self, prim, cons, fbx=None, fby=None):
        if prim.shape != self.cell_shape() or cons.shape != self.cell_shape():
            raise ValueError(f"prim/cons must have shape {self.cell_shape()}, got {prim.shape}, {cons.shape}")
        if self.mhd:
            if fbx is None or fby is None:
                raise ValueError("MHD grids need faceBx and faceBy")
            if fbx.shape != (self.ny, self.nx + 1) or fby.shape != (self.ny + 1, self.nx):
                raise ValueError(f"faceBx/faceBy must be {(self.ny, self.nx + 1)}/{(self.ny + 1, self.nx)}")

    # -- data movement ----------------------------------------------------
    def upload(self, prim, cons, fbx=None, fby=None):
        prim, cons = _as_f64c(prim), _as_f64c(cons)
        fbx = _as_f64c(fbx) if fbx is not None else None
        fby = _as_f64c(fby) if fby is not None else None
        self.check_shapes(prim, cons, fbx, fby)
        _lib.check(self.lib.mhd2d_upload(self._h, _ptr(prim), _ptr(cons), _ptr(fbx), _ptr(fby)),
                   "mhd2d_upload")

    def upload_device(self, prim, cons, fbx=None, fby=None):
        """Upload from contiguous float64 CUDA tensors of the handle's device (no host copy)."""
        import torch

        def ptr(t):
            if t is None:
                return None
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                raise ValueError("upload_device expects contiguous float64 CUDA tensors")
            return ctypes.c_void_p(t.data_ptr())
        torch.cuda.current_stream(prim.device).synchronize()
        _lib.check(self.lib.mhd2d_upload_device(self._h, ptr(prim), ptr(cons), ptr(fbx), ptr(fby)),
                   "mhd2d_upload_device")

    def download_device(self, which, prim, cons, fbx=None, fby=None):
        """Copy the current (which=0) or second-last (which=1) state into contiguous float64
        CUDA tensors of the handle's device."""
        import torch

        def ptr(t):
            if t is None:
                return None
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                raise ValueError("download_device expects contiguous float64 CUDA tensors")
            return ctypes.c_void_p(t.data_ptr())
        torch.cuda.current_stream(prim.device).synchronize()
        _lib.check(self.lib.mhd2d_download_device(self._h, int(which), ptr(prim), ptr(cons), ptr(fbx), ptr(fby)),
                   "mhd2d_download_device")

    def download(self, which=0, prim=None, cons=None, fbx=None, fby=None):
        """Copy the current (which=0) or second-last (which=1) state into new or given arrays."""
        prim = np.empty(self.cell_shape()) if prim is None else prim
        cons = np.empty(self.cell_shape()) if cons is None else cons
        if self.mhd:
            fbx = np.empty((self.ny, self.nx + 1)) if fbx is None else fbx
            fby = np.empty((self.ny + 1, self.nx)) if fby is None else fby
        for a in (prim, cons, fbx, fby):
            if a is not None and not (a.dtype == np.float64 and a.flags.c_contiguous):
                raise ValueError("download targets must be C-contiguous float64")
        _lib.check(self.lib.mhd2d_download(self._h, int(which), _ptr(prim), _ptr(cons), _ptr(fbx), _ptr(fby)),
                   "mhd2d_download")
        return (prim, cons, fbx, fby) if self.mhd else (prim, cons)

    def advance(self, t0, t_end, cycle0, max_cycles, cfl):
        t = ctypes.c_double()
        c = ctypes.c_longlong()
        tsl = ctypes.c_double()
        _lib.check(self.lib.mhd2d_advance(self._h, float(t0), float(t_end), int(cycle0), int(max_cycles),
                                          float(cfl), ctypes.byref(t), ctypes.byref(c), ctypes.byref(tsl)),
                   "mhd2d_advance")
        self.last_cycles = c.value - int(cycle0)
        return t.value, c.value, tsl.value

    def cfl_dt(self, cfl):
        """The CFL dt of the current state before the t_end clip (exact arithmetic)."""
        dt = ctypes.c_double()
        _lib.check(self.lib.mhd2d_cfl_dt(self._h, float(cfl), ctypes.byref(dt)), "mhd2d_cfl_dt")
        return dt.value

    def advance_dt(self, t0, t_end, cycle0, dt):
        """One cycle with the given dt (clipped to t_end); returns the new time."""
        t = ctypes.c_double()
        _lib.check(self.lib.mhd2d_advance_dt(self._h, float(t0), float(t_end), int(cycle0), float(dt),
                                             ctypes.byref(t)), "mhd2d_advance_dt")
        self.last_cycles = 1
        return t.value

    def peek(self, what):
        """Intermediates of the last cycle (see mhd2d_peek in include/pythonmhd_gb300.h)."""
        nv = 7 if self.mhd else 5
        nx, ny = self.nx, self.ny
        shapes = {0: (nv, ny, nx + 1), 1: (nv, ny, nx + 1), 2: (nv, ny + 1, nx), 3: (nv, ny + 1, nx),
                  4: (nv, ny, nx + 1), 5: (nv, ny + 1, nx), 6: (ny + 1, nx + 1), 7: (ny, nx + 1),
                  8: (ny + 1, nx)}
        out = np.empty(shapes[what])
        _lib.check(self.lib.mhd2d_peek(self._h, int(what), _ptr(out), out.size), "mhd2d_peek")
        return out

    def last_launches(self):
        n = ctypes.c_longlong()
        _lib.check(self.lib.mhd2d_last_launches(self._h, ctypes.byref(n)), "mhd2d_last_launches")
        return n.value

    def device_bytes(self):
        n = ctypes.c_size_t()
        _lib.check(self.lib.mhd2d_device_bytes(self._h, ctypes.byref(n)), "mhd2d_device_bytes")
        return n.value

    def validate(self):
        """Counts of the current state's bad values (``mhd2d_validate``)."""
        c = np.zeros(7, dtype=np.int64)
        _lib.check(self.lib.mhd2d_validate(self._h, c.ctypes.data), "mhd2d_validate")
        keys = ("nonfinite", "density_negative", "density_low", "pressure_negative", "pressure_low",
                "energy_negative", "energy_low")
        return dict(zip(keys, (int(x) for x in c)))

    def check_state(self):
        """Raise RuntimeError as the reference's validatePrimVars would
        (Source/SimulationGrid_HelperModule.py:282-410): negative values before
        values below the floor, density before pressure before energy; a NaN or
        Inf anywhere is reported first."""
        c = self.validate()
        if c["nonfinite"]:
            raise RuntimeError(f"{c['nonfinite']} cells of the state hold a NaN or Inf value")
        names = (("density", "primitive"), ("pressure", "primitive"), ("energy", "conservative"))
        for name, kind in names:
            if c[f"{name}_negative"]:
                raise RuntimeError(f"You have at least one negative {name} value in your {kind} variables matrix "
                                   f"({c[name + '_negative']} values).")
            if c[f"{name}_low"]:
                raise RuntimeError(f"You have at least one {name} value in your {kind} variables matrix that is "
                                   f"less than the minimum {name} value for the simulation "
                                   f"({c[name + '_low']} values).")

    def check_info(self):
        """Checked arithmetic: (kernel source line, index) of the first failed index check
        since the last upload, or (0, 0)."""
        line, idx = ctypes.c_longlong(), ctypes.c_longlong()
        _lib.check(self.lib.mhd2d_check_info(self._h, ctypes.byref(line), ctypes.byref(idx)), "mhd2d_check_info")
        return line.value, idx.value

    def stats(self):
        """Failure counters since the last upload: ``{"floor_hits": n, "nan": bool}``."""
        hits = ctypes.c_longlong()
        nan = ctypes.c_int()
        _lib.check(self.lib.mhd2d_stats(self._h, ctypes.byref(hits), ctypes.byref(nan)), "mhd2d_stats")
        return {"floor_hits": hits.value, "nan": bool(nan.value)}

    def state_ptrs(self, which=0):
        ptrs = [ctypes.c_void_p() for _ in range(4)]
        _lib.check(self.lib.mhd2d_state_ptrs(self._h, int(which), *[ctypes.byref(p) for p in ptrs]),
                   "mhd2d_state_ptrs")
        return [p.value for p in ptrs]

    def stream(self):
        s = ctypes.c_void_p()
        _lib.check(self.lib.mhd2d_stream(self._h, ctypes.byref(s)), "mhd2d_stream")
        return s.value


class Grid1D(Grid2D):
    """One 1D grid of n cells (the reference's evolve_1D_mhd / evolve_1D_hydro step).

    States are (nvars, n); ``advance``/``download`` are Grid2D's (no face arrays).
    MHD keeps B_x uniform at the uploaded prim[4][0], as the reference does.
    """

    def __init__(self, n, dx, bcx, gamma, mhd=True, recon=2, entropy_fix=False, eps=0.5, min_d=1e-12,
                 min_p=1e-12, min_e=1e-12, arith=None):
        self.lib = _lib.load()
        self.ny, self.nx = 1, int(n)
        self.mhd = bool(mhd)
        self.nvars = 8 if self.mhd else 5
        self.arith = arith or default_arith()
        h = ctypes.c_void_p()
        _lib.check(self.lib.mhd1d_create(self.nx, float(dx), int(bcx), float(gamma), 1 if self.mhd else 0,
                                         int(recon), 1 if entropy_fix else 0, float(eps), float(min_d),
                                         float(min_p), float(min_e), ARITH[self.arith], ctypes.byref(h)),
                   "mhd1d_create")
        self._h = h
        self.last_cycles = 0

    def upload(self, prim, cons, fbx=None, fby=None):
        prim, cons = _as_f64c(prim), _as_f64c(cons)
        if prim.shape != (self.nvars, self.nx) or cons.shape != prim.shape:
            raise ValueError(f"prim/cons must be {(self.nvars, self.nx)}")
        _lib.check(self.lib.mhd1d_upload(self._h, _ptr(prim), _ptr(cons)), "mhd1d_upload")

    def download(self, which=0, prim=None, cons=None, fbx=None, fby=None):
        """(prim, cons) of the current (0) or second-last (1) state, as (nvars, n) arrays."""
        p = np.empty((self.nvars, 1, self.nx))
        c = np.empty((self.nvars, 1, self.nx))
        _lib.check(self.lib.mhd2d_download(self._h, int(which), _ptr(p), _ptr(c), None, None), "mhd2d_download")
        p, c = p[:, 0, :], c[:, 0, :]
        if prim is not None:
            prim[...] = p
            p = prim
        if cons is not None:
            cons[...] = c
            c = cons
        return p, c


class Grid3D:
    """One ny x nx x nz grid (the reference's evolve_3D_hydro / evolve_3D_mhd step) on the GPU.

    States are (nvars, ny, nx, nz) with z fastest, the reference's layout; MHD grids
    also carry faceBx (ny, nx+1, nz), faceBy (ny+1, nx, nz) and faceBz (ny, nx, nz+1).
    The evolve loop and the second-last state behave as in :class:`Grid2D`.
    """

    def __init__(self, ny, nx, nz, dx, dy, dz, bcx, bcy, bcz, gamma, recon=2, entropy_fix=False, eps=0.5,
                 min_d=1e-12, min_p=1e-12, min_e=1e-12, arith=None, mhd=False):
        self.lib = _lib.load()
        self.ny, self.nx, self.nz = int(ny), int(nx), int(nz)
        self.mhd = bool(mhd)
        self.nvars = 8 if self.mhd else 5
        self.arith = arith or default_arith()
        h = ctypes.c_void_p()
        _lib.check(self.lib.mhd3d_create(self.ny, self.nx, self.nz, float(dx), float(dy), float(dz), int(bcx),
                                         int(bcy), int(bcz), float(gamma), 1 if self.mhd else 0, int(recon),
                                         1 if entropy_fix else 0, float(eps), float(min_d), float(min_p),
                                         float(min_e), ARITH[self.arith], ctypes.byref(h)), "mhd3d_create")
        self._h = h
        self.last_cycles = 0

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.lib.mhd3d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def cell_shape(self):
        return (self.nvars, self.ny, self.nx, self.nz)

    def face_shapes(self):
        return ((self.ny, self.nx + 1, self.nz), (self.ny + 1, self.nx, self.nz), (self.ny, self.nx, self.nz + 1))

    def _check_faces(self, fb, kind):
        if not self.mhd:
            return [None, None, None]
        if fb is None or len(fb) != 3 or any(f is None for f in fb):
            raise ValueError("MHD grids need faceBx, faceBy and faceBz")
        for f, shape in zip(fb, self.face_shapes()):
            if tuple(f.shape) != shape:
                raise ValueError(f"face B arrays must have shapes {self.face_shapes()}")
        return list(fb)

    def upload(self, prim, cons, fbx=None, fby=None, fbz=None):
        prim, cons = _as_f64c(prim), _as_f64c(cons)
        if prim.shape != self.cell_shape() or cons.shape != self.cell_shape():
            raise ValueError(f"prim/cons must have shape {self.cell_shape()}, got {prim.shape}, {cons.shape}")
        fb = self._check_faces(None if fbx is None else (fbx, fby, fbz), "host")
        fb = [_as_f64c(f) if f is not None else None for f in fb]
        _lib.check(self.lib.mhd3d_upload(self._h, _ptr(prim), _ptr(cons), *[_ptr(f) for f in fb]), "mhd3d_upload")

    def upload_device(self, prim, cons, fbx=None, fby=None, fbz=None):
        """Upload from contiguous float64 CUDA tensors of the handle's device (no host copy)."""
        import torch
        fb = self._check_faces(None if fbx is None else (fbx, fby, fbz), "device")
        for t in [prim, cons] + [f for f in fb if f is not None]:
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                raise ValueError("upload_device expects contiguous float64 CUDA tensors")
        for t in (prim, cons):
            if tuple(t.shape) != self.cell_shape():
                raise ValueError(f"prim/cons must have shape {self.cell_shape()}")
        torch.cuda.current_stream(prim.device).synchronize()
        ptrs = [ctypes.c_void_p(t.data_ptr()) if t is not None else None for t in [prim, cons] + fb]
        _lib.check(self.lib.mhd3d_upload_device(self._h, *ptrs), "mhd3d_upload_device")

    def download(self, which=0, prim=None, cons=None, fbx=None, fby=None, fbz=None):
        """(prim, cons) -- plus (faceBx, faceBy, faceBz) for MHD -- of the current
        (which=0) or second-last (which=1) state."""
        prim = np.empty(self.cell_shape()) if prim is None else prim
        cons = np.empty(self.cell_shape()) if cons is None else cons
        fb = [fbx, fby, fbz]
        if self.mhd:
            fb = [np.empty(sh) if f is None else f for f, sh in zip(fb, self.face_shapes())]
        for a in [prim, cons] + [f for f in fb if f is not None]:
            if not (a.dtype == np.float64 and a.flags.c_contiguous):
                raise ValueError("download targets must be C-contiguous float64")
        if prim.shape != self.cell_shape() or cons.shape != self.cell_shape():
            raise ValueError("download targets must have the cell shape")
        _lib.check(self.lib.mhd3d_download(self._h, int(which), _ptr(prim), _ptr(cons), *[_ptr(f) for f in fb]),
                   "mhd3d_download")
        return (prim, cons, fb[0], fb[1], fb[2]) if self.mhd else (prim, cons)

    def advance(self, t0, t_end, cycle0, max_cycles, cfl):
        t = ctypes.c_double()
        c = ctypes.c_longlong()
        tsl = ctypes.c_double()
        _lib.check(self.lib.mhd3d_advance(self._h, float(t0), float(t_end), int(cycle0), int(max_cycles),
                                          float(cfl), ctypes.byref(t), ctypes.byref(c), ctypes.byref(tsl)),
                   "mhd3d_advance")
        self.last_cycles = c.value - int(cycle0)
        return t.value, c.value, tsl.value

    def _info(self):
        n = ctypes.c_longlong()
        b = ctypes.c_size_t()
        s = ctypes.c_void_p()
        _lib.check(self.lib.mhd3d_info(self._h, ctypes.byref(n), ctypes.byref(b), ctypes.byref(s)), "mhd3d_info")
        return n.value, b.value, s.value

    def last_launches(self):
        return self._info()[0]

    def device_bytes(self):
        return self._info()[1]

    def stream(self):
        return self._info()[2]

    def state_ptrs(self, which=0):
        ptrs = [ctypes.c_void_p() for _ in range(5)]
        _lib.check(self.lib.mhd3d_state_ptrs(self._h, int(which), *[ctypes.byref(p) for p in ptrs]),
                   "mhd3d_state_ptrs")
        return [p.value for p in ptrs[:5 if self.mhd else 2]]


class Batch2D:
    """Many independent grids advanced together (one persistent launch per stage).

    ``grids`` is a list of dicts with keys ny, nx, dx, dy, bcx, bcy, gamma; all
    instances share physics, reconstruction, entropy fix, floors and arithmetic.
    """

    def __init__(self, grids, mhd=True, recon=2, entropy_fix=False, eps=0.5, min_d=1e-12, min_p=1e-12,
                 min_e=1e-12, arith=None):
        self.lib = _lib.load()
        self.mhd = bool(mhd)
        self.nvars = 8 if self.mhd else 5
        self.arith = arith or default_arith()
        self.shapes = [(int(g["ny"]), int(g["nx"])) for g in grids]
        n = len(grids)
        ny = np.array([s[0] for s in self.shapes], dtype=np.int32)
        nx = np.array([s[1] for s in self.shapes], dtype=np.int32)
        dx = np.array([g["dx"] for g in grids], dtype=np.float64)
        dy = np.array([g["dy"] for g in grids], dtype=np.float64)
        bcx = np.array([g.get("bcx", 1) for g in grids], dtype=np.int32)
        bcy = np.array([g.get("bcy", 1) for g in grids], dtype=np.int32)
        gam = np.array([g["gamma"] for g in grids], dtype=np.float64)
        self._keep = (ny, nx, dx, dy, bcx, bcy, gam)
        h = ctypes.c_void_p()
        _lib.check(self.lib.mhdb_create(n, ny.ctypes.data, nx.ctypes.data, dx.ctypes.data, dy.ctypes.data,
                                        bcx.ctypes.data, bcy.ctypes.data, gam.ctypes.data, 1 if self.mhd else 0,
                                        int(recon), 1 if entropy_fix else 0, float(eps), float(min_d),
                                        float(min_p), float(min_e), ARITH[self.arith], ctypes.byref(h)),
                   "mhdb_create")
        self._h = h
        self.count = n

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.lib.mhdb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, k, prim, cons, fbx=None, fby=None):
        prim, cons = _as_f64c(prim), _as_f64c(cons)
        fbx = _as_f64c(fbx) if fbx is not None else None
        fby = _as_f64c(fby) if fby is not None else None
        ny, nx = self.shapes[k]
        if prim.shape != (self.nvars, ny, nx) or cons.shape != prim.shape:
            raise ValueError(f"instance {k}: prim/cons must be {(self.nvars, ny, nx)}")
        _lib.check(self.lib.mhdb_upload(self._h, int(k), _ptr(prim), _ptr(cons), _ptr(fbx), _ptr(fby)),
                   "mhdb_upload")

    def upload_device(self, k, prim, cons, fbx=None, fby=None):
        """Upload instance k from contiguous float64 CUDA tensors of the batch's device."""
        import torch

        def ptr(t):
            if t is None:
                return None
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                raise ValueError("upload_device expects contiguous float64 CUDA tensors")
            return ctypes.c_void_p(t.data_ptr())
        ny, nx = self.shapes[k]
        if tuple(prim.shape) != (self.nvars, ny, nx) or tuple(cons.shape) != tuple(prim.shape):
            raise ValueError(f"instance {k}: prim/cons must be {(self.nvars, ny, nx)}")
        torch.cuda.current_stream(prim.device).synchronize()
        _lib.check(self.lib.mhdb_upload_device(self._h, int(k), ptr(prim), ptr(cons), ptr(fbx), ptr(fby)),
                   "mhdb_upload_device")

    def advance(self, t0, t_end, cycle0, max_cycles, cfl):
        n = self.count
        t0 = np.broadcast_to(np.asarray(t0, dtype=np.float64), (n,)).copy()
        te = np.broadcast_to(np.asarray(t_end, dtype=np.float64), (n,)).copy()
        c0 = np.broadcast_to(np.asarray(cycle0, dtype=np.int64), (n,)).copy()
        mc = np.broadcast_to(np.asarray(max_cycles, dtype=np.int64), (n,)).copy()
        t_out = np.empty(n)
        c_out = np.empty(n, dtype=np.int64)
        rc = self.lib.mhdb_advance(self._h, t0.ctypes.data, te.ctypes.data, c0.ctypes.data, mc.ctypes.data,
                                   float(cfl), t_out.ctypes.data, c_out.ctypes.data)
        if rc != 0:
            err = _lib.MhdError(rc, "mhdb_advance")
            # the healthy instances ran to their ends; say which ones did not
            err.t_out, err.cycle_out = t_out, c_out
            err.instance_status = self.instance_status() if rc == 5 else None
            raise err
        return t_out, c_out

    def get_tiles(self, space):
        """The installed work list of an index space as an (n, 4) int32 array."""
        n = ctypes.c_longlong()
        _lib.check(self.lib.mhdb_get_tiles(self._h, int(space), None, 0, ctypes.byref(n)), "mhdb_get_tiles")
        t = np.zeros((n.value, 4), dtype=np.int32)
        _lib.check(self.lib.mhdb_get_tiles(self._h, int(space), t.ctypes.data, n.value, ctypes.byref(n)),
                   "mhdb_get_tiles")
        return t

    def set_tiles(self, space, tiles):
        """Install a caller's order of an index space's work list (checked on the host)."""
        t = np.ascontiguousarray(tiles, dtype=np.int32).reshape(-1, 4)
        _lib.check(self.lib.mhdb_set_tiles(self._h, int(space), t.ctypes.data, len(t)), "mhdb_set_tiles")

    def stats(self):
        """Per-instance failure counters since each upload: (floor_hits, nan flags)."""
        hits = np.zeros(self.count, dtype=np.int64)
        nan = np.zeros(self.count, dtype=np.int32)
        _lib.check(self.lib.mhdb_stats(self._h, hits.ctypes.data, nan.ctypes.data), "mhdb_stats")
        return hits, nan.astype(bool)

    def instance_status(self):
        """Per-instance status of the last advance (0 ok, 5 the time or dt went non-finite)."""
        st = np.zeros(self.count, dtype=np.int32)
        _lib.check(self.lib.mhdb_instance_status(self._h, st.ctypes.data), "mhdb_instance_status")
        return st

    def download(self, k, which=0):
        ny, nx = self.shapes[k]
        prim = np.empty((self.nvars, ny, nx))
        cons = np.empty((self.nvars, ny, nx))
        fbx = np.empty((ny, nx + 1)) if self.mhd else None
        fby = np.empty((ny + 1, nx)) if self.mhd else None
        _lib.check(self.lib.mhdb_download(self._h, int(k), int(which), _ptr(prim), _ptr(cons), _ptr(fbx), _ptr(fby)),
                   "mhdb_download")
        return (prim, cons, fbx, fby) if self.mhd else (prim, cons)

    def configure(self, tile_width=128, fuse=1, blocks=None):
        """Launch shape of a batched cycle: tile width (32/64/128), fusion depth (1/2), persistent blocks."""
        if blocks is None:
            blocks = self.info()["blocks"]
        _lib.check(self.lib.mhdb_configure(self._h, int(tile_width), int(fuse), int(blocks)), "mhdb_configure")
        self.launch_shape = (int(tile_width), int(fuse), int(blocks))

    def info(self):
        n = ctypes.c_longlong()
        b = ctypes.c_size_t()
        blk = ctypes.c_int()
        s = ctypes.c_void_p()
        _lib.check(self.lib.mhdb_info(self._h, ctypes.byref(n), ctypes.byref(b), ctypes.byref(blk), ctypes.byref(s)),
                   "mhdb_info")
        return {"last_launches": n.value, "device_bytes": b.value, "blocks": blk.value, "stream": s.value}
