"""The allocation-free CFL timestep entry point (mhd2d_cfl_dt_noalloc).

It serves callers that cannot allocate device memory themselves -- code whose
device memory belongs to another framework's caching allocator, or a stepping
loop that must not call cudaMalloc/cudaFree every step -- so it takes device
pointers to the state and to its one-double output and keeps its scratch in a
static device array.  This test calls it through the C ABI on device buffers
owned by torch and checks it against the dt the regular handle-based entry
point uses (its first cycle from t = 0 ends at t = dt exactly), bit for bit as
the exact-arithmetic tests require, on two calls in a row: a larger MHD grid and
then a smaller hydro grid, so stale scratch from the first call cannot leak into
the second.  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from pythonmhd_gb300 import _lib
from pythonmhd_gb300 import initial_conditions as ic
from pythonmhd_gb300.solver import Grid2D

pytestmark = pytest.mark.gpu
G = 5.0 / 3.0
CFL = 0.4


def _dt_from_handle(mhd, prim, cons, fbx, fby, dx, dy, gamma):
    ny, nx = prim.shape[1:]
    g = Grid2D(ny, nx, dx, dy, 1, 1, gamma, mhd=mhd, recon=2, arith="exact")
    g.upload(prim, cons, fbx, fby)
    t, cyc, _ = g.advance(0.0, 1e30, 0, 1, CFL)
    g.close()
    assert cyc == 1
    return t


def _dt_noalloc(mhd, cons, fbx, fby, dx, dy, gamma):
    import torch
    lib = _lib.load()
    ny, nx = cons.shape[1:]
    dev = torch.device("cuda", torch.cuda.current_device())
    dc = torch.from_numpy(np.ascontiguousarray(cons)).to(dev)
    dbx = torch.from_numpy(np.ascontiguousarray(fbx)).to(dev) if mhd else None
    dby = torch.from_numpy(np.ascontiguousarray(fby)).to(dev) if mhd else None
    out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.mhd2d_cfl_dt_noalloc(1 if mhd else 0, ny, nx, dx, dy, gamma, CFL, dc.data_ptr(),
                                  dbx.data_ptr() if mhd else None, dby.data_ptr() if mhd else None,
                                  out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.mhd2d_strerror(rc)
    torch.cuda.synchronize(dev)
    return float(out.cpu()[0])


def test_noalloc_dt_matches_handle_dt_on_two_calls_in_a_row():
    # call 1: MHD turbulence, 256 x 256
    prim, cons, fbx, fby, dx, dy = ic.turbulence(256, seed=4, gamma=G)
    want1 = _dt_from_handle(True, prim, cons, fbx, fby, dx, dy, G)
    got1 = _dt_noalloc(True, cons, fbx, fby, dx, dy, G)
    assert got1 == want1
    # call 2: hydro blast on a smaller, non-square grid (fewer rows than call 1)
    hp = np.zeros((5, 40, 72))
    hp[0] = 1.0
    hp[4] = 0.1
    hp[4, 15:25, 30:42] = 10.0
    hp[1] = 0.3
    hc = ic.prim_to_cons_hydro(hp, 1.4)
    want2 = _dt_from_handle(False, hp, hc, None, None, 1 / 72, 1 / 40, 1.4)
    got2 = _dt_noalloc(False, hc, None, None, 1 / 72, 1 / 40, 1.4)
    assert got2 == want2


def test_noalloc_dt_is_nan_for_a_state_with_a_nan():
    # the handle's step reports MHD_ERR_NONFINITE on such a state; this entry point
    # must not hide the NaN behind a finite dt
    prim, cons, fbx, fby, dx, dy = ic.turbulence(64, seed=2, gamma=G)
    cons = cons.copy()
    cons[7, 40, 17] = np.nan
    assert np.isnan(_dt_noalloc(True, cons, fbx, fby, dx, dy, G))
    hp = np.ones((5, 24, 32))
    hp[1:4] = 0.1
    hc = ic.prim_to_cons_hydro(hp, 1.4)
    hc[1, 3, 5] = np.nan
    assert np.isnan(_dt_noalloc(False, hc, None, None, 1 / 32, 1 / 24, 1.4))


def test_noalloc_rejects_grids_above_its_row_limit():
    import torch
    lib = _lib.load()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rows = 16384 + 1
    rc = lib.mhd2d_cfl_dt_noalloc(0, rows, 2, 0.1, 0.1, 1.4, CFL, buf.data_ptr(), None, None,
                                  out.data_ptr(), None)
    assert rc == 6  # MHD_ERR_TOO_LARGE, rejected before anything is launched
