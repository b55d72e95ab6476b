"""Drop-in replacements for the reference's 1D and 2D evolve functions.

``evolve_2D_mhd`` and ``evolve_2D_hydro`` keep the reference signatures, the
preconditions they assert, their return tuples and their aliasing:

* Source/EvolveFunctions_MHD.py:393-697  evolve_2D_mhd(simulationGrid, tStart, tEnd,
  startCycle, maxCycles, gamma, cfl, minDens, minPres, minEnergy,
  reconstructOrder=0, entropyFix=False, epsilon=0.5)
  -> (prim, cons, faceBx, faceBy, time, cycle, secondLastPrim, secondLastCons,
      secondLastFaceBx, secondLastFaceBy, secondLastTime);
  faceBx/faceBy are updated in place in the grid's arrays and returned,
  prim/cons are new arrays (the grid's own objects when no cycle runs).
* Source/EvolveFunctions_Hydro.py:350-516 evolve_2D_hydro(...) (same arguments)
  -> (prim, cons, time, cycle, secondLastPrim, secondLastCons, secondLastTime);
  the grid's primVars/consVars are updated in place and returned.

``evolve_1D_mhd`` / ``evolve_1D_hydro`` (Source/EvolveFunctions_MHD.py:195-340,
Source/EvolveFunctions_Hydro.py:232-305) keep theirs too: the 1D MHD function
returns new arrays with B_x made uniform; the 1D hydro function updates the
grid's arrays in place and returns them.  ``evolve_3D_hydro``
(Source/EvolveFunctions_Hydro.py:559-806) updates the grid's (5, ny, nx, nz)
arrays in place and returns them, and ``evolve_3D_mhd``
(Source/EvolveFunctions_MHD.py:750-1157) returns new prim/cons arrays and updates
the three face-B arrays in place, as the reference does.

The cycles run on the GPU (``Grid2D.advance``); the host uploads the grid once
per call and downloads the result.  Handles are cached per grid geometry and
parameters, so the driver's repeated calls reuse device memory and CUDA graphs.
"""
from __future__ import annotations

import numpy as np

from .solver import Grid1D, Grid2D, Grid3D, default_arith

OUTFLOW = 0
PERIODIC = 1
# reconstructOrder value that selects PLM, an addition: the reference runs PPM for
# reconstructOrder == 2 and first order for every other value (its PLM branches are
# commented out, Source/EvolveFunctions_MHD.py:487-488, Source/EvolveFunctions_Hydro.py:
# 410-412), so an integer other than 2 keeps the reference's first-order behaviour.
PLM = "plm"


def _order(reconstructOrder):
    if reconstructOrder == PLM:
        return 1
    return 2 if reconstructOrder == 2 else 0

_cache: dict = {}
_CACHE_MAX = 4


def _handle(key, make):
    h = _cache.get(key)
    if h is None:
        while len(_cache) >= _CACHE_MAX:
            _cache.pop(next(iter(_cache))).close()
        h = make()
        _cache[key] = h
    return h


def clear_cache():
    while _cache:
        _cache.popitem()[1].close()


def evolve_2D_mhd(simulationGrid, tStart, tEnd, startCycle, maxCycles, gamma, cfl, minDens, minPres,
                  minEnergy, reconstructOrder=0, entropyFix=False, epsilon=0.5, arith=None):
    prim = simulationGrid.primVars
    bcx = simulationGrid.BcX
    assert (bcx == OUTFLOW or bcx == PERIODIC)
    bcy = simulationGrid.BcY
    assert (bcy == OUTFLOW or bcy == PERIODIC)
    assert (len(prim.shape) == 3)
    assert (prim.shape[0] == 8)
    assert (prim.shape[1] > 0)
    fbx = simulationGrid.faceBx
    fby = simulationGrid.faceBy
    cons = simulationGrid.consVars
    assert (prim.shape == cons.shape)
    dx = simulationGrid.dx
    assert (dx > 0)
    dy = simulationGrid.dy
    assert (dy > 0)
    assert (tStart <= tEnd)
    assert (startCycle >= 0)
    ny, nx = prim.shape[1:]
    order = _order(reconstructOrder)
    mode = arith or default_arith()
    key = ("mhd", ny, nx, float(dx), float(dy), bcx, bcy, float(gamma), order, bool(entropyFix),
           float(epsilon), float(minDens), float(minPres), float(minEnergy), mode)
    g = _handle(key, lambda: Grid2D(ny, nx, dx, dy, bcx, bcy, gamma, mhd=True, recon=order,
                                    entropy_fix=entropyFix, eps=epsilon, min_d=minDens, min_p=minPres,
                                    min_e=minEnergy, arith=mode))
    g.upload(prim, cons, fbx, fby)
    t, cyc, t_sl = g.advance(tStart, tEnd, startCycle, maxCycles, cfl)
    if g.last_cycles == 0:
        return (prim, cons, fbx, fby, tStart, startCycle, np.copy(prim), np.copy(cons), np.copy(fbx),
                np.copy(fby), tStart)
    new_prim, new_cons, new_fbx, new_fby = g.download(0)
    sl_prim, sl_cons, sl_fbx, sl_fby = g.download(1)
    np.copyto(fbx, new_fbx)
    np.copyto(fby, new_fby)
    return (new_prim, new_cons, fbx, fby, t, cyc, sl_prim, sl_cons, sl_fbx, sl_fby, t_sl)


def evolve_2D_hydro(simulationGrid, tStart, tEnd, startCycle, maxCycles, gamma, cfl, minDens, minPres,
                    minEnergy, reconstructOrder=0, entropyFix=False, epsilon=0.5, arith=None):
    prim = simulationGrid.primVars
    assert (len(prim.shape) == 3)
    cons = simulationGrid.consVars
    assert (prim.shape == cons.shape)
    nx = simulationGrid.numXCells
    assert (nx > 1)
    ny = simulationGrid.numYCells
    assert (ny > 1)
    dx = simulationGrid.dx
    assert (dx > 0)
    dy = simulationGrid.dy
    assert (dy > 0)
    bcx = simulationGrid.BcX
    assert (bcx == OUTFLOW or bcx == PERIODIC)
    bcy = simulationGrid.BcY
    assert (bcy == OUTFLOW or bcy == PERIODIC)
    assert (tStart <= tEnd)
    assert (startCycle >= 0 and maxCycles > 0)
    order = _order(reconstructOrder)
    mode = arith or default_arith()
    key = ("hydro", ny, nx, float(dx), float(dy), bcx, bcy, float(gamma), order, bool(entropyFix),
           float(epsilon), float(minDens), float(minPres), float(minEnergy), mode)
    g = _handle(key, lambda: Grid2D(ny, nx, dx, dy, bcx, bcy, gamma, mhd=False, recon=order,
                                    entropy_fix=entropyFix, eps=epsilon, min_d=minDens, min_p=minPres,
                                    min_e=minEnergy, arith=mode))
    g.upload(prim, cons)
    t, cyc, t_sl = g.advance(tStart, tEnd, startCycle, maxCycles, cfl)
    if g.last_cycles == 0:
        return prim, cons, tStart, startCycle, np.copy(prim), np.copy(cons), tStart
    sl_prim, sl_cons = g.download(1)
    new_prim, new_cons = g.download(0)
    np.copyto(prim, new_prim)
    np.copyto(cons, new_cons)
    return prim, cons, t, cyc, sl_prim, sl_cons, t_sl


# ---------------------------------------------------------------------------
# 1D (Source/EvolveFunctions_MHD.py:195-340, Source/EvolveFunctions_Hydro.py:232-305)
# ---------------------------------------------------------------------------
def evolve_1D_mhd(simulationGrid, tStart, tEnd, startCycle, maxCycles, gamma, cfl, minDens, minPres,
                  minEnergy, reconstructOrder=0, entropyFix=False, epsilon=0.5, arith=None):
    """evolve_1D_mhd: returns (prim, cons, time, cycle, secondLastPrim, secondLastCons,
    secondLastTime) as new arrays (the grid's arrays are not modified); B_x is the
    first cell's value everywhere, as in the reference."""
    prim = simulationGrid.primVars
    assert (len(prim.shape) == 2)
    assert (prim.shape[0] == 8)
    assert (prim.shape[1] > 0)
    cons = simulationGrid.consVars
    assert (prim.shape == cons.shape)
    dx = simulationGrid.dx
    assert (dx > 0)
    bcx = simulationGrid.BcX
    assert (bcx == OUTFLOW or bcx == PERIODIC)
    assert (tStart <= tEnd)
    assert (startCycle >= 0)
    n = prim.shape[1]
    order = _order(reconstructOrder)
    mode = arith or default_arith()
    key = ("mhd1d", n, float(dx), bcx, float(gamma), order, bool(entropyFix), float(epsilon), float(minDens),
           float(minPres), float(minEnergy), mode)
    g = _handle(key, lambda: Grid1D(n, dx, bcx, gamma, mhd=True, recon=order, entropy_fix=entropyFix,
                                    eps=epsilon, min_d=minDens, min_p=minPres, min_e=minEnergy, arith=mode))
    g.upload(prim, cons)
    t, cycle, t_sl = g.advance(tStart, tEnd, startCycle, maxCycles, cfl)
    new_prim, new_cons = g.download(0)
    if g.last_cycles > 0:
        sl_prim, sl_cons = g.download(1)
    else:
        sl_prim, sl_cons = np.copy(prim), np.copy(cons)
        # with no cycle the reference still returns B_x made uniform
        new_prim = np.array(prim, dtype=np.float64)
        new_cons = np.array(cons, dtype=np.float64)
        new_prim[4] = prim[4][0]
        new_cons[4] = prim[4][0]
    return new_prim, new_cons, t, cycle, sl_prim, sl_cons, t_sl


def evolve_1D_hydro(simulationGrid, tStart, tEnd, startCycle, maxCycles, gamma, cfl, minDens, minPres,
                    minEnergy, reconstructOrder=0, entropyFix=False, epsilon=0.5, arith=None):
    """evolve_1D_hydro: updates the grid's primVars/consVars in place and returns them,
    as the reference does: (prim, cons, time, cycle, secondLastPrim, secondLastCons,
    secondLastTime)."""
    prim = simulationGrid.primVars
    assert (len(prim.shape) == 2)
    cons = simulationGrid.consVars
    assert (prim.shape == cons.shape)
    dx = simulationGrid.dx
    assert (dx > 0)
    bcx = simulationGrid.BcX
    assert (bcx == OUTFLOW or bcx == PERIODIC)
    assert (tEnd >= tStart)
    assert (startCycle >= 0 and maxCycles > 0)
    n = prim.shape[1]
    order = _order(reconstructOrder)
    mode = arith or default_arith()
    key = ("hydro1d", n, float(dx), bcx, float(gamma), order, bool(entropyFix), float(epsilon),
           float(minDens), float(minPres), float(minEnergy), mode)
    g = _handle(key, lambda: Grid1D(n, dx, bcx, gamma, mhd=False, recon=order, entropy_fix=entropyFix,
                                    eps=epsilon, min_d=minDens, min_p=minPres, min_e=minEnergy, arith=mode))
    g.upload(prim, cons)
    t, cycle, t_sl = g.advance(tStart, tEnd, startCycle, maxCycles, cfl)
    if g.last_cycles > 0:
        sl_prim, sl_cons = g.download(1)
        g.download(0, prim, cons)
    else:
        sl_prim, sl_cons = np.copy(prim), np.copy(cons)
    return prim, cons, t, cycle, sl_prim, sl_cons, t_sl


# ---------------------------------------------------------------------------
# 3D hydro (Source/EvolveFunctions_Hydro.py:559-806)
# ---------------------------------------------------------------------------
def evolve_3D_hydro(simulationGrid, tStart, tEnd, startCycle, maxCycles, gamma, cfl, minDens, minPres,
                    minEnergy, reconstructOrder=0, entropyFix=False, epsilon=0.5, arith=None):
    """evolve_3D_hydro: updates the grid's primVars/consVars, (5, ny, nx, nz), in place
    and returns them: (prim, cons, time, cycle, secondLastPrim, secondLastCons,
    secondLastTime).  reconstructOrder 2 is PPM, :data:`PLM` is PLM, anything else
    first order, as in 2D."""
    prim = simulationGrid.primVars
    assert (len(prim.shape) - 1 == 3)
    cons = simulationGrid.consVars
    assert (prim.shape == cons.shape)
    nx = simulationGrid.numXCells
    assert (nx > 1)
    ny = simulationGrid.numYCells
    assert (ny > 1)
    nz = simulationGrid.numZCells
    assert (nz > 1)
    dx = simulationGrid.dx
    assert (dx > 0)
    dy = simulationGrid.dy
    assert (dy > 0)
    dz = simulationGrid.dz
    assert (dz > 0)
    bcx = simulationGrid.BcX
    assert (bcx == OUTFLOW or bcx == PERIODIC)
    bcy = simulationGrid.BcY
    assert (bcy == OUTFLOW or bcy == PERIODIC)
    bcz = simulationGrid.BcZ
    assert (bcz == OUTFLOW or bcz == PERIODIC)
    assert (tStart <= tEnd)
    assert (startCycle >= 0 and maxCycles > 0)
    order = _order(reconstructOrder)
    mode = arith or default_arith()
    key = ("hydro3d", ny, nx, nz, float(dx), float(dy), float(dz), bcx, bcy, bcz, float(gamma), order,
           bool(entropyFix), float(epsilon), float(minDens), float(minPres), float(minEnergy), mode)
    g = _handle(key, lambda: Grid3D(ny, nx, nz, dx, dy, dz, bcx, bcy, bcz, gamma, recon=order,
                                    entropy_fix=entropyFix, eps=epsilon, min_d=minDens, min_p=minPres,
                                    min_e=minEnergy, arith=mode))
    g.upload(prim, cons)
    t, cyc, t_sl = g.advance(tStart, tEnd, startCycle, maxCycles, cfl)
    if g.last_cycles == 0:
        return prim, cons, tStart, startCycle, np.copy(prim), np.copy(cons), tStart
    sl_prim, sl_cons = g.download(1)
    new_prim, new_cons = g.download(0)
    np.copyto(prim, new_prim)
    np.copyto(cons, new_cons)
    return prim, cons, t, cyc, sl_prim, sl_cons, t_sl


# ---------------------------------------------------------------------------
# 3D MHD (Source/EvolveFunctions_MHD.py:750-1157)
# ---------------------------------------------------------------------------
def evolve_3D_mhd(simulationGrid, tStart, tEnd, startCycle, maxCycles, gamma, cfl, minDens, minPres,
                  minEnergy, reconstructOrder=0, entropyFix=True, epsilon=0.5, arith=None):
    """evolve_3D_mhd: returns (prim, cons, faceBx, faceBy, faceBz, time, cycle,
    secondLastPrim, secondLastCons, secondLastFaceBx, secondLastFaceBy,
    secondLastFaceBz, secondLastTime); the face arrays are the grid's own, updated in
    place, and prim/cons are new arrays (the grid's own when no cycle runs), as in
    the reference.  Its entropy fix defaults to on, as the reference's does."""
    prim = simulationGrid.primVars
    bcx = simulationGrid.BcX
    assert (bcx == OUTFLOW or bcx == PERIODIC)
    bcy = simulationGrid.BcY
    assert (bcy == OUTFLOW or bcy == PERIODIC)
    bcz = simulationGrid.BcZ
    assert (bcz == OUTFLOW or bcz == PERIODIC)
    assert (len(prim.shape) == 4)
    assert (prim.shape[0] == 8)
    assert (prim.shape[1] > 0)
    fbx = simulationGrid.faceBx
    fby = simulationGrid.faceBy
    fbz = simulationGrid.faceBz
    cons = simulationGrid.consVars
    assert (prim.shape == cons.shape)
    dx = simulationGrid.dx
    assert (dx > 0)
    dy = simulationGrid.dy
    assert (dy > 0)
    dz = simulationGrid.dz
    assert (dz > 0)
    assert (tStart <= tEnd)
    assert (startCycle >= 0)
    ny, nx, nz = prim.shape[1:]
    order = _order(reconstructOrder)
    mode = arith or default_arith()
    key = ("mhd3d", ny, nx, nz, float(dx), float(dy), float(dz), bcx, bcy, bcz, float(gamma), order,
           bool(entropyFix), float(epsilon), float(minDens), float(minPres), float(minEnergy), mode)
    g = _handle(key, lambda: Grid3D(ny, nx, nz, dx, dy, dz, bcx, bcy, bcz, gamma, recon=order,
                                    entropy_fix=entropyFix, eps=epsilon, min_d=minDens, min_p=minPres,
                                    min_e=minEnergy, arith=mode, mhd=True))
    g.upload(prim, cons, fbx, fby, fbz)
    t, cyc, t_sl = g.advance(tStart, tEnd, startCycle, maxCycles, cfl)
    if g.last_cycles == 0:
        return (prim, cons, fbx, fby, fbz, tStart, startCycle, np.copy(prim), np.copy(cons), np.copy(fbx),
                np.copy(fby), np.copy(fbz), tStart)
    new_prim, new_cons, nbx, nby, nbz = g.download(0)
    sl = g.download(1)
    np.copyto(fbx, nbx)
    np.copyto(fby, nby)
    np.copyto(fbz, nbz)
    return (new_prim, new_cons, fbx, fby, fbz, t, cyc) + tuple(sl) + (t_sl,)
