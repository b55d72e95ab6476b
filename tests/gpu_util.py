"""Helpers for the GPU parity tests: run a golden case through the drop-in."""
from types import SimpleNamespace

import numpy as np

from pythonmhd_gb300 import evolve


def make_grid(p, i):
    ny, nx = i["prim"].shape[1:]
    g = SimpleNamespace(primVars=i["prim"].copy(), consVars=i["cons"].copy(), dx=p["dx"], dy=p["dy"],
                        BcX=p["bcx"], BcY=p["bcy"], numXCells=nx, numYCells=ny)
    if "fbx" in i:
        g.faceBx = i["fbx"].copy()
        g.faceBy = i["fby"].copy()
    return g


def run_dropin(physics, p, i, arith):
    g = make_grid(p, i)
    fn = evolve.evolve_2D_mhd if physics == "mhd" else evolve.evolve_2D_hydro
    res = fn(g, p["t_start"], p["t_end"], p["start_cycle"], p["max_cycles"], p["gamma"], p["cfl"],
             p["min_d"], p["min_p"], p["min_e"], p["order"], p["efix"], p["eps"], arith=arith)
    return g, res


def field_rel_err(a, b):
    """max |a-b| / max(|b|) per field (a field-scaled relative error)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.ndim == 0:
        return abs(float(a) - float(b)) / max(abs(float(b)), 1e-300)
    if a.ndim == 3:
        return max(field_rel_err(x, y) for x, y in zip(a, b))
    scale = np.max(np.abs(b))
    if scale == 0.0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / scale)
