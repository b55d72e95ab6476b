"""Generate the golden fixtures by running the reference PythonMHD step itself.

Run in a checkout that has the reference next to it (the fixtures are committed,
so the tests do not need the reference):

    python -B tests/golden/make_golden.py <PythonMHD checkout> [2d|1d|3d|all]

(or set ``PYTHONMHD_REFERENCE`` to the checkout)

For every case in ``tests/golden/cases.py`` (2D; the 1D cases with
``evolve_1D_mhd`` / ``evolve_1D_hydro``; the 3D cases with ``evolve_3D_hydro``) this imports the reference's own
``Source.EvolveFunctions_MHD.evolve_2D_mhd`` / ``Source.EvolveFunctions_Hydro.evolve_2D_hydro``
(which depend only on NumPy), calls it on a minimal grid object carrying the
attributes the reference reads (Source/EvolveFunctions_MHD.py:396-444,
Source/EvolveFunctions_Hydro.py:353-376), and stores inputs, parameters and the
returned tuple in ``tests/golden/<physics>_<case>.npz``.
"""
from __future__ import annotations

import contextlib
import io
import os
import sys
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.dont_write_bytecode = True

from tests.golden import cases  # noqa: E402

SCALARS = ("t_start", "t_end", "start_cycle", "max_cycles", "gamma", "cfl", "min_d", "min_p",
           "min_e", "order", "efix", "eps", "bcx", "bcy", "dx", "dy")


def run_reference(ref_root, physics, case):
    sys.path.insert(0, ref_root)
    import Source.EvolveFunctions_Hydro as ref_hydro  # noqa: E402
    import Source.EvolveFunctions_MHD as ref_mhd  # noqa: E402
    ny, nx = case["prim"].shape[1:]
    grid = SimpleNamespace(primVars=case["prim"].copy(), consVars=case["cons"].copy(),
                           dx=case["dx"], dy=case["dy"], BcX=case["bcx"], BcY=case["bcy"],
                           numXCells=nx, numYCells=ny)
    args = (grid, case["t_start"], case["t_end"], case["start_cycle"], case["max_cycles"],
            case["gamma"], case["cfl"], case["min_d"], case["min_p"], case["min_e"],
            case["order"], case["efix"], case["eps"])
    with contextlib.redirect_stdout(io.StringIO()):
        if physics == "mhd":
            grid.faceBx = case["fbx"].copy()
            grid.faceBy = case["fby"].copy()
            res = ref_mhd.evolve_2D_mhd(*args)
            keys = ("prim", "cons", "fbx", "fby", "t", "cycle", "sl_prim", "sl_cons", "sl_fbx",
                    "sl_fby", "sl_t")
        else:
            res = ref_hydro.evolve_2D_hydro(*args)
            keys = ("prim", "cons", "t", "cycle", "sl_prim", "sl_cons", "sl_t")
    return {"out_" + k: np.asarray(v) for k, v in zip(keys, res)}


SCALARS_1D = ("t_start", "t_end", "start_cycle", "max_cycles", "gamma", "cfl", "min_d", "min_p",
              "min_e", "order", "efix", "eps", "bcx", "dx")


def run_reference_1d(ref_root, physics, case):
    """evolve_1D_mhd / evolve_1D_hydro (Source/EvolveFunctions_MHD.py:195-340,
    Source/EvolveFunctions_Hydro.py:232-305) on a grid object with the attributes they read."""
    sys.path.insert(0, ref_root)
    import Source.EvolveFunctions_Hydro as ref_hydro  # noqa: E402
    import Source.EvolveFunctions_MHD as ref_mhd  # noqa: E402
    grid = SimpleNamespace(primVars=case["prim"].copy(), consVars=case["cons"].copy(), dx=case["dx"],
                           BcX=case["bcx"], numXCells=case["prim"].shape[1])
    args = (grid, case["t_start"], case["t_end"], case["start_cycle"], case["max_cycles"], case["gamma"],
            case["cfl"], case["min_d"], case["min_p"], case["min_e"], case["order"], case["efix"], case["eps"])
    with contextlib.redirect_stdout(io.StringIO()):
        fn = ref_mhd.evolve_1D_mhd if physics == "mhd" else ref_hydro.evolve_1D_hydro
        res = fn(*args)
    keys = ("prim", "cons", "t", "cycle", "sl_prim", "sl_cons", "sl_t")
    return {"out_" + k: np.asarray(v) for k, v in zip(keys, res)}


def main_1d(ref_root):
    for physics in ("mhd", "hydro"):
        for name in cases.names1d(physics):
            case = cases.build1d(physics, name)
            outs = run_reference_1d(ref_root, physics, case)
            arrays = {"in_prim": case["prim"], "in_cons": case["cons"]}
            for k in SCALARS_1D:
                arrays["p_" + k] = np.asarray(case[k])
            arrays.update(outs)
            path = os.path.join(HERE, f"{physics}1d_{name}.npz")
            np.savez_compressed(path, **arrays)
            print(f"{path}: cycles={int(outs['out_cycle'])} t={float(outs['out_t']):.6g}")


SCALARS_3D = ("t_start", "t_end", "start_cycle", "max_cycles", "gamma", "cfl", "min_d", "min_p",
              "min_e", "order", "efix", "eps", "bcx", "bcy", "bcz", "dx", "dy", "dz")


def run_reference_3d(ref_root, physics, case):
    """evolve_3D_hydro / evolve_3D_mhd (Source/EvolveFunctions_Hydro.py:559-806,
    Source/EvolveFunctions_MHD.py:750-1157) on a grid object with the attributes they read."""
    sys.path.insert(0, ref_root)
    import Source.EvolveFunctions_Hydro as ref_hydro  # noqa: E402
    import Source.EvolveFunctions_MHD as ref_mhd  # noqa: E402
    ny, nx, nz = case["prim"].shape[1:]
    grid = SimpleNamespace(primVars=case["prim"].copy(), consVars=case["cons"].copy(), dx=case["dx"],
                           dy=case["dy"], dz=case["dz"], BcX=case["bcx"], BcY=case["bcy"], BcZ=case["bcz"],
                           numXCells=nx, numYCells=ny, numZCells=nz)
    args = (grid, case["t_start"], case["t_end"], case["start_cycle"], case["max_cycles"], case["gamma"],
            case["cfl"], case["min_d"], case["min_p"], case["min_e"], case["order"], case["efix"], case["eps"])
    with contextlib.redirect_stdout(io.StringIO()):
        if physics == "mhd":
            grid.faceBx, grid.faceBy, grid.faceBz = case["fbx"].copy(), case["fby"].copy(), case["fbz"].copy()
            res = ref_mhd.evolve_3D_mhd(*args)
            keys = ("prim", "cons", "fbx", "fby", "fbz", "t", "cycle", "sl_prim", "sl_cons", "sl_fbx", "sl_fby",
                    "sl_fbz", "sl_t")
        else:
            res = ref_hydro.evolve_3D_hydro(*args)
            keys = ("prim", "cons", "t", "cycle", "sl_prim", "sl_cons", "sl_t")
    return {"out_" + k: np.asarray(v) for k, v in zip(keys, res)}


def main_3d(ref_root):
    for physics in ("hydro", "mhd"):
        for name in cases.names3d(physics):
            case = cases.build3d(physics, name)
            outs = run_reference_3d(ref_root, physics, case)
            arrays = {"in_prim": case["prim"], "in_cons": case["cons"]}
            if physics == "mhd":
                arrays.update(in_fbx=case["fbx"], in_fby=case["fby"], in_fbz=case["fbz"])
            for k in SCALARS_3D:
                arrays["p_" + k] = np.asarray(case[k])
            arrays.update(outs)
            path = os.path.join(HERE, f"{physics}3d_{name}.npz")
            np.savez_compressed(path, **arrays)
            print(f"{path}: cycles={int(outs['out_cycle'])} t={float(outs['out_t']):.6g}")


def main(ref_root):
    for physics in ("mhd", "hydro"):
        for name in cases.names(physics):
            case = cases.build(physics, name)
            outs = run_reference(ref_root, physics, case)
            arrays = {"in_prim": case["prim"], "in_cons": case["cons"]}
            if physics == "mhd":
                arrays.update(in_fbx=case["fbx"], in_fby=case["fby"])
            for k in SCALARS:
                arrays["p_" + k] = np.asarray(case[k])
            arrays.update(outs)
            path = os.path.join(HERE, f"{physics}_{name}.npz")
            np.savez_compressed(path, **arrays)
            print(f"{path}: cycles={int(outs['out_cycle'])} t={float(outs['out_t']):.6g}")


if __name__ == "__main__":
    # make_golden.py <reference root> [2d|1d|3d|all]
    from tests.golden.refpath import reference_root
    root = reference_root()
    which = sys.argv[2] if len(sys.argv) > 2 else "all"
    if which in ("2d", "all"):
        main(root)
    if which in ("1d", "all"):
        main_1d(root)
    if which in ("3d", "all"):
        main_3d(root)
