"""Digests of long runs of the reference's own evolve functions, for bit-for-bit GPU
checks after hundreds of cycles (the fixtures in ``tests/golden/*.npz`` hold 1-6
cycles each).

    python -B tests/golden/make_long_run_digests.py <PythonMHD checkout>

Writes ``tests/golden/long_run_digests.json``: per run, the final time, the cycle
count and the SHA-256 of the final prim and cons arrays (C-contiguous little-endian
float64).  Each run is also made with the oracle, whose digest must be the same.

Runs (``RUNS``):
* Brio-Wu shock tube, 800 cells, outflow, gamma 2, PPM, to t = 0.1 (``evolve_1D_mhd``);
* Sod shock tube, 800 cells, outflow, gamma 1.4, PPM, to t = 0.2 (``evolve_1D_hydro``);
* a circular blast, 128 x 128 periodic, gamma 1.4, PPM, to t = 0.1 (``evolve_2D_hydro``);
* a cubic blast, 32^3 periodic, gamma 1.4, PPM, to t = 0.1 (``evolve_3D_hydro``).
"""
from __future__ import annotations

import contextlib
import hashlib
import io
import json
import os
import sys
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "long_run_digests.json")
FLOORS = (1e-12, 1e-12, 1e-12)
MAX_CYCLES = 100000


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    return h.hexdigest()


def _brio_wu():
    from tests.golden import cases
    prim, cons = cases._brio_wu(800, gamma=2.0)
    return dict(physics="mhd", dims=1, prim=prim, cons=cons, d=(1.0 / 800,), bc=(0,), gamma=2.0, t_end=0.1)


def _sod():
    from tests.golden import cases
    prim, cons = cases._sod(800, gamma=1.4)
    return dict(physics="hydro", dims=1, prim=prim, cons=cons, d=(1.0 / 800,), bc=(0,), gamma=1.4, t_end=0.2)


def _blast_2d():
    from pythonmhd_gb300 import initial_conditions as ic
    n = 128
    x = (np.arange(n) + 0.5) / n - 0.5
    X, Y = np.meshgrid(x, x)
    prim = np.zeros((5, n, n))
    prim[0] = 1.0
    prim[4] = np.where(X * X + Y * Y < 0.01, 10.0, 0.1)
    return dict(physics="hydro", dims=2, prim=prim, cons=ic.prim_to_cons_hydro(prim, 1.4), d=(1.0 / n, 1.0 / n),
                bc=(1, 1), gamma=1.4, t_end=0.1)


def _blast_3d():
    from tests.golden import cases
    n = 32
    prim, cons = cases._blast_3d(n, n, n, gamma=1.4)
    return dict(physics="hydro", dims=3, prim=prim, cons=cons, d=(1.0 / n,) * 3, bc=(1, 1, 1), gamma=1.4, t_end=0.1)


RUNS = {"brio_wu_1d_800_ppm": _brio_wu, "sod_1d_800_ppm": _sod, "blast_2d_hydro_128_ppm": _blast_2d,
        "blast_3d_hydro_32_ppm": _blast_3d}


def grid_of(run):
    """A grid object with the attributes the reference's evolve functions read."""
    prim = run["prim"]
    g = SimpleNamespace(primVars=prim.copy(), consVars=run["cons"].copy(), dx=run["d"][0], BcX=run["bc"][0],
                        numXCells=prim.shape[-1] if run["dims"] == 1 else prim.shape[2])
    if run["dims"] >= 2:
        g.dy, g.BcY, g.numYCells = run["d"][1], run["bc"][1], prim.shape[1]
    if run["dims"] == 3:
        g.dz, g.BcZ, g.numZCells = run["d"][2], run["bc"][2], prim.shape[3]
    return g


def args_of(run):
    return (0.0, run["t_end"], 0, MAX_CYCLES, run["gamma"], 0.4, *FLOORS, 2, False, 0.5)


def evolve_name(run):
    return f"evolve_{run['dims']}D_{run['physics']}"


def run_reference(ref_root, run):
    sys.path.insert(0, ref_root)
    import Source.EvolveFunctions_Hydro as ref_hydro  # noqa: E402
    import Source.EvolveFunctions_MHD as ref_mhd  # noqa: E402
    mod = ref_mhd if run["physics"] == "mhd" else ref_hydro
    with contextlib.redirect_stdout(io.StringIO()):
        r = getattr(mod, evolve_name(run))(grid_of(run), *args_of(run))
    return {"t": float(r[2]), "cycle": int(r[3]), "sha256": digest(r[0], r[1])}


def run_oracle(run):
    from oracle import evolve1d, hydro2d, hydro3d
    a = args_of(run)
    if run["dims"] == 1:
        fn = evolve1d.evolve_mhd if run["physics"] == "mhd" else evolve1d.evolve_hydro
        r = fn(run["prim"], run["cons"], run["d"][0], run["bc"][0], *a)
    elif run["dims"] == 2:
        r = hydro2d.evolve(run["prim"], run["cons"], *run["d"], *run["bc"], *a)
    else:
        r = hydro3d.evolve(run["prim"], run["cons"], *run["d"], *run["bc"], *a)
    return {"t": float(r[2]), "cycle": int(r[3]), "sha256": digest(r[0], r[1])}


def main(ref_root):
    out = {}
    for name, make in RUNS.items():
        run = make()
        ref = run_reference(ref_root, run)
        orc = run_oracle(run)
        if ref != orc:
            raise SystemExit(f"{name}: the oracle's run differs from the reference's: {orc} vs {ref}")
        out[name] = ref
        print(name, ref, flush=True)
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    sys.dont_write_bytecode = True
    from tests.golden.refpath import reference_root
    main(reference_root())
