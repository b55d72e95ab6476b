"""Digests of full-length Orszag-Tang runs: 128 x 128 periodic, gamma = 5/3, CFL 0.4,
from t = 0 to t = 0.5 (about 400 cycles), the workload of the plain CPU-runnable
configuration.

    python -B tests/golden/make_ot128_digests.py [<PythonMHD checkout>]

Writes ``tests/golden/ot128_t05_digests.json`` with, per run, the final time, the
cycle count and the SHA-256 of the final prim, cons, faceBx and faceBy arrays
(C-contiguous little-endian float64):

* ``reference_ppm``: the reference's own ``evolve_2D_mhd`` (reconstructOrder 2,
  PPM), when the reference's root is given;
* ``oracle_ppm``: the oracle's restatement of the same run (must equal the
  reference's digest);
* ``oracle_plm``: the oracle with PLM, which the reference does not have.

A GPU test compares the digests of the same runs through ``evolve_2D_mhd``: equal
digests mean bit-for-bit equal states after the whole run.
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

OUT = os.path.join(HERE, "ot128_t05_digests.json")
N, GAMMA, CFL, T_END, MAX_CYCLES = 128, 5.0 / 3.0, 0.4, 0.5, 100000
FLOORS = (1e-12, 1e-12, 1e-12)


def digest(prim, cons, fbx, fby):
    h = hashlib.sha256()
    for a in (prim, cons, fbx, fby):
        h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    return h.hexdigest()


def initial_state():
    from pythonmhd_gb300 import initial_conditions as ic
    return ic.orszag_tang(N, N, gamma=GAMMA)


def run_oracle(order):
    from oracle import mhd2d
    prim, cons, fbx, fby, dx, dy = initial_state()
    r = mhd2d.evolve(prim, cons, fbx, fby, dx, dy, 1, 1, 0.0, T_END, 0, MAX_CYCLES, GAMMA, CFL, *FLOORS, order,
                     False, 0.5)
    return {"t": float(r[4]), "cycle": int(r[5]), "sha256": digest(*r[:4])}


def run_reference(ref_root):
    sys.path.insert(0, ref_root)
    import Source.EvolveFunctions_MHD as ref_mhd  # noqa: E402
    prim, cons, fbx, fby, dx, dy = initial_state()
    grid = SimpleNamespace(primVars=prim.copy(), consVars=cons.copy(), faceBx=fbx.copy(), faceBy=fby.copy(),
                           dx=dx, dy=dy, BcX=1, BcY=1, numXCells=N, numYCells=N)
    with contextlib.redirect_stdout(io.StringIO()):
        r = ref_mhd.evolve_2D_mhd(grid, 0.0, T_END, 0, MAX_CYCLES, GAMMA, CFL, *FLOORS, 2, False, 0.5)
    return {"t": float(r[4]), "cycle": int(r[5]), "sha256": digest(*r[:4])}


def main(ref_root=None):
    out = {"workload": f"Orszag-Tang {N}x{N} periodic, gamma 5/3, CFL {CFL}, t 0 -> {T_END}, no entropy fix"}
    out["oracle_ppm"] = run_oracle(2)
    out["oracle_plm"] = run_oracle(1)
    if ref_root:
        out["reference_ppm"] = run_reference(ref_root)
        if out["reference_ppm"] != out["oracle_ppm"]:
            raise SystemExit("the oracle's PPM run differs from the reference's")
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    sys.dont_write_bytecode = True
    from tests.golden.refpath import reference_root
    main(reference_root(required=False))
