"""A 40-cycle run of the reference's own ``evolve_3D_mhd`` (the 3D MHD fixtures in
``tests/golden/mhd3d_*.npz`` hold 1-6 cycles each).

    python -B tests/golden/make_mhd3d_long.py <PythonMHD checkout>

State: ``cases._random_mhd_3d(10, 10, 10, seed=71)`` (smooth random flow, rms Mach
~0.6, divergence-free face B), periodic in x, y and z, gamma 5/3, PPM, the entropy
fix on (``evolve_3D_mhd``'s default), CFL 0.4.  Writes the final prim, cons, faceBx,
faceBy, faceBz, time and cycle to ``tests/golden/long_run_mhd3d_10.npz``.

The reference computes part of its transverse predictor in long double, so a FP64
step agrees with it to rounding, not bit for bit: after the 40 cycles the oracle's
FP64-predictor form differs from it by at most 1.1e-13 relative per field.
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

OUT = os.path.join(HERE, "long_run_mhd3d_10.npz")
N, SEED, CYCLES = 10, 71, 40
# (t_start, t_end, start_cycle, max_cycles, gamma, cfl, min_d, min_p, min_e, order, efix, eps)
ARGS = (0.0, 1e30, 0, CYCLES, 5.0 / 3.0, 0.4, 1e-12, 1e-12, 1e-12, 2, True, 0.5)
KEYS = ("prim", "cons", "fbx", "fby", "fbz", "t", "cycle")


def initial_state():
    from tests.golden import cases
    return cases._random_mhd_3d(N, N, N, SEED)


def grid_of(prim, cons, fbx, fby, fbz, dx, dy, dz):
    return SimpleNamespace(primVars=prim.copy(), consVars=cons.copy(), faceBx=fbx.copy(), faceBy=fby.copy(),
                           faceBz=fbz.copy(), dx=dx, dy=dy, dz=dz, BcX=1, BcY=1, BcZ=1, numXCells=N,
                           numYCells=N, numZCells=N)


def main(ref_root):
    sys.path.insert(0, ref_root)
    import Source.EvolveFunctions_MHD as ref_mhd  # noqa: E402
    with contextlib.redirect_stdout(io.StringIO()):
        r = ref_mhd.evolve_3D_mhd(grid_of(*initial_state()), *ARGS)
    np.savez_compressed(OUT, **{k: np.asarray(v) for k, v in zip(KEYS, r[:7])})
    print("t", r[5], "cycle", r[6])


if __name__ == "__main__":
    sys.dont_write_bytecode = True
    from tests.golden.refpath import reference_root
    main(reference_root())
