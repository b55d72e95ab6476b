"""Time the reference's own NumPy step beside the oracle's restatement of it.

    python -B oracle/calibrate_port.py <PythonMHD checkout> [n] [cycles]

(or set ``PYTHONMHD_REFERENCE``).  TEST AND MEASUREMENT INFRASTRUCTURE ONLY: the
benchmark's reference arm and CPU baseline run the oracle (the reference cannot be
installed on the GPU hosts), so this script records how the oracle's speed stands
against the reference's own ``Source.EvolveFunctions_MHD.evolve_2D_mhd`` on one
core of the same host, on the same state (the benchmark's seeded turbulence
generator, PPM, CFL 0.4), and checks that both end bit for bit equal.  Prints one
JSON line.
"""
from __future__ import annotations

import contextlib
import io
import json
import os
import sys
import time
from types import SimpleNamespace

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main(ref_root, n=256, cycles=3):
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_root)
    import Source.EvolveFunctions_MHD as ref  # noqa: E402

    from oracle import mhd2d
    from pythonmhd_gb300 import initial_conditions as ic
    prim, cons, fbx, fby, dx, dy = ic.turbulence(n, seed=7, gamma=5.0 / 3.0)
    args = (0.0, 1e30, 0, cycles, 5.0 / 3.0, 0.4, 1e-12, 1e-12, 1e-12, 2, False, 0.5)
    out = {}
    for name in ("reference", "oracle", "reference_again", "oracle_again"):
        grid = SimpleNamespace(primVars=prim.copy(), consVars=cons.copy(), faceBx=fbx.copy(), faceBy=fby.copy(),
                               dx=dx, dy=dy, BcX=1, BcY=1, numXCells=n, numYCells=n)
        t0 = time.perf_counter()
        if name.startswith("reference"):
            with contextlib.redirect_stdout(io.StringIO()):
                r = ref.evolve_2D_mhd(grid, *args)
        else:
            r = mhd2d.evolve(prim, cons, fbx, fby, dx, dy, 1, 1, *args)
        out[name] = (time.perf_counter() - t0, r)
    same = all(np.array_equal(a, b) for a, b in zip(out["reference"][1][:4], out["oracle"][1][:4]))
    t_ref = min(out["reference"][0], out["reference_again"][0]) / cycles
    t_orc = min(out["oracle"][0], out["oracle_again"][0]) / cycles
    print(json.dumps({"workload": f"2D MHD turbulence {n}x{n}, PPM, CFL 0.4, {cycles} cycles, 1 core",
                      "reference_s_per_cycle": t_ref, "oracle_s_per_cycle": t_orc,
                      "reference_zone_updates_per_s": n * n / t_ref, "oracle_zone_updates_per_s": n * n / t_orc,
                      "oracle_over_reference_speed": t_ref / t_orc, "bitwise_equal": same,
                      "numpy": np.__version__, "cpu": os.uname().machine}))


if __name__ == "__main__":
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    sys.path.insert(0, ROOT)
    from tests.golden.refpath import reference_root
    root = reference_root()
    main(root, *(int(a) for a in sys.argv[2:4]))
