"""Floor counts of the reference's own evolve functions on the golden cases.

    python -B tests/golden/make_floor_counts.py <PythonMHD checkout>

(or set ``PYTHONMHD_REFERENCE``).  For every 2D and 1D fixture in
``tests/golden/*.npz`` this runs the reference's ``evolve_2D_*`` / ``evolve_1D_*``
on the fixture's input with the reference's floor routine
(``Source.PrimCons_HelperModule.applyFloors``, Source/PrimCons_HelperModule.py:499-554)
wrapped so that each call adds the number of values it raises -- the
``numLowValues`` its discarded warning reports -- to a tally.  Writes
``tests/golden/floor_counts.json``: case -> count.  The oracle's tally must give
the same numbers (tests/test_oracle_golden.py); the GPU's mhd2d_stats must give
the oracle's (tests/test_gpu_failure_counters.py).
"""
import contextlib
import io
import json
import os
import sys
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.dont_write_bytecode = True

from tests.golden_io import case_id, golden_files, load  # noqa: E402

OUT = os.path.join(HERE, "floor_counts.json")


def main(ref_root):
    sys.path.insert(0, ref_root)
    import Source.EvolveFunctions_Hydro as ref_hydro  # noqa: E402
    import Source.EvolveFunctions_MHD as ref_mhd  # noqa: E402
    import Source.PrimCons_HelperModule as pc  # noqa: E402
    tally = [0]
    original = pc.applyFloors

    def counting(vars, isPrimitive, minDens, minPres, minEnergy, calledFromString):
        last = minPres if isPrimitive else minEnergy
        tally[0] += int(np.count_nonzero(vars[0] < minDens)) + int(np.count_nonzero(vars[-1] < last))
        return original(vars, isPrimitive, minDens, minPres, minEnergy, calledFromString)

    pc.applyFloors = counting
    out = {}
    for f in golden_files("mhd") + golden_files("hydro") + golden_files("mhd1d") + golden_files("hydro1d"):
        name = case_id(f)
        p, i, _ = load(f)
        one_d = "1d" in name.split("_")[0]
        mhd = name.startswith("mhd")
        shape = i["prim"].shape[1:]
        g = SimpleNamespace(primVars=i["prim"].copy(), consVars=i["cons"].copy(), dx=p["dx"],
                            BcX=p["bcx"], numXCells=shape[-1])
        if not one_d:
            g.dy, g.BcY, g.numYCells = p["dy"], p["bcy"], shape[0]
            if mhd:
                g.faceBx, g.faceBy = i["fbx"].copy(), i["fby"].copy()
        fn = {(True, False): ref_mhd.evolve_2D_mhd, (False, False): ref_hydro.evolve_2D_hydro,
              (True, True): ref_mhd.evolve_1D_mhd, (False, True): ref_hydro.evolve_1D_hydro}[(mhd, one_d)]
        tally[0] = 0
        with contextlib.redirect_stdout(io.StringIO()):
            fn(g, p["t_start"], p["t_end"], p["start_cycle"], p["max_cycles"], p["gamma"], p["cfl"], p["min_d"],
               p["min_p"], p["min_e"], p["order"], p["efix"], p["eps"])
        out[name] = tally[0]
        print(name, tally[0], flush=True)
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
        fh.write("\n")


if __name__ == "__main__":
    from tests.golden.refpath import reference_root
    main(reference_root())
