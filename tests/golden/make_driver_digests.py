"""Digests of the reference's own driver runs (``Simulation(...).run()``), with stops.

    python -B tests/golden/make_driver_digests.py <PythonMHD checkout>

(or set ``PYTHONMHD_REFERENCE``).  The reference's ``Source.Simulation`` imports
matplotlib (through its visualizer) and cv2 / pyevtk (through its file saver); this
script puts stand-in modules for those under ``sys.modules`` and then runs the
reference's unmodified ``Simulation.run()`` (Source/Simulation.py:277-434) on the
workloads in ``CASES``, with data saves and plots switched on so that the driver
stops at each save and plot time, saves or plots there and reverts to the
second-last state (Source/Simulation.py:385-413), and with ``maxCycles`` cutting one
run short (:345).  Saves go to a temporary directory.

It records, at every stop (``FileSaver.saveDataFiles`` and ``SimVisualizer.visualize``
calls, merged per time into a kinds mask: bit 0 save, bit 1 plot), the time, the
cycle count (from the evolve function the driver called last) and the SHA-256 of
the state the driver holds (prim, cons and, for MHD, faceBx, faceBy; C-contiguous
little-endian float64), and at the end the final time, cycle and state digest.
The initial state is built with ``pythonmhd_gb300.initial_conditions``; its
digest after the reference's grid construction is stored too.

Writes ``tests/golden/driver_digests.json``.  ``oracle/driver.py`` must reproduce
it on the CPU (tests/test_oracle_golden.py) and ``mhd2d_run`` on the GPU
(tests/test_gpu_driver.py).
"""
from __future__ import annotations

import contextlib
import hashlib
import io
import json
import os
import sys
import tempfile
from unittest import mock

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "driver_digests.json")
STUBS = ("matplotlib", "matplotlib.pyplot", "matplotlib.colors", "mpl_toolkits", "mpl_toolkits.axes_grid1", "cv2",
         "pyevtk", "pyevtk.hl")

# name -> workload; times and intervals force several save/plot stops and reverts
CASES = {
    "mhd_ot64_ppm_save_plot": dict(physics="mhd", nx=64, ny=64, order=2, t_lim=0.1, save_dt=0.02, plot_dt=0.03,
                                   max_cycles=100000),
    "mhd_ot48x40_order0_max_cycles": dict(physics="mhd", nx=48, ny=40, order=0, t_lim=0.2, save_dt=0.025,
                                          plot_dt=-1.0, max_cycles=37),
    "mhd_ot40x56_ppm_no_stops": dict(physics="mhd", nx=40, ny=56, order=2, t_lim=0.03, save_dt=-1.0, plot_dt=-1.0,
                                     max_cycles=100000),
    "hydro_blast_ppm_save_plot": dict(physics="hydro", nx=48, ny=40, order=2, t_lim=0.05, save_dt=0.01,
                                      plot_dt=0.0075, max_cycles=100000),
}
GAMMA = {"mhd": 5.0 / 3.0, "hydro": 1.4}
CFL = 0.4


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    return h.hexdigest()


def initial_state(case):
    """(prim, cons, faceBx, faceBy) of a case (faces None for hydro), dx, dy, bcx, bcy."""
    from pythonmhd_gb300 import initial_conditions as ic
    c = CASES[case]
    if c["physics"] == "mhd":
        prim, cons, fbx, fby, dx, dy = ic.orszag_tang(c["nx"], c["ny"], gamma=GAMMA["mhd"])
        return (prim, cons, fbx, fby), dx, dy, 1, 1
    nx, ny = c["nx"], c["ny"]
    prim = np.zeros((5, ny, nx))
    prim[0] = 1.0
    prim[1] = 0.2
    prim[4] = 0.1
    prim[4, ny // 2 - 4:ny // 2 + 3, nx // 2 - 5:nx // 2 + 2] = 10.0
    return (prim, ic.prim_to_cons_hydro(prim, GAMMA["hydro"]), None, None), 1.0 / nx, 1.0 / ny, 0, 0


def run_reference(case, S, C, tmp):
    c = CASES[case]
    mhd = c["physics"] == "mhd"
    state, dx, dy, bcx, bcy = initial_state(case)
    grid_par = {C.NUM_X_CELLS: c["nx"], C.MIN_X: 0.0, C.MAX_X: 1.0, C.NUM_Y_CELLS: c["ny"], C.MIN_Y: 0.0,
                C.MAX_Y: 1.0, C.BC_X: bcx, C.BC_Y: bcy}
    sim_par = {C.IS_MHD: mhd, C.GAMMA: GAMMA[c["physics"]], C.TLIM: c["t_lim"], C.CFL: CFL,
               C.MAX_CYCLES: c["max_cycles"], C.RECONSTRUCT_ORDER: c["order"]}
    if c["save_dt"] > 0:
        sim_par.update({C.SAVE_DATA: True, C.SAVE_DATA_DT: c["save_dt"], C.SAVE_DATA_FORMAT: C.DATA_FORMAT_MAT,
                        C.OUTPUT_FOLDER_PATH: tmp, C.OUTPUT_FOLDER_NAME: case, C.OUTPUT_FILE_NAME: case})
    vis_par = {}
    if c["plot_dt"] > 0:
        sim_par.update({C.PLOT_DATA: True, C.PLOT_DATA_DT: c["plot_dt"]})
        vis_par = {C.FIGURES: [{C.FIGURE_TITLE: case, C.PLOTS: [{C.PLOT_VAR: C.PRESSURE}]}]}
    kw = dict(faceBx=state[2].copy(), faceBy=state[3].copy()) if mhd else {}
    with contextlib.redirect_stdout(io.StringIO()):
        sim = S.Simulation(sim_par, grid_par, state[0].copy(), vis_par, **kw)

    def grid_state():
        g = sim.grid
        return (g.primVars, g.consVars, g.faceBx, g.faceBy) if mhd else (g.primVars, g.consVars)

    init = digest(*grid_state())
    stops, last_cycle, last_t = [], [0], [0.0]

    def record(kind, t):
        d = digest(*grid_state())
        if stops and stops[-1]["t"] == float(t):
            stops[-1]["kinds"] |= kind
            assert stops[-1]["sha256"] == d
        else:
            stops.append({"t": float(t), "cycle": last_cycle[0], "kinds": kind, "sha256": d})

    mod = S.evolveMHD if mhd else S.evolveHydro
    name = "evolve_2D_mhd" if mhd else "evolve_2D_hydro"
    ref_evolve = getattr(mod, name)

    def evolve(*a, **k):
        r = ref_evolve(*a, **k)
        last_cycle[0] = int(r[5] if mhd else r[3])
        last_t[0] = float(r[4] if mhd else r[2])
        return r

    orig_save, orig_vis = S.FileSaver.saveDataFiles, S.SimVisualizer.visualize

    def save(self, g, t, fmt):
        record(1, t)
        return orig_save(self, g, t, fmt)

    def vis(self, g, t):
        record(2, t)

    with mock.patch.object(mod, name, evolve), mock.patch.object(S.FileSaver, "saveDataFiles", save), \
            mock.patch.object(S.SimVisualizer, "visualize", vis), contextlib.redirect_stdout(io.StringIO()):
        sim.run()
    return {"workload": dict(c, gamma=GAMMA[c["physics"]], cfl=CFL, dx=dx, dy=dy, bcx=bcx, bcy=bcy),
            "initial_sha256": init, "stops": stops,
            "final": {"t": last_t[0], "cycle": last_cycle[0], "sha256": digest(*grid_state())}}


def main(ref_root):
    for m in STUBS:
        sys.modules[m] = mock.MagicMock()
    sys.path.insert(0, ref_root)
    import Source.PythonMHD_Constants as C  # noqa: E402
    import Source.Simulation as S  # noqa: E402
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for case in CASES:
            out[case] = run_reference(case, S, C, tmp)
            print(case, len(out[case]["stops"]), "stops, final cycle", out[case]["final"]["cycle"], flush=True)
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    sys.dont_write_bytecode = True
    from tests.golden.refpath import reference_root
    main(reference_root())
