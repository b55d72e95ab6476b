"""CPU restatement of the reference driver's time loop (test infrastructure only).

Source/Simulation.py:290-413 (``Simulation.__run_sim``): from t = 0 it calls the
evolve function up to the next stop time (min of the next save time, next plot
time and the time limit; the save/plot times are rounded with numpy.round to
the FileSaver / visualizer precisions), saves/plots at the stop, and, while the
run goes on, reverts to the state at the start of the last cycle (keeping the
cycle count).  This restatement runs the oracle's evolve functions and records
the stops instead of writing files or figures.
"""
from __future__ import annotations

import numpy as np

from . import hydro2d, mhd2d


def run(prim, cons, fbx, fby, dx, dy, bcx, bcy, t_lim, max_cycles, gamma, cfl, min_d, min_p, min_e, order,
        efix, eps, save_dt=-1.0, save_prec=0, plot_dt=-1.0, plot_prec=0):
    """Returns (t, cycle, stops, final_state); stops = [(t, cycle, kinds, state), ...]."""
    mhd = prim.shape[0] == 8
    save, plot = save_dt > 0, plot_dt > 0
    prim, cons = prim.copy(), cons.copy()
    fbx = fbx.copy() if mhd else None
    fby = fby.copy() if mhd else None
    stops = []

    def snap():
        return tuple(a.copy() for a in ((prim, cons, fbx, fby) if mhd else (prim, cons)))

    if save or plot:
        stops.append((0.0, 0, (1 if save else 0) | (2 if plot else 0), snap()))
    sim_t, cycles = 0.0, 0
    next_plot = next_save = t_lim
    last_plot = last_save = 0.0
    if plot:
        next_plot = np.minimum(next_plot, plot_dt)
    if save:
        next_save = np.minimum(next_save, save_dt)
    next_stop = np.minimum(next_plot, next_save)
    while sim_t < t_lim and cycles < max_cycles:
        if mhd:
            (p2, c2, bx2, by2, t2, cyc2, psl, csl, bxsl, bysl, tsl) = mhd2d.evolve(
                prim, cons, fbx, fby, dx, dy, bcx, bcy, sim_t, next_stop, cycles, max_cycles, gamma, cfl,
                min_d, min_p, min_e, order, efix, eps)
        else:
            (p2, c2, t2, cyc2, psl, csl, tsl) = hydro2d.evolve(
                prim, cons, dx, dy, bcx, bcy, sim_t, next_stop, cycles, max_cycles, gamma, cfl, min_d, min_p,
                min_e, order, efix, eps)
        prim, cons = p2, c2
        if mhd:
            fbx, fby = bx2, by2
        sim_t, cycles = t2, cyc2
        kinds = 0
        if save and next_stop == next_save:
            last_save = sim_t
            kinds |= 1
        if plot and next_stop == next_plot:
            last_plot = sim_t
            kinds |= 2
        if kinds:
            stops.append((sim_t, cycles, kinds, snap()))
        next_plot = next_save = t_lim
        if plot:
            next_plot = np.round(np.minimum(next_plot, last_plot + plot_dt), plot_prec)
        if save:
            next_save = np.round(np.minimum(next_save, last_save + save_dt), save_prec)
        next_stop = np.minimum(next_plot, next_save)
        if sim_t < t_lim and cycles < max_cycles:
            prim, cons, sim_t = psl, csl, tsl
            if mhd:
                fbx, fby = bxsl, bysl
    return sim_t, cycles, stops, snap()
