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

from . import hydro2d, hydro3d, mhd2d


def _drive(state, evolve, t_lim, max_cycles, save_dt, save_prec, plot_dt, plot_prec):
    """The loop itself.  ``evolve(state, t0, t_end, cycle0)`` returns (state, t, cycle,
    second_last_state, second_last_t); a state is a tuple of arrays."""
    save, plot = save_dt > 0, plot_dt > 0
    stops = []

    def snap():
        return tuple(a.copy() for a in state)

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
        state, sim_t, cycles, sl_state, tsl = evolve(state, sim_t, next_stop, cycles)
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
            state, sim_t = sl_state, tsl
    return sim_t, cycles, stops, snap()


def run(prim, cons, fbx, fby, dx, dy, bcx, bcy, t_lim, max_cycles, gamma, cfl, min_d, min_p, min_e, order,
        efix, eps, save_dt=-1.0, save_prec=0, plot_dt=-1.0, plot_prec=0):
    """2D driver run.  Returns (t, cycle, stops, final_state); stops = [(t, cycle, kinds, state), ...]."""
    mhd = prim.shape[0] == 8

    def evolve(st, t0, t_end, cyc0):
        if mhd:
            (p2, c2, bx2, by2, t2, cyc2, psl, csl, bxsl, bysl, tsl) = mhd2d.evolve(
                *st, dx, dy, bcx, bcy, t0, t_end, cyc0, max_cycles, gamma, cfl, min_d, min_p, min_e, order, efix,
                eps)
            return (p2, c2, bx2, by2), t2, cyc2, (psl, csl, bxsl, bysl), tsl
        (p2, c2, t2, cyc2, psl, csl, tsl) = hydro2d.evolve(
            *st, dx, dy, bcx, bcy, t0, t_end, cyc0, max_cycles, gamma, cfl, min_d, min_p, min_e, order, efix, eps)
        return (p2, c2), t2, cyc2, (psl, csl), tsl

    state = (prim.copy(), cons.copy(), fbx.copy(), fby.copy()) if mhd else (prim.copy(), cons.copy())
    return _drive(state, evolve, t_lim, max_cycles, save_dt, save_prec, plot_dt, plot_prec)


def run3d(prim, cons, dx, dy, dz, bcx, bcy, bcz, t_lim, max_cycles, gamma, cfl, min_d, min_p, min_e, order, efix,
          eps, save_dt=-1.0, save_prec=0, plot_dt=-1.0, plot_prec=0):
    """The same loop around the 3D hydro evolve function (oracle/hydro3d.py)."""
    def evolve(st, t0, t_end, cyc0):
        (p2, c2, t2, cyc2, psl, csl, tsl) = hydro3d.evolve(
            *st, dx, dy, dz, bcx, bcy, bcz, t0, t_end, cyc0, max_cycles, gamma, cfl, min_d, min_p, min_e, order,
            efix, eps)
        return (p2, c2), t2, cyc2, (psl, csl), tsl

    return _drive((prim.copy(), cons.copy()), evolve, t_lim, max_cycles, save_dt, save_prec, plot_dt, plot_prec)


def run3d_mhd(prim, cons, fbx, fby, fbz, dx, dy, dz, bcx, bcy, bcz, t_lim, max_cycles, gamma, cfl, min_d, min_p,
              min_e, order, efix, eps, save_dt=-1.0, save_prec=0, plot_dt=-1.0, plot_prec=0, long_double=True):
    """The same loop around the 3D MHD evolve function (oracle/mhd3d.py); ``long_double``
    is passed through to its transverse predictor."""
    from . import mhd3d

    def evolve(st, t0, t_end, cyc0):
        r = mhd3d.evolve(*st, dx, dy, dz, bcx, bcy, bcz, t0, t_end, cyc0, max_cycles, gamma, cfl, min_d, min_p,
                         min_e, order, efix, eps, long_double=long_double)
        return tuple(r[:5]), r[5], r[6], tuple(r[7:12]), r[12]

    state = tuple(a.copy() for a in (prim, cons, fbx, fby, fbz))
    return _drive(state, evolve, t_lim, max_cycles, save_dt, save_prec, plot_dt, plot_prec)
