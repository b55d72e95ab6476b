// The reference driver's time loop (Source/Simulation.py:290-413), shared by the
// 2D and 3D handles' run entry points: evolve to the next stop (the minimum of the
// next save time, the next plot time and the time limit; save and plot times are
// rounded to their precisions as numpy.round does, Source/FileSaver.py:140-168),
// report the stop, and -- while the run goes on -- continue from the state before
// the short cycle that reached the stop, keeping that cycle's count.
#pragma once
#include <algorithm>
#include <cmath>

#include "../../include/pythonmhd_gb300.h"

namespace mhdk {

// numpy.round(x, decimals) for decimals >= 0: rint(x * 10**decimals) / 10**decimals
inline double round_decimals(double x, int decimals) {
  const double p = std::pow(10.0, (double)decimals);
  return std::nearbyint(x * p) / p;
}

// advance(t0, t_end, cycle0, max_cycles, &t, &cycle, &t_second_last, &cycles_run) runs
// the evolve loop; revert() makes the state before the last cycle current.
template <class Advance, class Revert>
int driver_loop(double t_lim, long long max_cycles, double save_dt, int save_prec, double plot_dt, int plot_prec,
                mhd2d_stop_fn on_stop, void* user, Advance advance, Revert revert, double* t_out,
                long long* cycle_out, long long* stops_out) {
  if (!(t_lim > 0.0) || max_cycles < 0 || save_prec < 0 || plot_prec < 0 || save_prec > 15 || plot_prec > 15)
    return MHD_ERR_ARG;
  const bool save = save_dt > 0.0, plot = plot_dt > 0.0;
  double sim_t = 0.0;
  long long cycles = 0, stops = 0;
  // the initial state is saved / shown before the first cycle
  if ((save || plot) && on_stop) {
    const int r = on_stop(user, 0.0, 0, (save ? 1 : 0) | (plot ? 2 : 0));
    if (r) return MHD_ERR_ABORTED;
  }
  double next_plot = t_lim, next_save = t_lim, last_plot = 0.0, last_save = 0.0;
  if (plot) next_plot = std::min(next_plot, plot_dt);
  if (save) next_save = std::min(next_save, save_dt);
  double next_stop = std::min(next_plot, next_save);
  while (sim_t < t_lim && cycles < max_cycles) {
    double t_new = 0.0, t_sl = 0.0;
    long long c_new = 0, ran = 0;
    int rc = advance(sim_t, next_stop, cycles, max_cycles, &t_new, &c_new, &t_sl, &ran);
    if (rc) return rc;
    sim_t = t_new;
    cycles = c_new;
    int kinds = 0;
    if (save && next_stop == next_save) { last_save = sim_t; kinds |= 1; }
    if (plot && next_stop == next_plot) { last_plot = sim_t; kinds |= 2; }
    if (kinds) {
      ++stops;
      if (on_stop && on_stop(user, sim_t, cycles, kinds)) return MHD_ERR_ABORTED;
    }
    next_plot = t_lim;
    next_save = t_lim;
    if (plot) next_plot = round_decimals(std::min(next_plot, last_plot + plot_dt), plot_prec);
    if (save) next_save = round_decimals(std::min(next_save, last_save + save_dt), save_prec);
    next_stop = std::min(next_plot, next_save);
    // still running: continue from the state before the short cycle that reached the stop
    if (sim_t < t_lim && cycles < max_cycles && ran > 0) {
      revert();
      sim_t = t_sl;
    }
  }
  if (t_out) *t_out = sim_t;
  if (cycle_out) *cycle_out = cycles;
  if (stops_out) *stops_out = stops;
  return MHD_OK;
}

}  // namespace mhdk
