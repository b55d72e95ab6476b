/*
 * C ABI of the GB300 2D unsplit Godunov step (adiabatic hydro / ideal MHD).
 *
 * One handle = one grid on one GPU with its own CUDA stream.  The handle owns
 * the device state (two ping-pong state buffers, so the state at the start of
 * the last cycle -- the reference's "second-last" state -- is always kept) and
 * the scratch of a cycle.  Arrays crossing this boundary are C-contiguous
 * float64 in the reference's layout:
 *   prim, cons : (nvars, ny, nx)  nvars = 8 for MHD [rho,vx,vy,vz,Bx,By,Bz,p] /
 *                                                  [rho,mx,my,mz,Bx,By,Bz,E],
 *                                  5 for hydro [rho,vx,vy,vz,p] / [rho,mx,my,mz,E]
 *   faceBx     : (ny, nx+1)       faceBy : (ny+1, nx)   (MHD only; NULL for hydro)
 * Every call returns a status code (0 = MHD_OK); mhd2d_strerror() names it.
 * A handle is not re-entrant: one host thread at a time per handle.
 *
 * These entry points replace the reference's Python evolve functions, which
 * take the grid object and the same scalar parameters:
 *   Source/EvolveFunctions_MHD.py:393-394    evolve_2D_mhd(simulationGrid, tStart, tEnd,
 *                                            startCycle, maxCycles, gamma, cfl, minDens,
 *                                            minPres, minEnergy, reconstructOrder,
 *                                            entropyFix, epsilon)
 *   Source/EvolveFunctions_Hydro.py:350-351  evolve_2D_hydro(...)  (same arguments)
 * The reference crosses no native boundary; the Python mirror in
 * pythonmhd_gb300/evolve.py binds these with ctypes and keeps those signatures.
 */
#ifndef PYTHONMHD_GB300_H
#define PYTHONMHD_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum mhd2d_status {
  MHD_OK = 0,
  MHD_ERR_ARG = 1,         /* invalid argument (shape, BC code, null pointer, ...) */
  MHD_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  MHD_ERR_NOMEM = 3,       /* device or pinned-host allocation failed */
  MHD_ERR_STATE = 4,       /* call out of order (e.g. advance before upload) */
  MHD_ERR_NONFINITE = 5,   /* the time or dt became NaN/Inf during advance */
  MHD_ERR_TOO_LARGE = 6,   /* size above a fixed limit of the entry point */
  MHD_ERR_ABORTED = 7,     /* mhd2d_run: the stop callback asked to stop */
  MHD_ERR_INDEX = 8        /* checked arithmetic: an index fell outside its array */
};

enum mhd2d_physics { MHD2D_HYDRO = 0, MHD2D_MHD = 1 };
/* EXACT: the reference's float64 arithmetic bit for bit; FAST: multiply-adds fused
 * except in the scalars that decide branches; CHECKED: EXACT's arithmetic with
 * every global index of the 2D and 1D kernels (single and batched) checked before
 * use -- a failed check never touches memory outside the array, sets the handle's
 * error word and makes the advance call return MHD_ERR_INDEX (mhd2d_check_info
 * says where).  A debugging build of the same source, slower. */
enum mhd2d_arith { MHD2D_ARITH_EXACT = 0, MHD2D_ARITH_FAST = 1, MHD2D_ARITH_CHECKED = 2 };

/* Create a handle for an ny x nx grid.  bcx/bcy: 0 outflow, 1 periodic
 * (Source/PythonMHD_Constants.py:11-12).  recon: 0 first order, 2 PPM
 * (Source/EvolveFunctions_MHD.py:483-511), 1 PLM (an addition: the reference's
 * PLM branches are commented out, Source/EvolveFunctions_MHD.py:487-488).  arith: MHD2D_ARITH_EXACT reproduces
 * the reference's float64 arithmetic bit for bit; MHD2D_ARITH_FAST lets the
 * compiler fuse multiply-adds (results agree to rounding).  Requires nx, ny >= 2. */
int mhd2d_create(int ny, int nx, double dx, double dy, int bcx, int bcy, double gamma,
                 int physics, int recon, int entropy_fix, double eps, double min_d,
                 double min_p, double min_e, int arith, void** handle);

/* A 1D grid of n cells: the reference's evolve_1D_mhd / evolve_1D_hydro
 * (Source/EvolveFunctions_MHD.py:195-340, Source/EvolveFunctions_Hydro.py:232-305):
 * x-sweep reconstruction (recon 2 PPM, 0 first order; 1 PLM as an addition) and
 * Roe fluxes, then cons -= dt/dx (F_right - F_left); MHD keeps B_x uniform at
 * the uploaded prim[4][0] and has no face B or CT.  States are (nvars, n); the
 * handle is then used with mhd2d_advance / mhd2d_download (NULL face arrays). */
int mhd1d_create(int n, double dx, int bcx, double gamma, int physics, int recon, int entropy_fix,
                 double eps, double min_d, double min_p, double min_e, int arith, void** handle);
int mhd1d_upload(void* handle, const double* prim, const double* cons);

/* Copy a host state in (becomes the current state).  The reference reads
 * grid.primVars, grid.consVars, grid.faceBx, grid.faceBy at the start of an
 * evolve call (Source/EvolveFunctions_MHD.py:396-444). */
int mhd2d_upload(void* handle, const double* prim, const double* cons,
                 const double* faceBx, const double* faceBy);

/* The same from device memory of the handle's GPU (no host round trip). */
int mhd2d_upload_device(void* handle, const double* prim, const double* cons,
                        const double* faceBx, const double* faceBy);

/* Run the evolve loop on the device: while t < t_end and cycle < max_cycles,
 * one CTU(+CT) cycle with the CFL dt clipped to t_end
 * (Source/EvolveFunctions_MHD.py:464-692).  Returns the final time/cycle and the
 * time at the start of the last cycle (t0 when no cycle ran). */
int mhd2d_advance(void* handle, double t0, double t_end, long long cycle0,
                  long long max_cycles, double cfl, double* t_out, long long* cycle_out,
                  double* t_second_last);

/* Domain decomposition support.  A grid split into blocks over several GPUs
 * advances each block (with a halo of neighbour cells) on its own handle; all
 * blocks must use the one global dt, the minimum over blocks of their CFL dts
 * (exact: dt = cfl / max(speed), and a correctly rounded division is monotone, so
 * the minimum of the blocks' dts is the dt of the whole grid; the reference takes
 * the global maximum speed, Source/EvolveFunctions_MHD.py:472-475).
 * mhd2d_cfl_dt: the CFL dt of the current state before the t_end clip, in the
 * exact step's arithmetic (2D handles).  mhd2d_advance_dt: one cycle from (t0,
 * cycle0) with the given dt, clipped to t_end as the step clips its own; t_out
 * gets the time after it. */
int mhd2d_cfl_dt(void* handle, double cfl, double* dt);
int mhd2d_advance_dt(void* handle, double t0, double t_end, long long cycle0, double dt, double* t_out);

/* The reference driver's time loop (Source/Simulation.py:290-413) with the state
 * kept on the device: from t = 0 and cycle 0 it advances to each stop time (the
 * next save every save_dt and plot every plot_dt, rounded to save_prec /
 * plot_prec decimals as the driver does, and t_lim), calls on_stop there
 * (kinds: bit 0 save, bit 1 plot; the callback may mhd2d_download the state;
 * nonzero return stops the run with MHD_ERR_ABORTED), and -- while the run goes
 * on -- continues from the state before the short cycle that reached the stop,
 * keeping that cycle's count, as the driver does.  save_dt / plot_dt <= 0
 * disable the stop kind.  A save or plot run also calls on_stop for the
 * initial state (t = 0).  Returns the final time, cycle count and the number of
 * stops. */
typedef int (*mhd2d_stop_fn)(void* user, double t, long long cycle, int kinds);
int mhd2d_run(void* handle, double t_lim, long long max_cycles, double cfl, double save_dt, int save_prec,
              double plot_dt, int plot_prec, mhd2d_stop_fn on_stop, void* user, double* t_out,
              long long* cycle_out, long long* stops_out);

/* Log each cycle's dt on the device: the cycle numbered c (the loop's cycle counter,
 * cycle0 + cycles run) writes its dt to dt_log[c] when c < capacity.  dt_log is a
 * device pointer of the handle's GPU that must stay valid while the log is set;
 * capacity 0 (dt_log NULL) switches the log off.  Used by the adjoint's forward
 * pass to record the CFL dts of many cycles in one advance call. */
int mhd2d_set_dt_log(void* handle, double* dt_log, long long capacity);

/* Copy a state out: which = 0 the current state, 1 the state at the start of
 * the last cycle (the reference's secondLast* arrays).  Any pointer may be
 * NULL to skip that array. */
int mhd2d_download(void* handle, int which, double* prim, double* cons,
                   double* faceBx, double* faceBy);

/* mhd2d_download into device memory of the handle's GPU (no host round trip). */
int mhd2d_download_device(void* handle, int which, double* prim, double* cons,
                          double* faceBx, double* faceBy);

/* Device pointers of the current state (for zero-copy use from a framework on
 * the same device).  Pointers stay valid until the next advance/upload. */
int mhd2d_state_ptrs(void* handle, int which, double** prim, double** cons,
                     double** faceBx, double** faceBy);

/* Debug view of a cycle's intermediates after an advance (in float64, row-major):
 * what = 0..3 x-face left/right, y-face left/right states (prim, nvars-1 slots),
 * 4/5 x/y fluxes, 6 corner EMF ((ny+1) x (nx+1)), 7/8 half-step faceBx/faceBy. */
int mhd2d_peek(void* handle, int what, double* out, size_t count);

/* Number of kernel launches the last mhd2d_advance call enqueued (graph nodes
 * times graph launches; replays past the end of the run count too). */
int mhd2d_last_launches(void* handle, long long* launches);

/* Bytes of device memory the handle holds. */
int mhd2d_device_bytes(void* handle, size_t* bytes);

/* Failure counters of the state since the last upload (SURVEY-planned stats; the
 * reference clamps floors silently, Source/PrimCons_HelperModule.py:499-554, and
 * builds a warning it never prints):
 *   floor_hits: how many values the density / pressure / energy floors raised,
 *               counted per face-state value as the reference's applyFloors
 *               calls clamp them (reconstructed prim states and CTU cons states);
 *   nan_flag:   1 if a cycle wrote a NaN or Inf into the state, or an advance
 *               ended with MHD_ERR_NONFINITE.
 * Either pointer may be NULL.  Waits for the handle's stream. */
int mhd2d_stats(void* handle, long long* floor_hits, int* nan_flag);

/* Check the current state as the reference's validatePrimVars does before a run
 * (Source/SimulationGrid_HelperModule.py:282-410): energy per cell in the
 * reference's arithmetic, then counts[7] = { cells with a NaN/Inf prim value,
 * density < 0, density < min_d, pressure < 0, pressure < min_p, energy < 0,
 * energy < min_e }.  The reference raises RuntimeError on the first nonzero
 * class (negative before below-floor, density, then pressure, then energy);
 * the Python mirror (solver.Grid2D.check_state) does the same from these counts. */
int mhd2d_validate(void* handle, long long* counts);

/* Checked arithmetic: the kernel source line and the index of the first failed
 * index check since the last upload (0, 0: none). */
int mhd2d_check_info(void* handle, long long* line, long long* index);

/* The CUDA stream the handle's work runs on (a cudaStream_t). */
int mhd2d_stream(void* handle, void** stream);

/* Largest ny accepted by mhd2d_cfl_dt_noalloc (its static scratch holds two
 * doubles per grid row). */
#define MHD2D_NOALLOC_MAX_ROWS 16384

/* CFL timestep of one state without allocating anything.  No counterpart in the
 * reference: it is the reference's CFL formula (calcDt_2D_mhd / calcDt_2D_hydro)
 * offered to callers that cannot allocate device memory -- code whose device
 * memory is owned by another framework's caching allocator, or a stepping loop
 * that must not call cudaMalloc/cudaFree each step (cudaFree synchronises the
 * device).  The caller passes device pointers: cons (nvars, ny, nx), faceBx
 * (ny, nx+1) and faceBy (ny+1, nx) for MHD (NULL for hydro), and dt_out (one
 * double); the work is queued on `stream` (NULL = the default stream) and the
 * call returns without waiting.  Scratch is a static device array of
 * 2 * MHD2D_NOALLOC_MAX_ROWS doubles (256 KB) that every GPU loading the library
 * holds until exit; ny > MHD2D_NOALLOC_MAX_ROWS returns MHD_ERR_TOO_LARGE.  The
 * first call on each device looks up that array's device address
 * (cudaGetSymbolAddress), so make it before any stream capture.  All calls share
 * the array: calls that overlap on the GPU (different streams, or different
 * host threads with the same device) race and may return a wrong dt.  The result
 * equals the dt the exact-arithmetic step uses, bit for bit; a state holding a
 * NaN gives a NaN dt.  The cached array address is not refreshed after a
 * cudaDeviceReset of that device, so calling this entry point after such a
 * reset is not supported.  If a CUDA error is already pending on the calling
 * thread, the call launches nothing, leaves that error pending and returns
 * MHD_ERR_CUDA; otherwise MHD_ERR_CUDA reports a failure of its own launches. */
int mhd2d_cfl_dt_noalloc(int physics, int ny, int nx, double dx, double dy, double gamma,
                         double cfl, const double* cons, const double* faceBx,
                         const double* faceBy, double* dt_out, void* stream);

/* ---------------------------------------------------------------------------
 * Initial states on the GPU (inputs of the runs; the reference builds its initial
 * states on the host in its initialization files, e.g. the Orszag-Tang vortex of
 * InitializationFiles/SampleSimulations/2D_MHD/OrszagTang_InitializationFile.py:134-194).
 * All pointers are device pointers of the current GPU; the work is queued on
 * `stream` (NULL: the default stream).
 *
 * mhd_ic_scatter_spectrum: spec[idx[k]] = re[k] + i im[k] for k < count, into an
 *   interleaved complex half-spectrum the caller zeroed (the in-band coefficients
 *   of a seeded Gaussian random field, drawn on the host).
 * mhd_ic_turbulence_2d: the driven-free turbulence state of an n x n periodic unit
 *   box from the four inverse-transformed fields g, vx, vy, A_z (in that order of
 *   the random stream): rho = exp(0.1 g / std g), p = 1/gamma, velocities scaled to
 *   rms Mach `mach`, face B from A_z scaled to plasma beta `beta`, prim, cons,
 *   faceBx (n, n+1), faceBy (n+1, n).  `work` holds mhd_ic_work_words() doubles.
 * mhd_ic_orszag_tang: the Orszag-Tang vortex on nx x ny with B0 scaled by b0_scale,
 *   face B from the corner vector potential, and the density multiplied by
 *   (1 + rho_perturb noise) when `noise` (ny, nx) is not NULL.
 * ------------------------------------------------------------------------- */
long long mhd_ic_work_words(void);
int mhd_ic_scatter_spectrum(long long count, const int* idx, const double* re, const double* im, double* spec,
                            void* stream);
int mhd_ic_turbulence_2d(int n, double gamma, double mach, double beta, const double* g, const double* vx,
                         const double* vy, const double* az, double* prim, double* cons, double* fbx, double* fby,
                         double* work, long long work_words, void* stream);
int mhd_ic_orszag_tang(int nx, int ny, double gamma, double b0_scale, double rho_perturb, const double* noise,
                       double* prim, double* cons, double* fbx, double* fby, void* stream);

/* ---------------------------------------------------------------------------
 * Batched form: many independent grids (uneven sizes, per-instance gamma, dx,
 * dy, boundary conditions, dt, time and cycle count) advanced together with one
 * persistent-kernel launch per stage over a work list of row tiles; a whole
 * cycle of all instances is one CUDA graph.  No counterpart in the reference,
 * which advances one grid per evolve call; per instance the result equals the
 * single-grid entry points' result bit for bit.
 * ------------------------------------------------------------------------- */
int mhdb_create(int count, const int* ny, const int* nx, const double* dx, const double* dy,
                const int* bcx, const int* bcy, const double* gamma, int physics, int recon,
                int entropy_fix, double eps, double min_d, double min_p, double min_e,
                int arith, void** handle);
int mhdb_upload(void* handle, int instance, const double* prim, const double* cons,
                const double* faceBx, const double* faceBy);
/* Per-instance t0/t_end/cycle0/max_cycles arrays; every instance runs the
 * reference loop (while t < t_end and cycle < max_cycles) with its own dt.  An
 * instance whose time or dt becomes non-finite stops there while the others run
 * to their ends; t_out / cycle_out are written for every instance, and the call
 * then returns MHD_ERR_NONFINITE (mhdb_instance_status names the instances). */
int mhdb_advance(void* handle, const double* t0, const double* t_end, const long long* cycle0,
                 const long long* max_cycles, double cfl, double* t_out, long long* cycle_out);
/* Per-instance status of the last mhdb_advance (count ints: MHD_OK or
 * MHD_ERR_NONFINITE). */
int mhdb_instance_status(void* handle, int* status);
/* mhd2d_stats per instance: count entries in each array (either may be NULL). */
int mhdb_stats(void* handle, long long* floor_hits, int* nan_flag);
int mhdb_download(void* handle, int instance, int which, double* prim, double* cons,
                  double* faceBx, double* faceBy);
/* Launch shape of a batched cycle (the autotuner's knobs): tile_width work
 * items per tile = threads per block (32, 64 or 128; default 128), fuse = 1
 * for one launch per stage and direction or 2 to run the independent x and y
 * launches of a stage as one launch, blocks = blocks of each persistent launch
 * (default 2 per SM).  Results do not depend on these. */
int mhdb_configure(void* handle, int tile_width, int fuse, int blocks);
/* Work lists: a batched cycle runs, per index space, a list of row tiles
 * {instance, row, x0, 0} (4 ints each) that its persistent blocks stride through.
 * Spaces: 0 cells (nx x ny), 1 x-extended cells (nx+2 x ny), 2 y-extended cells
 * (nx x ny+2), 3 x-faces (nx+1 x ny), 4 y-faces (nx x ny+1), 5 corners
 * (nx+1 x ny+1); x0 is a multiple of the tile width.  mhdb_get_tiles copies the
 * installed list of a space (tiles NULL: just its length); mhdb_set_tiles installs a
 * caller's order of it, e.g. largest instances first.  The list is checked on the
 * host before anything is copied or launched: every tile of every instance exactly
 * once and nothing out of range, else MHD_ERR_ARG and the installed list stays.
 * mhdb_configure with a new tile width rebuilds every list in the default order. */
int mhdb_get_tiles(void* handle, int space, int* tiles, long long capacity, long long* count);
int mhdb_set_tiles(void* handle, int space, const int* tiles, long long count);
/* mhdb_upload from device memory of the handle's GPU. */
int mhdb_upload_device(void* handle, int inst, const double* prim, const double* cons,
                       const double* faceBx, const double* faceBy);
/* Copy instance `inst`'s current MHD state into the packed device layout
 * prim (8,ny,nx) | cons (8,ny,nx) | faceBx | faceBy (the adjoint's state layout). */
int mhdb_pack_state(void* handle, int inst, double* dst);
/* Device pointers of instance `inst`'s current (which = 0) or second-last (1) state;
 * valid until the next advance or upload. */
int mhdb_state_ptrs(void* handle, int inst, int which, double** prim, double** cons,
                    double** faceBx, double** faceBy);
int mhdb_info(void* handle, long long* last_launches, size_t* device_bytes, int* blocks,
              void** stream);
void mhdb_destroy(void* handle);

/* ---------------------------------------------------------------------------
 * Adjoint (reverse mode) of the MHD step, first-order (recon 0), PLM (recon 1)
 * and PPM (recon 2) reconstruction.  No counterpart in the reference.  States are
 * "packed" device arrays of mhd2d_adj_info()'s state_words doubles:
 *   prim (8, ny, nx) | cons (8, ny, nx) | faceBx (ny, nx+1) | faceBy (ny+1, nx);
 * an adjoint ("bar") array has the same layout.  dt is frozen: the forward
 * pass records the CFL dt of each cycle and the backward pass treats it as a
 * constant.  The forward sweep equals the exact-arithmetic step bit for bit.
 * Every call queues on the handle's own stream and waits for it before
 * returning.
 * ------------------------------------------------------------------------- */
int mhd2d_adj_create(int ny, int nx, double dx, double dy, int bcx, int bcy, double gamma, int recon,
                     int entropy_fix, double eps, double min_d, double min_p, double min_e, void** handle);
/* One cycle with the given dt: state_in -> state_out (device, packed). */
int mhd2d_adj_cycle(void* handle, double dt, const double* state_in, double* state_out);
/* Vector-Jacobian product of one cycle at state_in: bar_out -> bar_in. */
int mhd2d_adj_cycle_reverse(void* handle, double dt, const double* state_in, const double* bar_out,
                            double* bar_in);
/* `steps` cycles from state_in to state_out with the CFL dt of each cycle (or
 * the host array fixed_dt when it is not NULL), recorded into the host array
 * dt_log (may be NULL).  Keeps a state checkpoint every `every` cycles
 * (0 = ceil(sqrt(steps))) for mhd2d_adj_backward. */
int mhd2d_adj_forward(void* handle, const double* state_in, int steps, double cfl, const double* fixed_dt,
                      int every, double* state_out, double* dt_log);
/* Adjoint of the last mhd2d_adj_forward: bar_final -> bar_initial.  Each
 * checkpoint segment is recomputed once from its checkpoint; when the arrays of
 * all its cycles fit the segment budget they stay resident for the reverse
 * sweep, otherwise each cycle is recomputed again right before its reverse. */
int mhd2d_adj_backward(void* handle, const double* bar_final, double* bar_initial);
/* Bytes the backward pass may hold to keep a whole segment resident
 * (0 = 85% of the free device memory at mhd2d_adj_forward time). */
int mhd2d_adj_configure(void* handle, size_t segment_bytes);
/* Re-target a handle to another grid with the same reconstruction, entropy fix
 * and floors (drops its forward record).  Device memory is reused while large
 * enough, so one handle can run the backward passes of many grids in turn. */
int mhd2d_adj_reshape(void* handle, int ny, int nx, double dx, double dy, int bcx, int bcy, double gamma);
/* Device bytes one resident cycle takes in the backward pass (its arrays and
 * tapes) for an ny x nx grid: a whole checkpoint segment stays resident when
 * `every` times this fits the segment budget. */
int mhd2d_adj_cycle_bytes(int ny, int nx, int recon, int entropy_fix, size_t* bytes);
/* q[i] = b[i] / v[i] as the reverse sweeps compute it (n elements, device
 * pointers; blocks until done): a refined reciprocal within two ulps of the
 * correctly rounded quotient for divisors of magnitude 2^-1000 .. 2^1000, the
 * correctly rounded quotient otherwise.  Exposed so that bound can be tested. */
int mhd2d_adj_quotient(const double* b, const double* v, double* q, long long n);
/* q[i] = x[i] / 6 as the exact-arithmetic kernels compute it in the PPM interface
 * values (n elements, device pointers; blocks until done): one multiply and two FMAs
 * (Markstein's remainder correction), correctly rounded, so equal bit for bit to
 * the IEEE division.  Exposed so that the equality can be tested. */
int mhd_quotient6(const double* x, double* q, long long n);
/* out[i] = x[i] op y[i] (op 0 add, 1 subtract, 2 multiply, 3 divide) or sqrt(x[i])
 * (op 4; y unused) as the step kernels compute them on the integer pipes (n
 * elements, device pointers; blocks until done).  Each equals the IEEE-754
 * operation rounded to nearest even bit for bit; exposed so that can be tested.
 * No counterpart in the reference: it tests arithmetic the reference leaves to
 * NumPy. */
int mhd_softfp(int op, const double* x, const double* y, double* out, long long n);
/* Install a forward record made elsewhere (e.g. by the batched step): `steps`
 * cycles with the host dts `dt`, and the packed device states at cycles 0,
 * every, 2*every, ... in `checkpoints` (ceil(steps/every) states, one after the
 * other; the memory stays the caller's and must outlive the backward pass).
 * mhd2d_adj_backward then runs from it. */
int mhd2d_adj_restore(void* handle, const double* checkpoints, int steps, int every, const double* dt);
/* state_words: length of a packed state; device_bytes: memory held now;
 * segment_sets: cycles kept resident per segment by the last forward (1 =
 * recompute mode). */
int mhd2d_adj_info(void* handle, size_t* state_words, size_t* device_bytes, int* segment_sets);
/* Tail of the forward record: when the backward pass can keep segments resident,
 * mhd2d_adj_forward runs the last cycles of the run (as many as the segment budget
 * holds, at least the checkpoint interval) with the taped kernels and leaves their
 * arrays resident, so the first mhd2d_adj_backward reverses them without
 * recomputing them.  max_cycles: -1 (default) as many as fit, 0 no tail, n at most n. */
int mhd2d_adj_set_tail(void* handle, int max_cycles);
/* The last record: its cycles, checkpoint interval and tail length (0: none). */
int mhd2d_adj_record(void* handle, int* steps, int* every, int* tail);
/* Branch-frozen forward passes, for checking the backward pass by finite
 * differences.  The discrete step is piecewise smooth: limiter and floor clamps,
 * the Roe upwind switch, the entropy-fix window, the corner-EMF upwinding and |x|
 * change branch at kinks, and over hundreds of cycles a perturbation of 1e-6
 * crosses some of them, so free central differences measure a different piece
 * than the one the adjoint differentiates.  mode 1 runs `steps` cycles from
 * state_in with the host dts `dt` and records every branch decision of every
 * stage (conditions and the sign of each |x|) in the handle; mode 2 runs the same
 * cycles from another state with each decision replayed from that record, i.e. on
 * the recorded piece.  Mode 2 from the recorded initial state reproduces mode 1
 * bit for bit; it needs a record of at least `steps` cycles (else MHD_ERR_STATE).
 * Both reuse the first value arena, so a pending resident tail of the forward
 * record is recomputed from its checkpoint by the next mhd2d_adj_backward.  The
 * record takes 4 bytes x (tape words per cycle) x steps of device memory (about
 * 92 B per cell and cycle for PLM). */
int mhd2d_adj_branches(void* handle, int mode, const double* state_in, int steps, const double* dt,
                       double* state_out);
void mhd2d_adj_destroy(void* handle);

/* ---------------------------------------------------------------------------
 * 3D step: replaces the reference's
 *   Source/EvolveFunctions_Hydro.py:559-560  evolve_3D_hydro(simulationGrid, tStart, tEnd,
 *                                            startCycle, maxCycles, gamma, cfl, minDens,
 *                                            minPres, minEnergy, reconstructOrder,
 *                                            entropyFix, epsilon)
 *   Source/EvolveFunctions_MHD.py:750-751    evolve_3D_mhd(...)  (same arguments)
 * States are (nvars, ny, nx, nz), z fastest (the reference's layout, also the device
 * layout); MHD adds faceBx (ny, nx+1, nz), faceBy (ny+1, nx, nz), faceBz (ny, nx, nz+1)
 * (NULL for hydro).  bcx/bcy/bcz: 0 outflow, 1 periodic; recon: 2 PPM, 0 first
 * order, 1 PLM (an addition).  The evolve loop, second-last state and download
 * semantics are mhd2d_advance's / mhd2d_download's.  nx, ny, nz >= 2;
 * (nx+2)(ny+2)(nz+2) below 2^32.  The MHD x predictor's y terms, which the reference
 * computes in long double (Source/CTU_HelperModule.py:455), are FP64 here: results
 * match the reference to rounding, not bit for bit.
 * ------------------------------------------------------------------------- */
int mhd3d_create(int ny, int nx, int nz, double dx, double dy, double dz, int bcx, int bcy, int bcz,
                 double gamma, int physics, int recon, int entropy_fix, double eps, double min_d, double min_p,
                 double min_e, int arith, void** handle);
int mhd3d_upload(void* handle, const double* prim, const double* cons, const double* faceBx, const double* faceBy,
                 const double* faceBz);
/* as mhd3d_upload, from device pointers */
int mhd3d_upload_device(void* handle, const double* prim, const double* cons, const double* faceBx,
                        const double* faceBy, const double* faceBz);
int mhd3d_advance(void* handle, double t0, double t_end, long long cycle0, long long max_cycles, double cfl,
                  double* t_out, long long* cycle_out, double* t_second_last);
/* mhd2d_run's driver loop (Source/Simulation.py:290-413) on a 3D handle */
int mhd3d_run(void* handle, double t_lim, long long max_cycles, double cfl, double save_dt, int save_prec,
              double plot_dt, int plot_prec, mhd2d_stop_fn on_stop, void* user, double* t_out,
              long long* cycle_out, long long* stops_out);
int mhd3d_download(void* handle, int which, double* prim, double* cons, double* faceBx, double* faceBy,
                   double* faceBz);
/* device pointers of the current (which = 0) or second-last (1) state */
int mhd3d_state_ptrs(void* handle, int which, double** prim, double** cons, double** faceBx, double** faceBy,
                     double** faceBz);
/* kernel launches of the last advance, device bytes held, the handle's cudaStream_t */
int mhd3d_info(void* handle, long long* last_launches, size_t* device_bytes, void** stream);
void mhd3d_destroy(void* handle);

const char* mhd2d_strerror(int status);
void mhd2d_destroy(void* handle);

#ifdef __cplusplus
}
#endif
#endif /* PYTHONMHD_GB300_H */
