// Host/device shared layout of the 2D Godunov step: device buffers of one
// grid and the device-resident loop state.  Plain C types only.
#pragma once
#include <cstddef>
#include <cstdint>

#include <vector_types.h>

#ifdef __CUDACC__
#define MHD_HD __host__ __device__
#else
#define MHD_HD
#endif

namespace mhdk {

enum Physics : int { HYDRO = 0, MHD = 1 };
enum Bc : int { OUTFLOW = 0, PERIODIC = 1 };

// Device-resident loop state of one grid.  Written by the 1-thread bookkeeping
// kernels, read by every kernel of a cycle; the host only reads it back.
struct LoopState {
  double t;             // simulation time at the start of the next cycle
  double t_end;         // stop time
  double t_prev;        // time at the start of the last completed cycle
  double dt;            // dt of the cycle in flight (or the last one)
  double cfl;           // CFL number of this advance call
  long long cycle;      // cycle counter
  long long max_cycles;
  long long cycles_run; // cycles completed by this advance call
  unsigned long long max_sx;  // bits of max(|vx| + c_fx) over cells (non-negative double)
  unsigned long long max_sy;
  int active;           // 1 while the cycle in flight is a real cycle
  int cur;              // state buffer (0/1) holding the current state
  int pad[2];
  unsigned long long max_sz;  // 3D grids: bits of max(|vz| + c) over cells
  double dt_fixed;      // > 0: the cycle uses this dt (before the t_end clip) instead of
                        // the CFL dt of the grid (a domain-decomposed run's global dt)
};

// One state buffer: SoA planes, row-major (x fastest).
// prim/cons: 8 planes (MHD) or 5 (hydro) of Ny*Nx; fbx: Ny*(Nx+1); fby: (Ny+1)*Nx.
struct StateBuf {
  double* prim;
  double* cons;
  double* fbx;
  double* fby;
};

struct Grid {
  int nx, ny;
  double dx, dy;
  int bcx, bcy;
  int physics;   // HYDRO / MHD
  int recon;     // 0 first order, 1 PLM, 2 PPM
  int efix;
  double gamma, eps, min_d, min_p, min_e;

  StateBuf st[2];
  // scratch (NV = 7 for MHD, 5 for hydro)
  double* xl; double* xr;      // NV planes of x-face states (prim)
  double* yl; double* yr;      // NV planes of y-face states (prim)
  double* uxl; double* uxr;    // MHD: 7 planes of CTU-corrected x-face cons states
  double* uyl; double* uyr;
  double* fx; double* fy;      // NV planes of fluxes
  double* emf;                 // (Ny+1)*(Nx+1) corner EMF
  double* nfbx; double* nfby;  // half-step face B
  double* hez;                 // half-step cell Ez
  double* slopes;              // NV planes over the x-sweep-extended grid
  double* eig;                 // eigen words over the x-sweep-extended grid
  double* slopes_y;            // the same for the y sweep (separate, so both sweeps
  double* eig_y;               // can run at once)
  size_t ext_plane;            // plane stride of slopes / eig (max of x/y extended sizes)
  LoopState* loop;             // device
  int* status;                 // device error word (0 = ok; kStatusNonfinite, kStatusIndex bits)
  unsigned long long* floor_hits;  // device count of floored values (may be null)
  long long* bad;                  // checked builds: first failed index check (source line, index)
  // 1D grids (ny = 1): the x sweep only, no transverse or CT stages; MHD keeps
  // B_x uniform at bx1d (the reference's evolve_1D_mhd)
  int one_d;
  double bx1d;
  // optional device log of each cycle's dt, indexed by the loop's cycle counter
  // (cycles at or past dt_log_cap are not logged)
  double* dt_log;
  long long dt_log_cap;
};

// bits of the device error word Grid::status
constexpr int kStatusNonfinite = 1;  // a NaN or Inf was written to the state by a cycle
constexpr int kStatusIndex = 2;      // checked builds: an index fell outside its array

// index spaces of the batched work lists
enum Space : int { SPACE_CELL = 0, SPACE_EXT_X, SPACE_EXT_Y, SPACE_XFACE, SPACE_YFACE, SPACE_CORNER, kNumSpaces };

// Device view of a batch: the per-instance grids and one work list of tiles per
// index space (tile = int4 {instance, row, x0, 0}, a row segment of work items).
struct BatchView {
  const Grid* grids;
  const int4* tiles[kNumSpaces];
  int ntiles[kNumSpaces];
  int ninst;
};

MHD_HD inline size_t cell_plane(const Grid& g) { return (size_t)g.nx * g.ny; }
MHD_HD inline size_t xface_plane(const Grid& g) { return (size_t)(g.nx + 1) * g.ny; }
MHD_HD inline size_t yface_plane(const Grid& g) { return (size_t)g.nx * (g.ny + 1); }
MHD_HD inline size_t corner_plane(const Grid& g) { return (size_t)(g.nx + 1) * (g.ny + 1); }

}  // namespace mhdk
