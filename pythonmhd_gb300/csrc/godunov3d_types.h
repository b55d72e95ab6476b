// Host/device shared layout of the 3D Godunov step.  Plain C types only.
//
// Arrays follow the reference's 3D layout (Source/EvolveFunctions_Hydro.py:559-806):
// SoA planes of (ny, nx, nz) with z fastest.  An array whose extent along one
// direction is one larger (faces) or two larger (sweep-extended cells) keeps the
// same [y][x][z] order with that extent changed.
#pragma once
#include <cstddef>

#include "godunov2d_types.h"

namespace mhdk {

// One 3D state buffer: prim/cons planes of ny*nx*nz; MHD face B (x: ny*(nx+1)*nz,
// y: (ny+1)*nx*nz, z: ny*nx*(nz+1)).
struct StateBuf3 {
  double* prim;
  double* cons;
  double* fb[3];
};

struct Grid3 {
  int n[3];          // cells along x, y, z
  double d[3];       // dx, dy, dz
  int bc[3];         // OUTFLOW / PERIODIC per direction
  int physics;       // HYDRO / MHD
  int recon;         // 0 first order, 1 PLM, 2 PPM
  int efix;
  double gamma, eps, min_d, min_p, min_e;

  StateBuf3 st[2];
  double* wl[3];     // NV planes of face prim states per direction, minus side
  double* wr[3];     // plus side
  double* f[3];      // NV planes of fluxes per direction
  double* slopes;    // NV planes over the extended cells of the current sweep
  double* eig;       // eigen words over the same cells (one sweep at a time)
  size_t ext_plane;  // plane stride of slopes / eig (largest extended grid)
  LoopState* loop;
  int* status;
  // MHD only
  double* ul[3];     // 7 planes of face cons states per direction, minus side
  double* ur[3];     // plus side
  double* emf[3];    // edge EMF components (x, y, z) on the (ny+1)(nx+1)(nz+1) edge grid
  double* nfb[3];    // half-step face B
  double* ce[3];     // cell E field: stage 1, then the half step
};

// extent of an array along direction a (0 x, 1 y, 2 z) that is `add` cells larger along `dir`
MHD_HD inline int ext_n(const Grid3& g, int a, int dir, int add) { return g.n[a] + (a == dir ? add : 0); }
MHD_HD inline size_t cells3(const Grid3& g) { return (size_t)g.n[0] * g.n[1] * g.n[2]; }
MHD_HD inline size_t edges3(const Grid3& g) { return (size_t)(g.n[0] + 1) * (g.n[1] + 1) * (g.n[2] + 1); }
MHD_HD inline size_t plane3(const Grid3& g, int dir, int add) {
  return (size_t)ext_n(g, 0, dir, add) * ext_n(g, 1, dir, add) * ext_n(g, 2, dir, add);
}

}  // namespace mhdk
