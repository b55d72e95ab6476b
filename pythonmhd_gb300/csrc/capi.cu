// C ABI of the 2D Godunov step: handle lifetime, host<->device copies and the
// device-resident evolve loop (CUDA graphs of two cycles replayed in chunks).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/pythonmhd_gb300.h"
#include "driver_loop.h"
#include "godunov2d_types.h"

namespace mhdk {
namespace exact {
void enqueue_cycle(const Grid& g, int parity, int dt_blocks, cudaStream_t s);
void enqueue_cycle_batch_tuned(const BatchView& V, int physics, int recon, unsigned blocks, unsigned tw, int fuse,
                               cudaStream_t s);
}  // namespace exact
void enqueue_validate(int mhd, size_t plane, double gamma, double min_d, double min_p, double min_e,
                      const double* prim, unsigned long long* counts, int blocks, cudaStream_t s);
namespace fast {
void enqueue_cycle(const Grid& g, int parity, int dt_blocks, cudaStream_t s);
void enqueue_cycle_batch_tuned(const BatchView& V, int physics, int recon, unsigned blocks, unsigned tw, int fuse,
                               cudaStream_t s);
}  // namespace fast
namespace checked {
void enqueue_cycle(const Grid& g, int parity, int dt_blocks, cudaStream_t s);
void enqueue_cycle_batch_tuned(const BatchView& V, int physics, int recon, unsigned blocks, unsigned tw, int fuse,
                               cudaStream_t s);
}  // namespace checked
}  // namespace mhdk

using mhdk::Grid;
using mhdk::LoopState;

namespace {

struct Handle {
  Grid g{};
  int arith = 0;
  int device = 0;
  int nvars = 8;
  cudaStream_t stream = nullptr;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  LoopState* host_loop = nullptr;  // pinned
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // two cycles starting at parity p
  int cur = 0;            // state buffer holding the current state
  int have_state = 0;
  long long last_cycles_run = 0;
  long long last_launches = 0;
  size_t graph_nodes[2] = {0, 0};
  int dt_blocks = 0;
  int nonfinite_seen = 0;  // an advance since the last upload ended with MHD_ERR_NONFINITE
  unsigned long long* d_check = nullptr;  // 7 counters of mhd2d_validate (device)
  double* d_dt = nullptr;                 // mhd2d_cfl_dt's result (device)
};

int cuda_fail(cudaError_t e) {
  if (e == cudaErrorMemoryAllocation) return MHD_ERR_NOMEM;
  return MHD_ERR_CUDA;
}

#define CK(call)                                  \
  do {                                            \
    cudaError_t _e = (call);                      \
    if (_e != cudaSuccess) return cuda_fail(_e);  \
  } while (0)

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

// Lay out every buffer of one grid from `base` (256-byte aligned pieces) and
// return the bytes used; with base == nullptr only the size is computed.
size_t carve_grid(Grid& g, int nvars, char* base) {
  const int nv = g.physics == MHD2D_MHD ? 7 : 5;
  const int nw = g.physics == MHD2D_MHD ? 42 : 10;
  const size_t cp = mhdk::cell_plane(g), xp = mhdk::xface_plane(g), yp = mhdk::yface_plane(g),
               kp = mhdk::corner_plane(g);
  g.ext_plane = std::max((size_t)(g.nx + 2) * g.ny, (size_t)g.nx * (g.ny + 2));
  const bool mhd = g.physics == MHD2D_MHD;
  size_t off = 0;
  auto take = [&](double** p, size_t n) {
    if (base) *p = reinterpret_cast<double*>(base + off);
    off += align256(n * sizeof(double));
  };
  for (int b = 0; b < 2; ++b) {
    take(&g.st[b].prim, (size_t)nvars * cp);
    take(&g.st[b].cons, (size_t)nvars * cp);
    if (mhd) { take(&g.st[b].fbx, xp); take(&g.st[b].fby, yp); }
  }
  take(&g.xl, nv * xp); take(&g.xr, nv * xp);
  take(&g.yl, nv * yp); take(&g.yr, nv * yp);
  take(&g.fx, nv * xp); take(&g.fy, nv * yp);
  if (mhd) {
    take(&g.uxl, nv * xp); take(&g.uxr, nv * xp);
    take(&g.uyl, nv * yp); take(&g.uyr, nv * yp);
    take(&g.emf, kp); take(&g.nfbx, xp); take(&g.nfby, yp);
    take(&g.hez, cp);
  }
  if (g.recon >= 1) {
    take(&g.slopes, nv * g.ext_plane);
    take(&g.eig, nw * g.ext_plane);
    take(&g.slopes_y, nv * g.ext_plane);
    take(&g.eig_y, nw * g.ext_plane);
  }
  return off;
}

void enqueue(Handle* h, int parity) {
  if (h->arith == MHD2D_ARITH_EXACT) mhdk::exact::enqueue_cycle(h->g, parity, h->dt_blocks, h->stream);
  else if (h->arith == MHD2D_ARITH_CHECKED) mhdk::checked::enqueue_cycle(h->g, parity, h->dt_blocks, h->stream);
  else mhdk::fast::enqueue_cycle(h->g, parity, h->dt_blocks, h->stream);
}

int build_graph(Handle* h, int parity) {
  if (h->graph[parity]) return MHD_OK;
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  enqueue(h, parity);
  enqueue(h, parity ^ 1);
  cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
  if (e != cudaSuccess) return cuda_fail(e);
  size_t nodes = 0;
  cudaGraphGetNodes(graph, nullptr, &nodes);
  h->graph_nodes[parity] = nodes;
  e = cudaGraphInstantiate(&h->graph[parity], graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e);
  return MHD_OK;
}

// ---------------------------------------------------------------------------
// Batched handles: many independent grids advanced by one launch per stage.
// ---------------------------------------------------------------------------
struct BatchHandle {
  int count = 0;
  int physics = 1, recon = 2, arith = 0, nvars = 8;
  int device = 0;
  std::vector<Grid> grids;         // host copies (device pointers inside)
  Grid* d_grids = nullptr;
  int4* d_tiles = nullptr;         // all work lists, one after the other (own allocation)
  int tile_width = 128;            // work items per tile = threads per block
  int fuse = 1;                    // 1: one launch per stage and direction; 2: x+y fused
  mhdk::BatchView view{};
  void* arena = nullptr;
  size_t arena_bytes = 0;
  LoopState* d_loops = nullptr;
  LoopState* h_loops = nullptr;    // pinned
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  size_t graph_nodes = 0;
  unsigned blocks = 0;
  long long last_launches = 0;
  std::vector<int> uploaded;
  std::vector<int> inst_status;    // per-instance status of the last mhdb_advance
  std::vector<std::vector<int4>> host_tiles;  // the installed work lists
  int* d_status = nullptr;         // per-instance device error words
  unsigned long long* d_floor_hits = nullptr;  // per-instance floor-hit counts
};

void enqueue_batch(BatchHandle* b) {
  if (b->arith == MHD2D_ARITH_EXACT)
    mhdk::exact::enqueue_cycle_batch_tuned(b->view, b->physics, b->recon, b->blocks, (unsigned)b->tile_width, b->fuse,
                                           b->stream);
  else if (b->arith == MHD2D_ARITH_CHECKED)
    mhdk::checked::enqueue_cycle_batch_tuned(b->view, b->physics, b->recon, b->blocks, (unsigned)b->tile_width,
                                             b->fuse, b->stream);
  else
    mhdk::fast::enqueue_cycle_batch_tuned(b->view, b->physics, b->recon, b->blocks, (unsigned)b->tile_width, b->fuse,
                                          b->stream);
}

// Width and height of index space `sp` of grid g (work items per row, rows).
void space_extent(const Grid& g, int sp, int* w, int* h) {
  const int ws[mhdk::kNumSpaces] = {g.nx, g.nx + 2, g.nx, g.nx + 1, g.nx, g.nx + 1};
  const int hs[mhdk::kNumSpaces] = {g.ny, g.ny, g.ny + 2, g.ny, g.ny + 1, g.ny + 1};
  *w = ws[sp];
  *h = hs[sp];
}

// A work list for space sp must name every row tile {instance, row, x0} of every
// instance exactly once (x0 a multiple of `width` below the row width).  A tile out
// of range would make a kernel index past its instance's arrays; a missing or
// repeated tile would skip or race on work items.  Checked on the host, before
// anything is copied or launched.
bool tiles_valid(const BatchHandle* b, int sp, int width, const std::vector<int4>& t) {
  std::vector<size_t> first(b->count + 1, 0);
  for (int i = 0; i < b->count; ++i) {
    int w, h;
    space_extent(b->grids[i], sp, &w, &h);
    first[i + 1] = first[i] + (size_t)h * ((w + width - 1) / width);
  }
  if (t.size() != first[b->count]) return false;
  std::vector<unsigned char> seen(t.size(), 0);
  for (const int4& q : t) {
    if (q.x < 0 || q.x >= b->count || q.w != 0) return false;
    int w, h;
    space_extent(b->grids[q.x], sp, &w, &h);
    if (q.y < 0 || q.y >= h || q.z < 0 || q.z >= w || q.z % width != 0) return false;
    const size_t slot = first[q.x] + (size_t)q.y * ((w + width - 1) / width) + q.z / width;
    if (seen[slot]) return false;
    seen[slot] = 1;
  }
  return true;
}

// Install per-space work lists (already validated) on the device.
int install_tiles(BatchHandle* b, int width, std::vector<int4> (&tiles)[mhdk::kNumSpaces]) {
  size_t total = 0;
  for (auto& t : tiles) total += t.size();
  int4* d = nullptr;
  cudaError_t e = cudaMalloc(&d, total * sizeof(int4));
  if (e != cudaSuccess) return cuda_fail(e);
  size_t off = 0;
  mhdk::BatchView v = b->view;
  for (int sp = 0; sp < mhdk::kNumSpaces && e == cudaSuccess; ++sp) {
    v.tiles[sp] = d + off;
    v.ntiles[sp] = (int)tiles[sp].size();
    e = cudaMemcpyAsync(d + off, tiles[sp].data(), tiles[sp].size() * sizeof(int4), cudaMemcpyHostToDevice,
                        b->stream);
    off += tiles[sp].size();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) { cudaFree(d); return cuda_fail(e); }
  if (b->d_tiles) cudaFree(b->d_tiles);
  b->d_tiles = d;
  b->view = v;
  b->tile_width = width;
  b->host_tiles.resize(mhdk::kNumSpaces);
  for (int sp = 0; sp < mhdk::kNumSpaces; ++sp) b->host_tiles[sp] = tiles[sp];
  return MHD_OK;
}

// (Re)build the per-space work lists for tiles of `width` items, row-major per instance.
int build_tiles(BatchHandle* b, int width) {
  std::vector<int4> tiles[mhdk::kNumSpaces];
  for (int i = 0; i < b->count; ++i) {
    for (int sp = 0; sp < mhdk::kNumSpaces; ++sp) {
      int w, h;
      space_extent(b->grids[i], sp, &w, &h);
      for (int r = 0; r < h; ++r)
        for (int x0 = 0; x0 < w; x0 += width) tiles[sp].push_back(make_int4(i, r, x0, 0));
    }
  }
  return install_tiles(b, width, tiles);
}

int build_batch_graph(BatchHandle* b) {
  if (b->graph) return MHD_OK;
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_batch(b);
  cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
  if (e != cudaSuccess) return cuda_fail(e);
  size_t nodes = 0;
  cudaGraphGetNodes(graph, nullptr, &nodes);
  b->graph_nodes = nodes;
  e = cudaGraphInstantiate(&b->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e);
  return MHD_OK;
}

void free_batch(BatchHandle* b) {
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->d_tiles) cudaFree(b->d_tiles);
  if (b->h_loops) cudaFreeHost(b->h_loops);
  if (b->arena) cudaFree(b->arena);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // namespace

extern "C" {

const char* mhd2d_strerror(int status) {
  switch (status) {
    case MHD_OK: return "ok";
    case MHD_ERR_ARG: return "invalid argument";
    case MHD_ERR_CUDA: return "CUDA runtime error";
    case MHD_ERR_NOMEM: return "out of memory";
    case MHD_ERR_STATE: return "call out of order (no state uploaded)";
    case MHD_ERR_NONFINITE: return "time or timestep became non-finite";
    case MHD_ERR_TOO_LARGE: return "size above the entry point's fixed limit";
    case MHD_ERR_ABORTED: return "stopped by the caller's stop callback";
    case MHD_ERR_INDEX: return "an index fell outside its array (checked build)";
    default: return "unknown status";
  }
}

static int create_grid(int ny, int nx, double dx, double dy, int bcx, int bcy, double gamma, int physics,
                       int recon, int entropy_fix, double eps, double min_d, double min_p, double min_e,
                       int arith, int one_d, void** handle) {
  if (!handle) return MHD_ERR_ARG;
  *handle = nullptr;
  if (nx < 2 || ny < (one_d ? 1 : 2) || !(dx > 0.0) || !(dy > 0.0)) return MHD_ERR_ARG;
  if ((bcx != 0 && bcx != 1) || (bcy != 0 && bcy != 1)) return MHD_ERR_ARG;
  if (physics != MHD2D_HYDRO && physics != MHD2D_MHD) return MHD_ERR_ARG;
  if (recon != 0 && recon != 1 && recon != 2) return MHD_ERR_ARG;
  if (arith != MHD2D_ARITH_EXACT && arith != MHD2D_ARITH_FAST && arith != MHD2D_ARITH_CHECKED) return MHD_ERR_ARG;
  if ((long long)nx * ny > (1LL << 31)) return MHD_ERR_TOO_LARGE;

  Handle* h = new (std::nothrow) Handle();
  if (!h) return MHD_ERR_NOMEM;
  Grid& g = h->g;
  g.nx = nx; g.ny = ny; g.dx = dx; g.dy = dy; g.bcx = bcx; g.bcy = bcy;
  g.physics = physics; g.recon = recon; g.efix = entropy_fix ? 1 : 0;
  g.gamma = gamma; g.eps = eps; g.min_d = min_d; g.min_p = min_p; g.min_e = min_e;
  g.one_d = one_d;
  g.bx1d = 0.0;
  h->arith = arith;
  h->nvars = physics == MHD2D_MHD ? 8 : 5;

  cudaError_t e = cudaGetDevice(&h->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete h; return cuda_fail(e); }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  h->dt_blocks = std::max(1, sms) * 8;

  const size_t total = carve_grid(g, h->nvars, nullptr) + align256(sizeof(LoopState)) + align256(sizeof(int)) +
                       align256(sizeof(unsigned long long)) + align256(7 * sizeof(unsigned long long)) +
                       align256(sizeof(double)) + align256(2 * sizeof(long long));
  e = cudaMalloc(&h->arena, total);
  if (e != cudaSuccess) {
    cudaStreamDestroy(h->stream);
    delete h;
    return cuda_fail(e);
  }
  h->arena_bytes = total;
  char* base = static_cast<char*>(h->arena);
  size_t off = carve_grid(g, h->nvars, base);
  g.loop = reinterpret_cast<LoopState*>(base + off);
  off += align256(sizeof(LoopState));
  g.status = reinterpret_cast<int*>(base + off);
  off += align256(sizeof(int));
  g.floor_hits = reinterpret_cast<unsigned long long*>(base + off);
  off += align256(sizeof(unsigned long long));
  h->d_check = reinterpret_cast<unsigned long long*>(base + off);
  off += align256(7 * sizeof(unsigned long long));
  h->d_dt = reinterpret_cast<double*>(base + off);
  off += align256(sizeof(double));
  g.bad = reinterpret_cast<long long*>(base + off);
  e = cudaMemsetAsync(h->arena, 0, total, h->stream);
  if (e == cudaSuccess) e = cudaMallocHost(&h->host_loop, sizeof(LoopState));
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    if (h->host_loop) cudaFreeHost(h->host_loop);
    cudaFree(h->arena);
    cudaStreamDestroy(h->stream);
    delete h;
    return cuda_fail(e);
  }
  *handle = h;
  return MHD_OK;
}

int mhd2d_create(int ny, int nx, double dx, double dy, int bcx, int bcy, double gamma, int physics,
                 int recon, int entropy_fix, double eps, double min_d, double min_p, double min_e,
                 int arith, void** handle) {
  return create_grid(ny, nx, dx, dy, bcx, bcy, gamma, physics, recon, entropy_fix, eps, min_d, min_p, min_e,
                     arith, 0, handle);
}

int mhd1d_create(int n, double dx, int bcx, double gamma, int physics, int recon, int entropy_fix, double eps,
                 double min_d, double min_p, double min_e, int arith, void** handle) {
  return create_grid(1, n, dx, 1.0, bcx, 1, gamma, physics, recon, entropy_fix, eps, min_d, min_p, min_e, arith,
                     1, handle);
}

static int upload_state(void* handle, const double* prim, const double* cons, const double* faceBx,
                        const double* faceBy, cudaMemcpyKind kind);

int mhd1d_upload(void* handle, const double* prim, const double* cons) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !prim || !cons) return MHD_ERR_ARG;
  if (!h->g.one_d) return MHD_ERR_STATE;
  const int n = h->g.nx;
  if (h->g.physics == MHD2D_HYDRO) return upload_state(handle, prim, cons, nullptr, nullptr, cudaMemcpyHostToDevice);
  // B_x is the first cell's value everywhere (Source/EvolveFunctions_MHD.py:201-205); the
  // face array of both state buffers holds it for the Roe solver's normal B
  const double bx = prim[4 * (size_t)n];
  std::vector<double> fbx((size_t)n + 1, bx), fby(2 * (size_t)n, 0.0);
  int rc = upload_state(handle, prim, cons, fbx.data(), fby.data(), cudaMemcpyHostToDevice);
  if (rc) return rc;
  const mhdk::StateBuf& other = h->g.st[h->cur ^ 1];
  CK(cudaMemcpyAsync(other.fbx, fbx.data(), fbx.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (h->g.bx1d != bx) {
    // the kernels take the grid by value: rebuild the cycle graphs with the new B_x
    h->g.bx1d = bx;
    for (auto& ge : h->graph)
      if (ge) { cudaGraphExecDestroy(ge); ge = nullptr; }
  }
  return MHD_OK;
}

void mhd2d_destroy(void* handle) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& ge : h->graph)
    if (ge) cudaGraphExecDestroy(ge);
  if (h->host_loop) cudaFreeHost(h->host_loop);
  if (h->arena) cudaFree(h->arena);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

static int upload_state(void* handle, const double* prim, const double* cons, const double* faceBx,
                        const double* faceBy, cudaMemcpyKind kind) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !prim || !cons) return MHD_ERR_ARG;
  const bool mhd = h->g.physics == MHD2D_MHD;
  if (mhd && (!faceBx || !faceBy)) return MHD_ERR_ARG;
  const mhdk::StateBuf& s = h->g.st[h->cur];
  const size_t cb = (size_t)h->nvars * mhdk::cell_plane(h->g) * sizeof(double);
  CK(cudaMemcpyAsync(s.prim, prim, cb, kind, h->stream));
  CK(cudaMemcpyAsync(s.cons, cons, cb, kind, h->stream));
  if (mhd) {
    CK(cudaMemcpyAsync(s.fbx, faceBx, mhdk::xface_plane(h->g) * sizeof(double), kind, h->stream));
    CK(cudaMemcpyAsync(s.fby, faceBy, mhdk::yface_plane(h->g) * sizeof(double), kind, h->stream));
  }
  // a new state starts with clean counters (floor hits, error word)
  CK(cudaMemsetAsync(h->g.status, 0, sizeof(int), h->stream));
  CK(cudaMemsetAsync(h->g.floor_hits, 0, sizeof(unsigned long long), h->stream));
  CK(cudaMemsetAsync(h->g.bad, 0, 2 * sizeof(long long), h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->have_state = 1;
  h->last_cycles_run = 0;
  h->nonfinite_seen = 0;
  return MHD_OK;
}

int mhd2d_upload(void* handle, const double* prim, const double* cons, const double* faceBx,
                 const double* faceBy) {
  return upload_state(handle, prim, cons, faceBx, faceBy, cudaMemcpyHostToDevice);
}

int mhd2d_upload_device(void* handle, const double* prim, const double* cons, const double* faceBx,
                        const double* faceBy) {
  return upload_state(handle, prim, cons, faceBx, faceBy, cudaMemcpyDeviceToDevice);
}

static int advance_impl(Handle* h, double t0, double t_end, long long cycle0, long long max_cycles, double cfl,
                        double dt_fixed, double* t_out, long long* cycle_out, double* t_second_last);

int mhd2d_advance(void* handle, double t0, double t_end, long long cycle0, long long max_cycles, double cfl,
                  double* t_out, long long* cycle_out, double* t_second_last) {
  return advance_impl(static_cast<Handle*>(handle), t0, t_end, cycle0, max_cycles, cfl, 0.0, t_out, cycle_out,
                      t_second_last);
}

int mhd2d_advance_dt(void* handle, double t0, double t_end, long long cycle0, double dt, double* t_out) {
  if (!(dt > 0.0) || !std::isfinite(dt)) return MHD_ERR_ARG;
  return advance_impl(static_cast<Handle*>(handle), t0, t_end, cycle0, cycle0 + 1, 0.0, dt, t_out, nullptr, nullptr);
}

int mhd2d_cfl_dt(void* handle, double cfl, double* dt) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !dt) return MHD_ERR_ARG;
  if (!h->have_state) return MHD_ERR_STATE;
  if (h->g.one_d) return MHD_ERR_STATE;
  const mhdk::StateBuf& st = h->g.st[h->cur];
  const bool mhd = h->g.physics == MHD2D_MHD;
  int rc = mhd2d_cfl_dt_noalloc(h->g.physics, h->g.ny, h->g.nx, h->g.dx, h->g.dy, h->g.gamma, cfl, st.cons,
                                mhd ? st.fbx : nullptr, mhd ? st.fby : nullptr, h->d_dt, h->stream);
  if (rc) return rc;
  CK(cudaMemcpyAsync(dt, h->d_dt, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

static int advance_impl(Handle* h, double t0, double t_end, long long cycle0, long long max_cycles, double cfl,
                        double dt_fixed, double* t_out, long long* cycle_out, double* t_second_last) {
  if (!h) return MHD_ERR_ARG;
  if (!h->have_state) return MHD_ERR_STATE;
  if (!(t0 <= t_end) || cycle0 < 0) return MHD_ERR_ARG;
  static_assert(sizeof(LoopState) % 8 == 0, "layout");
  LoopState init{};
  init.t = t0;
  init.t_end = t_end;
  init.t_prev = t0;
  init.dt = 0.0;
  init.dt_fixed = dt_fixed;
  init.cfl = cfl;
  init.cycle = cycle0;
  init.max_cycles = max_cycles;
  init.cycles_run = 0;
  init.active = 0;
  init.cur = h->cur;
  *h->host_loop = init;
  CK(cudaMemcpyAsync(h->g.loop, h->host_loop, sizeof(LoopState), cudaMemcpyHostToDevice, h->stream));
  long long budget_pairs = 1;
  h->last_launches = 0;
  LoopState st = init;
  while (st.t < st.t_end && st.cycle < st.max_cycles) {
    const int parity = st.cur;
    int rc = build_graph(h, parity);
    if (rc) return rc;
    for (long long k = 0; k < budget_pairs; ++k) CK(cudaGraphLaunch(h->graph[parity], h->stream));
    h->last_launches += budget_pairs * (long long)h->graph_nodes[parity];
    CK(cudaMemcpyAsync(h->host_loop, h->g.loop, sizeof(LoopState), cudaMemcpyDeviceToHost, h->stream));
    int status = 0;
    if (h->arith == MHD2D_ARITH_CHECKED)
      CK(cudaMemcpyAsync(&status, h->g.status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    st = *h->host_loop;
    if (status & mhdk::kStatusIndex) {
      h->cur = st.cur;
      h->last_cycles_run = st.cycles_run;
      return MHD_ERR_INDEX;
    }
    if (!std::isfinite(st.t) || !std::isfinite(st.dt)) {
      h->cur = st.cur;
      h->last_cycles_run = st.cycles_run;
      h->nonfinite_seen = 1;
      return MHD_ERR_NONFINITE;
    }
    // size the next chunk from the remaining cycles (graphs past the end are no-ops)
    long long remaining = st.max_cycles - st.cycle;
    if (st.dt > 0.0) {
      const double est = std::ceil((st.t_end - st.t) / st.dt) + 1.0;
      if (est < (double)remaining) remaining = (long long)est;
    }
    budget_pairs = std::max(1LL, std::min((remaining + 1) / 2, 256LL));
  }
  h->cur = st.cur;
  h->last_cycles_run = st.cycles_run;
  if (t_out) *t_out = st.t;
  if (cycle_out) *cycle_out = st.cycle;
  if (t_second_last) *t_second_last = st.cycles_run > 0 ? st.t_prev : t0;
  return MHD_OK;
}

int mhd2d_run(void* handle, double t_lim, long long max_cycles, double cfl, double save_dt, int save_prec,
              double plot_dt, int plot_prec, mhd2d_stop_fn on_stop, void* user, double* t_out,
              long long* cycle_out, long long* stops_out) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h) return MHD_ERR_ARG;
  if (!h->have_state) return MHD_ERR_STATE;
  auto advance = [&](double t0, double t_end, long long c0, long long cmax, double* t, long long* c, double* tsl,
                     long long* ran) {
    int rc = mhd2d_advance(handle, t0, t_end, c0, cmax, cfl, t, c, tsl);
    *ran = h->last_cycles_run;
    return rc;
  };
  auto revert = [&]() {
    h->cur ^= 1;
    h->last_cycles_run = 0;
  };
  return mhdk::driver_loop(t_lim, max_cycles, save_dt, save_prec, plot_dt, plot_prec, on_stop, user, advance, revert,
                           t_out, cycle_out, stops_out);
}

int mhd2d_set_dt_log(void* handle, double* dt_log, long long capacity) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || capacity < 0 || (capacity > 0 && !dt_log)) return MHD_ERR_ARG;
  if (h->g.dt_log == dt_log && h->g.dt_log_cap == capacity) return MHD_OK;
  CK(cudaStreamSynchronize(h->stream));
  h->g.dt_log = capacity > 0 ? dt_log : nullptr;
  h->g.dt_log_cap = capacity;
  // the kernels take the grid by value: rebuild the cycle graphs with the new log
  for (auto& ge : h->graph)
    if (ge) { cudaGraphExecDestroy(ge); ge = nullptr; }
  return MHD_OK;
}

static int download_state(void* handle, int which, double* prim, double* cons, double* faceBx, double* faceBy,
                          cudaMemcpyKind kind);

int mhd2d_download(void* handle, int which, double* prim, double* cons, double* faceBx, double* faceBy) {
  return download_state(handle, which, prim, cons, faceBx, faceBy, cudaMemcpyDeviceToHost);
}

int mhd2d_download_device(void* handle, int which, double* prim, double* cons, double* faceBx, double* faceBy) {
  return download_state(handle, which, prim, cons, faceBx, faceBy, cudaMemcpyDeviceToDevice);
}

static int download_state(void* handle, int which, double* prim, double* cons, double* faceBx, double* faceBy,
                          cudaMemcpyKind kind) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || (which != 0 && which != 1)) return MHD_ERR_ARG;
  if (!h->have_state) return MHD_ERR_STATE;
  int b = h->cur;
  if (which == 1 && h->last_cycles_run > 0) b ^= 1;
  const mhdk::StateBuf& s = h->g.st[b];
  const size_t cb = (size_t)h->nvars * mhdk::cell_plane(h->g) * sizeof(double);
  if (prim) CK(cudaMemcpyAsync(prim, s.prim, cb, kind, h->stream));
  if (cons) CK(cudaMemcpyAsync(cons, s.cons, cb, kind, h->stream));
  if (h->g.physics == MHD2D_MHD) {
    if (faceBx) CK(cudaMemcpyAsync(faceBx, s.fbx, mhdk::xface_plane(h->g) * sizeof(double), kind, h->stream));
    if (faceBy) CK(cudaMemcpyAsync(faceBy, s.fby, mhdk::yface_plane(h->g) * sizeof(double), kind, h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd2d_state_ptrs(void* handle, int which, double** prim, double** cons, double** faceBx, double** faceBy) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || (which != 0 && which != 1)) return MHD_ERR_ARG;
  int b = h->cur;
  if (which == 1 && h->last_cycles_run > 0) b ^= 1;
  const mhdk::StateBuf& s = h->g.st[b];
  if (prim) *prim = s.prim;
  if (cons) *cons = s.cons;
  if (faceBx) *faceBx = s.fbx;
  if (faceBy) *faceBy = s.fby;
  return MHD_OK;
}

int mhd2d_peek(void* handle, int what, double* out, size_t count) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !out) return MHD_ERR_ARG;
  const Grid& g = h->g;
  const int nv = g.physics == MHD2D_MHD ? 7 : 5;
  const double* src = nullptr;
  size_t n = 0;
  switch (what) {
    case 0: src = g.xl; n = nv * mhdk::xface_plane(g); break;
    case 1: src = g.xr; n = nv * mhdk::xface_plane(g); break;
    case 2: src = g.yl; n = nv * mhdk::yface_plane(g); break;
    case 3: src = g.yr; n = nv * mhdk::yface_plane(g); break;
    case 4: src = g.fx; n = nv * mhdk::xface_plane(g); break;
    case 5: src = g.fy; n = nv * mhdk::yface_plane(g); break;
    case 6: src = g.emf; n = mhdk::corner_plane(g); break;
    case 7: src = g.nfbx; n = mhdk::xface_plane(g); break;
    case 8: src = g.nfby; n = mhdk::yface_plane(g); break;
    default: return MHD_ERR_ARG;
  }
  if (!src || count < n) return MHD_ERR_ARG;
  CK(cudaMemcpyAsync(out, src, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd2d_last_launches(void* handle, long long* launches) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !launches) return MHD_ERR_ARG;
  *launches = h->last_launches;
  return MHD_OK;
}

int mhd2d_device_bytes(void* handle, size_t* bytes) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !bytes) return MHD_ERR_ARG;
  *bytes = h->arena_bytes;
  return MHD_OK;
}

int mhd2d_stats(void* handle, long long* floor_hits, int* nan_flag) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h) return MHD_ERR_ARG;
  unsigned long long hits = 0;
  int status = 0;
  CK(cudaMemcpyAsync(&hits, h->g.floor_hits, sizeof(hits), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(&status, h->g.status, sizeof(status), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (floor_hits) *floor_hits = (long long)hits;
  if (nan_flag) *nan_flag = ((status & mhdk::kStatusNonfinite) || h->nonfinite_seen) ? 1 : 0;
  return MHD_OK;
}

int mhd2d_validate(void* handle, long long* counts) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !counts) return MHD_ERR_ARG;
  if (!h->have_state) return MHD_ERR_STATE;
  unsigned long long c[7] = {};
  CK(cudaMemsetAsync(h->d_check, 0, sizeof(c), h->stream));
  mhdk::enqueue_validate(h->g.physics == MHD2D_MHD, mhdk::cell_plane(h->g), h->g.gamma, h->g.min_d, h->g.min_p,
                         h->g.min_e, h->g.st[h->cur].prim, h->d_check, h->dt_blocks, h->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(c, h->d_check, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < 7; ++k) counts[k] = (long long)c[k];
  return MHD_OK;
}

int mhd2d_check_info(void* handle, long long* line, long long* index) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h) return MHD_ERR_ARG;
  long long bad[2] = {0, 0};
  CK(cudaMemcpyAsync(bad, h->g.bad, sizeof(bad), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (line) *line = bad[0];
  if (index) *index = bad[1];
  return MHD_OK;
}

int mhd2d_stream(void* handle, void** stream) {
  Handle* h = static_cast<Handle*>(handle);
  if (!h || !stream) return MHD_ERR_ARG;
  *stream = h->stream;
  return MHD_OK;
}

}  // extern "C"

extern "C" {

int mhdb_create(int count, const int* ny, const int* nx, const double* dx, const double* dy, const int* bcx,
                const int* bcy, const double* gamma, int physics, int recon, int entropy_fix, double eps,
                double min_d, double min_p, double min_e, int arith, void** handle) {
  if (!handle) return MHD_ERR_ARG;
  *handle = nullptr;
  if (count < 1 || !ny || !nx || !dx || !dy || !bcx || !bcy || !gamma) return MHD_ERR_ARG;
  if (physics != MHD2D_HYDRO && physics != MHD2D_MHD) return MHD_ERR_ARG;
  if (recon != 0 && recon != 1 && recon != 2) return MHD_ERR_ARG;
  if (arith != MHD2D_ARITH_EXACT && arith != MHD2D_ARITH_FAST && arith != MHD2D_ARITH_CHECKED) return MHD_ERR_ARG;
  for (int i = 0; i < count; ++i) {
    if (nx[i] < 2 || ny[i] < 2 || !(dx[i] > 0.0) || !(dy[i] > 0.0)) return MHD_ERR_ARG;
    if ((bcx[i] != 0 && bcx[i] != 1) || (bcy[i] != 0 && bcy[i] != 1)) return MHD_ERR_ARG;
    if ((long long)nx[i] * ny[i] > (1LL << 31)) return MHD_ERR_TOO_LARGE;
  }
  BatchHandle* b = new (std::nothrow) BatchHandle();
  if (!b) return MHD_ERR_NOMEM;
  b->count = count;
  b->physics = physics;
  b->recon = recon;
  b->arith = arith;
  b->nvars = physics == MHD2D_MHD ? 8 : 5;
  b->grids.resize(count);
  b->uploaded.assign(count, 0);
  b->inst_status.assign(count, MHD_OK);
  cudaError_t e = cudaGetDevice(&b->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { free_batch(b); return cuda_fail(e); }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  b->blocks = (unsigned)std::max(1, sms) * 2;

  size_t grid_bytes = 0;
  for (int i = 0; i < count; ++i) {
    Grid& g = b->grids[i];
    g = Grid{};
    g.nx = nx[i]; g.ny = ny[i]; g.dx = dx[i]; g.dy = dy[i]; g.bcx = bcx[i]; g.bcy = bcy[i];
    g.physics = physics; g.recon = recon; g.efix = entropy_fix ? 1 : 0;
    g.gamma = gamma[i]; g.eps = eps; g.min_d = min_d; g.min_p = min_p; g.min_e = min_e;
    grid_bytes += carve_grid(g, b->nvars, nullptr);
  }
  const size_t total = grid_bytes + align256(count * sizeof(LoopState)) + align256(count * sizeof(Grid)) +
                       align256(count * sizeof(int)) + align256(count * sizeof(unsigned long long)) +
                       align256(2 * sizeof(long long));
  e = cudaMalloc(&b->arena, total);
  if (e != cudaSuccess) { free_batch(b); return cuda_fail(e); }
  b->arena_bytes = total;
  char* base = static_cast<char*>(b->arena);
  size_t off = 0;
  for (int i = 0; i < count; ++i) off += carve_grid(b->grids[i], b->nvars, base + off);
  b->d_loops = reinterpret_cast<LoopState*>(base + off);
  off += align256(count * sizeof(LoopState));
  b->d_grids = reinterpret_cast<Grid*>(base + off);
  off += align256(count * sizeof(Grid));
  int* status = reinterpret_cast<int*>(base + off);
  off += align256(count * sizeof(int));
  unsigned long long* hits = reinterpret_cast<unsigned long long*>(base + off);
  off += align256(count * sizeof(unsigned long long));
  long long* bad = reinterpret_cast<long long*>(base + off);
  b->d_status = status;
  b->d_floor_hits = hits;
  for (int i = 0; i < count; ++i) {
    b->grids[i].loop = b->d_loops + i;
    b->grids[i].status = status + i;
    b->grids[i].floor_hits = hits + i;
    b->grids[i].bad = bad;
  }
  e = cudaMemsetAsync(b->arena, 0, total, b->stream);
  b->view.grids = b->d_grids;
  b->view.ninst = count;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_grids, b->grids.data(), count * sizeof(Grid), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_loops, count * sizeof(LoopState));
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) { free_batch(b); return cuda_fail(e); }
  std::memset(b->h_loops, 0, count * sizeof(LoopState));
  const int rc = build_tiles(b, 128);
  if (rc != MHD_OK) { free_batch(b); return rc; }
  *handle = b;
  return MHD_OK;
}

void mhdb_destroy(void* handle) {
  if (handle) free_batch(static_cast<BatchHandle*>(handle));
}

static int batch_upload(void* handle, int inst, const double* prim, const double* cons, const double* faceBx,
                        const double* faceBy, cudaMemcpyKind kind) {
  BatchHandle* b = static_cast<BatchHandle*>(handle);
  if (!b || inst < 0 || inst >= b->count || !prim || !cons) return MHD_ERR_ARG;
  const Grid& g = b->grids[inst];
  const bool mhd = b->physics == MHD2D_MHD;
  if (mhd && (!faceBx || !faceBy)) return MHD_ERR_ARG;
  const mhdk::StateBuf& s = g.st[b->h_loops[inst].cur];
  const size_t cb = (size_t)b->nvars * mhdk::cell_plane(g) * sizeof(double);
  CK(cudaMemcpyAsync(s.prim, prim, cb, kind, b->stream));
  CK(cudaMemcpyAsync(s.cons, cons, cb, kind, b->stream));
  if (mhd) {
    CK(cudaMemcpyAsync(s.fbx, faceBx, mhdk::xface_plane(g) * sizeof(double), kind, b->stream));
    CK(cudaMemcpyAsync(s.fby, faceBy, mhdk::yface_plane(g) * sizeof(double), kind, b->stream));
  }
  CK(cudaMemsetAsync(b->d_status + inst, 0, sizeof(int), b->stream));
  CK(cudaMemsetAsync(b->d_floor_hits + inst, 0, sizeof(unsigned long long), b->stream));
  CK(cudaStreamSynchronize(b->stream));
  b->uploaded[inst] = 1;
  b->h_loops[inst].cycles_run = 0;
  return MHD_OK;
}

int mhdb_upload(void* handle, int inst, const double* prim, const double* cons, const double* faceBx,
                const double* faceBy) {
  return batch_upload(handle, inst, prim, cons, faceBx, faceBy, cudaMemcpyHostToDevice);
}

int mhdb_upload_device(void* handle, int inst, const double* prim, const double* cons, const double* faceBx,
                       const double* faceBy) {
  return batch_upload(handle, inst, prim, cons, faceBx, faceBy, cudaMemcpyDeviceToDevice);
}

int mhdb_pack_state(void* handle, int inst, double* dst) {
  BatchHandle* b = static_cast<BatchHandle*>(handle);
  if (!b || inst < 0 || inst >= b->count || !dst || b->physics != MHD2D_MHD) return MHD_ERR_ARG;
  if (!b->uploaded[inst]) return MHD_ERR_STATE;
  const Grid& g = b->grids[inst];
  const mhdk::StateBuf& s = g.st[b->h_loops[inst].cur];
  const size_t cp = (size_t)b->nvars * mhdk::cell_plane(g), xp = mhdk::xface_plane(g), yp = mhdk::yface_plane(g);
  CK(cudaMemcpyAsync(dst, s.prim, cp * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  CK(cudaMemcpyAsync(dst + cp, s.cons, cp * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  CK(cudaMemcpyAsync(dst + 2 * cp, s.fbx, xp * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  CK(cudaMemcpyAsync(dst + 2 * cp + xp, s.fby, yp * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return MHD_OK;
}

int mhdb_state_ptrs(void* handle, int inst, int which, double** prim, double** cons, double** faceBx,
                    double** faceBy) {
  BatchHandle* b = static_cast<BatchHandle*>(handle);
  if (!b || inst < 0 || inst >= b->count || (which != 0 && which != 1)) return MHD_ERR_ARG;
  if (!b->uploaded[inst]) return MHD_ERR_STATE;
  int buf = b->h_loops[inst].cur;
  if (which == 1 && b->h_loops[inst].cycles_run > 0) buf ^= 1;
  const mhdk::StateBuf& s = b->grids[inst].st[buf];
  if (prim) *prim = s.prim;
  if (cons) *cons = s.cons;
  if (faceBx) *faceBx = s.fbx;
  if (faceBy) *faceBy = s.fby;
  return MHD_OK;
}

int mhdb_advance(void* handle, const double* t0, const double* t_end, const long long* cycle0,
                 const long long* max_cycles, double cfl, double* t_out, long long* cycle_out) {
  BatchHandle* b = static_cast<BatchHandle*>(handle);
  if (!b || !t0 || !t_end || !cycle0 || !max_cycles) return MHD_ERR_ARG;
  for (int i = 0; i < b->count; ++i) {
    if (!b->uploaded[i]) return MHD_ERR_STATE;
    if (!(t0[i] <= t_end[i]) || cycle0[i] < 0) return MHD_ERR_ARG;
  }
  for (int i = 0; i < b->count; ++i) {
    LoopState& L = b->h_loops[i];
    const int cur = L.cur;
    L = LoopState{};
    L.t = t0[i]; L.t_end = t_end[i]; L.t_prev = t0[i]; L.cfl = cfl;
    L.cycle = cycle0[i]; L.max_cycles = max_cycles[i]; L.cur = cur;
  }
  b->inst_status.assign(b->count, MHD_OK);
  CK(cudaMemcpyAsync(b->d_loops, b->h_loops, b->count * sizeof(LoopState), cudaMemcpyHostToDevice, b->stream));
  int rc = build_batch_graph(b);
  if (rc) return rc;
  b->last_launches = 0;
  long long budget = 1;
  for (;;) {
    bool running = false;
    long long remaining = 0;
    for (int i = 0; i < b->count; ++i) {
      const LoopState& L = b->h_loops[i];
      if (L.t < L.t_end && L.cycle < L.max_cycles) {
        running = true;
        long long r = L.max_cycles - L.cycle;
        if (L.dt > 0.0) {
          const double est = std::ceil((L.t_end - L.t) / L.dt) + 1.0;
          if (est < (double)r) r = (long long)est;
        }
        remaining = std::max(remaining, r);
      }
    }
    if (!running) break;
    for (long long k = 0; k < budget; ++k) CK(cudaGraphLaunch(b->graph, b->stream));
    b->last_launches += budget * (long long)b->graph_nodes;
    CK(cudaMemcpyAsync(b->h_loops, b->d_loops, b->count * sizeof(LoopState), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    if (b->arith == MHD2D_ARITH_CHECKED) {
      std::vector<int> st(b->count);
      CK(cudaMemcpy(st.data(), b->d_status, b->count * sizeof(int), cudaMemcpyDeviceToHost));
      for (int i = 0; i < b->count; ++i)
        if (st[i] & mhdk::kStatusIndex) return MHD_ERR_INDEX;
    }
    // An instance whose time or dt went non-finite has stopped by itself (NaN < t_end
    // is false, so its kernels skip it); the others keep advancing.
    for (int i = 0; i < b->count; ++i)
      if (!std::isfinite(b->h_loops[i].t) || !std::isfinite(b->h_loops[i].dt)) b->inst_status[i] = MHD_ERR_NONFINITE;
    budget = std::max(1LL, std::min(remaining - budget, 512LL));
  }
  int rc_all = MHD_OK;
  for (int i = 0; i < b->count; ++i) {
    if (t_out) t_out[i] = b->h_loops[i].t;
    if (cycle_out) cycle_out[i] = b->h_loops[i].cycle;
    if (b->inst_status[i] != MHD_OK) rc_all = b->inst_status[i];
  }
  return rc_all;
}

int mhdb_stats(void* handle, long long* floor_hits, int* nan_flag) {
  BatchHandle* b = static_cast<BatchHandle*>(handle);
  if (!b) return MHD_ERR_ARG;
  std::vector<unsigned long long> hits(b->count);
  std::vector<int> st(b->count);
  CK(cudaMemcpyAsync(hits.data(), b->d_floor_hits, b->count * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     b->stream));
  CK(cudaMemcpyAsync(st.data(), b->d_status, b->count * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < b->count; ++i) {
    if (floor_hits) floor_hits[i] = (long long)hits[i];
    if (nan_flag) nan_flag[i] = ((st[i] & mhdk::kStatusNonfinite) || b->inst_status[i] != MHD_OK) ? 1 : 0;
  }
  return MHD_OK;
}

int mhdb_instance_status(void* handle, int* status) {
  BatchHandle* b = static_cast<BatchHandle*>(handle);
  if (!b || !status) return MHD_ERR_ARG;
  for (int i = 0; i < b->count; ++i) status[i] = b->inst_status[i];
  return MHD_OK;
}

int mhdb_download(void* handle, int inst, int which, double* prim, double* cons, double* faceBx,
                  double* faceBy) {
  BatchHandle* b = static_cast<BatchHandle*>(handle);
  if (!b || inst < 0 || inst >= b->count || (which != 0 && which != 1)) return MHD_ERR_ARG;
  if (!b->uploaded[inst]) return MHD_ERR_STATE;
  const Grid& g = b->grids[inst];
  int buf = b->h_loops[inst].cur;
  if (which == 1 && b->h_loops[inst].cycles_run > 0) buf ^= 1;
  const mhdk::StateBuf& s = g.st[buf];
  const size_t cb = (size_t)b->nvars * mhdk::cell_plane(g) * sizeof(double);
  if (prim) CK(cudaMemcpyAsync(prim, s.prim, cb, cudaMemcpyDeviceToHost, b->stream));
  if (cons) CK(cudaMemcpyAsync(cons, s.cons, cb, cudaMemcpyDeviceToHost, b->stream));
  if (b->physics == MHD2D_MHD) {
    if (faceBx) CK(cudaMemcpyAsync(faceBx, s.fbx, mhdk::xface_plane(g) * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    if (faceBy) CK(cudaMemcpyAsync(faceBy, s.fby, mhdk::yface_plane(g) * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  }
  CK(cudaStreamSynchronize(b->stream));
  return MHD_OK;
}

int mhdb_configure(void* handle, int tile_width, int fuse, int blocks) {
  BatchHandle* b = static_cast<BatchHandle*>(handle);
  if (!b || blocks < 1 || (fuse != 1 && fuse != 2)) return MHD_ERR_ARG;
  if (tile_width != 32 && tile_width != 64 && tile_width != 128) return MHD_ERR_ARG;
  if (tile_width != b->tile_width) {
    const int rc = build_tiles(b, tile_width);
    if (rc != MHD_OK) return rc;
  }
  b->fuse = fuse;
  b->blocks = (unsigned)blocks;
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
  return MHD_OK;
}

int mhdb_set_tiles(void* handle, int space, const int* tiles, long long count) {
  BatchHandle* b = static_cast<BatchHandle*>(handle);
  if (!b || space < 0 || space >= mhdk::kNumSpaces || count < 0 || (count > 0 && !tiles)) return MHD_ERR_ARG;
  std::vector<int4> t((size_t)count);
  for (long long k = 0; k < count; ++k)
    t[k] = make_int4(tiles[4 * k], tiles[4 * k + 1], tiles[4 * k + 2], tiles[4 * k + 3]);
  if (!tiles_valid(b, space, b->tile_width, t)) return MHD_ERR_ARG;
  std::vector<int4> all[mhdk::kNumSpaces];
  for (int sp = 0; sp < mhdk::kNumSpaces; ++sp) all[sp] = sp == space ? t : b->host_tiles[sp];
  CK(cudaStreamSynchronize(b->stream));
  const int rc = install_tiles(b, b->tile_width, all);
  if (rc != MHD_OK) return rc;
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
  return MHD_OK;
}

int mhdb_get_tiles(void* handle, int space, int* tiles, long long capacity, long long* count) {
  BatchHandle* b = static_cast<BatchHandle*>(handle);
  if (!b || space < 0 || space >= mhdk::kNumSpaces || !count) return MHD_ERR_ARG;
  const std::vector<int4>& t = b->host_tiles[space];
  *count = (long long)t.size();
  if (!tiles) return MHD_OK;
  if (capacity < (long long)t.size()) return MHD_ERR_ARG;
  for (size_t k = 0; k < t.size(); ++k) {
    tiles[4 * k] = t[k].x; tiles[4 * k + 1] = t[k].y; tiles[4 * k + 2] = t[k].z; tiles[4 * k + 3] = t[k].w;
  }
  return MHD_OK;
}

int mhdb_info(void* handle, long long* launches, size_t* device_bytes, int* blocks, void** stream) {
  // blocks of each persistent launch; see mhdb_configure for the other knobs
  BatchHandle* b = static_cast<BatchHandle*>(handle);
  if (!b) return MHD_ERR_ARG;
  if (launches) *launches = b->last_launches;
  if (device_bytes) *device_bytes = b->arena_bytes;
  if (blocks) *blocks = (int)b->blocks;
  if (stream) *stream = b->stream;
  return MHD_OK;
}

}  // extern "C"
