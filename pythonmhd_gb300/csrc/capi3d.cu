// C ABI of the 3D Godunov step (hydro and MHD): handle lifetime, host<->device copies and
// the device-resident evolve loop, CUDA graphs of two cycles replayed in chunks as
// in 2D.  State arrays cross the boundary in the reference's 3D layout
// (nvars, ny, nx, nz), z fastest, which is also the device layout.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>

#include "../../include/pythonmhd_gb300.h"
#include "driver_loop.h"
#include "godunov3d_types.h"

namespace mhdk {
namespace exact {
void enqueue_cycle3(const Grid3& g, int parity, int dt_blocks, cudaStream_t s);
}  // namespace exact
namespace fast {
void enqueue_cycle3(const Grid3& g, int parity, int dt_blocks, cudaStream_t s);
}  // namespace fast
}  // namespace mhdk

using mhdk::Grid3;
using mhdk::LoopState;

namespace {

struct Handle3 {
  Grid3 g{};
  int arith = 0;
  int nvars = 5;
  cudaStream_t stream = nullptr;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  LoopState* host_loop = nullptr;  // pinned
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  size_t graph_nodes[2] = {0, 0};
  int cur = 0;
  int have_state = 0;
  long long last_cycles_run = 0;
  long long last_launches = 0;
  int dt_blocks = 0;
};

int fail(cudaError_t e) { return e == cudaErrorMemoryAllocation ? MHD_ERR_NOMEM : MHD_ERR_CUDA; }

#define CK3(call)                              \
  do {                                         \
    cudaError_t _e = (call);                   \
    if (_e != cudaSuccess) return fail(_e);    \
  } while (0)

size_t al256(size_t n) { return (n + 255) & ~size_t(255); }

// Lay out every buffer from `base` (256-byte aligned pieces); returns the bytes used.
size_t carve3(Grid3& g, int nvars, char* base) {
  const bool mhd = g.physics == MHD2D_MHD;
  const int nv = mhd ? 7 : 5, nw = mhd ? 42 : 10;
  const size_t cp = mhdk::cells3(g);
  g.ext_plane = std::max(mhdk::plane3(g, 0, 2), std::max(mhdk::plane3(g, 1, 2), mhdk::plane3(g, 2, 2)));
  size_t off = 0;
  auto take = [&](double** p, size_t n) {
    if (base) *p = reinterpret_cast<double*>(base + off);
    off += al256(n * sizeof(double));
  };
  for (int b = 0; b < 2; ++b) {
    take(&g.st[b].prim, (size_t)nvars * cp);
    take(&g.st[b].cons, (size_t)nvars * cp);
    for (int d = 0; d < 3; ++d) {
      if (mhd) take(&g.st[b].fb[d], mhdk::plane3(g, d, 1));
      else g.st[b].fb[d] = nullptr;
    }
  }
  for (int d = 0; d < 3; ++d) {
    const size_t fp = mhdk::plane3(g, d, 1);
    take(&g.wl[d], nv * fp);
    take(&g.wr[d], nv * fp);
    take(&g.f[d], nv * fp);
    if (mhd) {
      take(&g.ul[d], nv * fp);
      take(&g.ur[d], nv * fp);
      take(&g.emf[d], mhdk::edges3(g));
      take(&g.nfb[d], fp);
      take(&g.ce[d], cp);
    } else {
      g.ul[d] = g.ur[d] = g.emf[d] = g.nfb[d] = g.ce[d] = nullptr;
    }
  }
  if (g.recon >= 1) {
    take(&g.slopes, nv * g.ext_plane);
    take(&g.eig, nw * g.ext_plane);
  } else {
    g.slopes = nullptr;
    g.eig = nullptr;
  }
  return off;
}

void enqueue3(Handle3* h, int parity) {
  if (h->arith == MHD2D_ARITH_EXACT) mhdk::exact::enqueue_cycle3(h->g, parity, h->dt_blocks, h->stream);
  else mhdk::fast::enqueue_cycle3(h->g, parity, h->dt_blocks, h->stream);
}

int build_graph3(Handle3* h, int parity) {
  if (h->graph[parity]) return MHD_OK;
  cudaGraph_t graph = nullptr;
  CK3(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  enqueue3(h, parity);
  enqueue3(h, parity ^ 1);
  cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
  if (e != cudaSuccess) return fail(e);
  size_t nodes = 0;
  cudaGraphGetNodes(graph, nullptr, &nodes);
  h->graph_nodes[parity] = nodes;
  e = cudaGraphInstantiate(&h->graph[parity], graph, 0);
  cudaGraphDestroy(graph);
  return e == cudaSuccess ? MHD_OK : fail(e);
}

int upload3(Handle3* h, const double* prim, const double* cons, const double* const* fb, cudaMemcpyKind kind) {
  if (!h || !prim || !cons) return MHD_ERR_ARG;
  const bool mhd = h->g.physics == MHD2D_MHD;
  if (mhd && (!fb[0] || !fb[1] || !fb[2])) return MHD_ERR_ARG;
  const mhdk::StateBuf3& s = h->g.st[h->cur];
  const size_t cb = (size_t)h->nvars * mhdk::cells3(h->g) * sizeof(double);
  CK3(cudaMemcpyAsync(s.prim, prim, cb, kind, h->stream));
  CK3(cudaMemcpyAsync(s.cons, cons, cb, kind, h->stream));
  if (mhd)
    for (int d = 0; d < 3; ++d)
      CK3(cudaMemcpyAsync(s.fb[d], fb[d], mhdk::plane3(h->g, d, 1) * sizeof(double), kind, h->stream));
  CK3(cudaStreamSynchronize(h->stream));
  h->have_state = 1;
  h->last_cycles_run = 0;
  return MHD_OK;
}

}  // namespace

extern "C" {

int mhd3d_create(int ny, int nx, int nz, double dx, double dy, double dz, int bcx, int bcy, int bcz,
                 double gamma, int physics, int recon, int entropy_fix, double eps, double min_d, double min_p,
                 double min_e, int arith, void** handle) {
  if (!handle) return MHD_ERR_ARG;
  *handle = nullptr;
  if (nx < 2 || ny < 2 || nz < 2 || !(dx > 0.0) || !(dy > 0.0) || !(dz > 0.0)) return MHD_ERR_ARG;
  for (int bc : {bcx, bcy, bcz})
    if (bc != 0 && bc != 1) return MHD_ERR_ARG;
  if (physics != MHD2D_HYDRO && physics != MHD2D_MHD) return MHD_ERR_ARG;
  if (recon != 0 && recon != 1 && recon != 2) return MHD_ERR_ARG;
  if (arith != MHD2D_ARITH_EXACT && arith != MHD2D_ARITH_FAST) return MHD_ERR_ARG;
  // work items are 32-bit linear indices of the largest (sweep-extended) array
  const long long big = (long long)(nx + 2) * (ny + 2) * (nz + 2);
  if (big >= (1LL << 32) - 1024) return MHD_ERR_TOO_LARGE;

  Handle3* h = new (std::nothrow) Handle3();
  if (!h) return MHD_ERR_NOMEM;
  Grid3& g = h->g;
  g.n[0] = nx; g.n[1] = ny; g.n[2] = nz;
  g.d[0] = dx; g.d[1] = dy; g.d[2] = dz;
  g.bc[0] = bcx; g.bc[1] = bcy; g.bc[2] = bcz;
  g.physics = physics; g.recon = recon; g.efix = entropy_fix ? 1 : 0;
  g.gamma = gamma; g.eps = eps; g.min_d = min_d; g.min_p = min_p; g.min_e = min_e;
  h->arith = arith;
  h->nvars = physics == MHD2D_MHD ? 8 : 5;

  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete h; return fail(e); }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  h->dt_blocks = std::max(1, sms) * 8;

  const size_t total = carve3(g, h->nvars, nullptr) + al256(sizeof(LoopState)) + al256(sizeof(int));
  e = cudaMalloc(&h->arena, total);
  if (e != cudaSuccess) {
    cudaStreamDestroy(h->stream);
    delete h;
    return fail(e);
  }
  h->arena_bytes = total;
  char* base = static_cast<char*>(h->arena);
  size_t off = carve3(g, h->nvars, base);
  g.loop = reinterpret_cast<LoopState*>(base + off);
  off += al256(sizeof(LoopState));
  g.status = reinterpret_cast<int*>(base + off);
  e = cudaMemsetAsync(h->arena, 0, total, h->stream);
  if (e == cudaSuccess) e = cudaMallocHost(&h->host_loop, sizeof(LoopState));
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    if (h->host_loop) cudaFreeHost(h->host_loop);
    cudaFree(h->arena);
    cudaStreamDestroy(h->stream);
    delete h;
    return fail(e);
  }
  *handle = h;
  return MHD_OK;
}

void mhd3d_destroy(void* handle) {
  Handle3* h = static_cast<Handle3*>(handle);
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& ge : h->graph)
    if (ge) cudaGraphExecDestroy(ge);
  if (h->host_loop) cudaFreeHost(h->host_loop);
  if (h->arena) cudaFree(h->arena);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int mhd3d_upload(void* handle, const double* prim, const double* cons, const double* faceBx, const double* faceBy,
                 const double* faceBz) {
  const double* fb[3] = {faceBx, faceBy, faceBz};
  return upload3(static_cast<Handle3*>(handle), prim, cons, fb, cudaMemcpyHostToDevice);
}

int mhd3d_upload_device(void* handle, const double* prim, const double* cons, const double* faceBx,
                        const double* faceBy, const double* faceBz) {
  const double* fb[3] = {faceBx, faceBy, faceBz};
  return upload3(static_cast<Handle3*>(handle), prim, cons, fb, cudaMemcpyDeviceToDevice);
}

int mhd3d_advance(void* handle, double t0, double t_end, long long cycle0, long long max_cycles, double cfl,
                  double* t_out, long long* cycle_out, double* t_second_last) {
  Handle3* h = static_cast<Handle3*>(handle);
  if (!h) return MHD_ERR_ARG;
  if (!h->have_state) return MHD_ERR_STATE;
  if (!(t0 <= t_end) || cycle0 < 0) return MHD_ERR_ARG;
  LoopState init{};
  init.t = t0;
  init.t_end = t_end;
  init.t_prev = t0;
  init.cfl = cfl;
  init.cycle = cycle0;
  init.max_cycles = max_cycles;
  init.cur = h->cur;
  *h->host_loop = init;
  CK3(cudaMemcpyAsync(h->g.loop, h->host_loop, sizeof(LoopState), cudaMemcpyHostToDevice, h->stream));
  long long pairs = 1;
  h->last_launches = 0;
  LoopState st = init;
  while (st.t < st.t_end && st.cycle < st.max_cycles) {
    const int parity = st.cur;
    int rc = build_graph3(h, parity);
    if (rc) return rc;
    for (long long k = 0; k < pairs; ++k) CK3(cudaGraphLaunch(h->graph[parity], h->stream));
    h->last_launches += pairs * (long long)h->graph_nodes[parity];
    CK3(cudaMemcpyAsync(h->host_loop, h->g.loop, sizeof(LoopState), cudaMemcpyDeviceToHost, h->stream));
    CK3(cudaStreamSynchronize(h->stream));
    st = *h->host_loop;
    if (!std::isfinite(st.t) || !std::isfinite(st.dt)) {
      h->cur = st.cur;
      h->last_cycles_run = st.cycles_run;
      return MHD_ERR_NONFINITE;
    }
    long long remaining = st.max_cycles - st.cycle;
    if (st.dt > 0.0) {
      const double est = std::ceil((st.t_end - st.t) / st.dt) + 1.0;
      if (est < (double)remaining) remaining = (long long)est;
    }
    pairs = std::max(1LL, std::min((remaining + 1) / 2, 256LL));
  }
  h->cur = st.cur;
  h->last_cycles_run = st.cycles_run;
  if (t_out) *t_out = st.t;
  if (cycle_out) *cycle_out = st.cycle;
  if (t_second_last) *t_second_last = st.cycles_run > 0 ? st.t_prev : t0;
  return MHD_OK;
}

int mhd3d_run(void* handle, double t_lim, long long max_cycles, double cfl, double save_dt, int save_prec,
              double plot_dt, int plot_prec, mhd2d_stop_fn on_stop, void* user, double* t_out,
              long long* cycle_out, long long* stops_out) {
  Handle3* h = static_cast<Handle3*>(handle);
  if (!h) return MHD_ERR_ARG;
  if (!h->have_state) return MHD_ERR_STATE;
  auto advance = [&](double t0, double t_end, long long c0, long long cmax, double* t, long long* c, double* tsl,
                     long long* ran) {
    int rc = mhd3d_advance(handle, t0, t_end, c0, cmax, cfl, t, c, tsl);
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

int mhd3d_download(void* handle, int which, double* prim, double* cons, double* faceBx, double* faceBy,
                   double* faceBz) {
  Handle3* h = static_cast<Handle3*>(handle);
  if (!h || (which != 0 && which != 1)) return MHD_ERR_ARG;
  if (!h->have_state) return MHD_ERR_STATE;
  int b = h->cur;
  if (which == 1 && h->last_cycles_run > 0) b ^= 1;
  const mhdk::StateBuf3& s = h->g.st[b];
  const size_t cb = (size_t)h->nvars * mhdk::cells3(h->g) * sizeof(double);
  if (prim) CK3(cudaMemcpyAsync(prim, s.prim, cb, cudaMemcpyDeviceToHost, h->stream));
  if (cons) CK3(cudaMemcpyAsync(cons, s.cons, cb, cudaMemcpyDeviceToHost, h->stream));
  double* fb[3] = {faceBx, faceBy, faceBz};
  if (h->g.physics == MHD2D_MHD)
    for (int d = 0; d < 3; ++d)
      if (fb[d])
        CK3(cudaMemcpyAsync(fb[d], s.fb[d], mhdk::plane3(h->g, d, 1) * sizeof(double), cudaMemcpyDeviceToHost,
                            h->stream));
  CK3(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd3d_state_ptrs(void* handle, int which, double** prim, double** cons, double** faceBx, double** faceBy,
                     double** faceBz) {
  Handle3* h = static_cast<Handle3*>(handle);
  if (!h || (which != 0 && which != 1)) return MHD_ERR_ARG;
  int b = h->cur;
  if (which == 1 && h->last_cycles_run > 0) b ^= 1;
  const mhdk::StateBuf3& s = h->g.st[b];
  if (prim) *prim = s.prim;
  if (cons) *cons = s.cons;
  if (faceBx) *faceBx = s.fb[0];
  if (faceBy) *faceBy = s.fb[1];
  if (faceBz) *faceBz = s.fb[2];
  return MHD_OK;
}

int mhd3d_info(void* handle, long long* last_launches, size_t* device_bytes, void** stream) {
  Handle3* h = static_cast<Handle3*>(handle);
  if (!h) return MHD_ERR_ARG;
  if (last_launches) *last_launches = h->last_launches;
  if (device_bytes) *device_bytes = h->arena_bytes;
  if (stream) *stream = h->stream;
  return MHD_OK;
}

}  // extern "C"
