// FP64 pipe throughput probe: DFMA / DADD / DMUL / sqrt / div lane-operations per
// second on the current device, and two forms of a compare-and-select: an FP64
// compare (DSETP) and the same test on the 64-bit pattern (integer pipe).  Eight
// (four for sqrt/div) independent chains per thread, 4-16 resident blocks of 256
// threads per SM.  bench.py runs it to get the FP64 roof of the step on the same
// box; prints one JSON line with --json.
#include <cstdio>
#include <cstring>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("err %s line %d\n", cudaGetErrorString(e), __LINE__); return 1;}}while(0)
// one compare-and-select step that moves x by one or three units in the last place
template<int OP>
__device__ __forceinline__ double cmp_step(double x, double a, long long ab) {
  const long long xb = __double_as_longlong(x);
  const bool gt = OP == 5 ? (x > a) : (xb > ab);
  return __longlong_as_double(xb + (gt ? 1LL : 3LL));
}
template<int OP>
__global__ void k(double* out, int iters, double a, double b) {
  const long long ab = __double_as_longlong(a);
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < iters; ++i) {
    if (OP == 0) { x0 = fma(x0,a,b); x1 = fma(x1,a,b); x2 = fma(x2,a,b); x3 = fma(x3,a,b); x4 = fma(x4,a,b); x5 = fma(x5,a,b); x6 = fma(x6,a,b); x7 = fma(x7,a,b); }
    if (OP == 1) { x0 = __dadd_rn(x0,a); x1 = __dadd_rn(x1,a); x2 = __dadd_rn(x2,a); x3 = __dadd_rn(x3,a); x4 = __dadd_rn(x4,a); x5 = __dadd_rn(x5,a); x6 = __dadd_rn(x6,a); x7 = __dadd_rn(x7,a); }
    if (OP == 2) { x0 = __dmul_rn(x0,a); x1 = __dmul_rn(x1,a); x2 = __dmul_rn(x2,a); x3 = __dmul_rn(x3,a); x4 = __dmul_rn(x4,a); x5 = __dmul_rn(x5,a); x6 = __dmul_rn(x6,a); x7 = __dmul_rn(x7,a); }
    if (OP == 3) { x0 = sqrt(x0+a); x1 = sqrt(x1+a); x2 = sqrt(x2+a); x3 = sqrt(x3+a); }
    if (OP == 4) { x0 = b/(x0+a); x1 = b/(x1+a); x2 = b/(x2+a); x3 = b/(x3+a); }
    if (OP >= 5) { x0 = cmp_step<OP>(x0,a,ab); x1 = cmp_step<OP>(x1,a,ab); x2 = cmp_step<OP>(x2,a,ab); x3 = cmp_step<OP>(x3,a,ab);
                   x4 = cmp_step<OP>(x4,a,ab); x5 = cmp_step<OP>(x5,a,ab); x6 = cmp_step<OP>(x6,a,ab); x7 = cmp_step<OP>(x7,a,ab); }
  }
  double s = x0+x1+x2+x3+x4+x5+x6+x7;
  if (s == 12345.678) out[0] = s;
}
int main(int argc, char** argv) {
  const bool json = argc > 1 && std::strcmp(argv[1], "--json") == 0;
  double best[7] = {0, 0, 0, 0, 0, 0, 0};
  double* d; CK(cudaMalloc(&d, 8));
  int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  int clk; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  if (!json) printf("SMs %d clock %d kHz\n", sms, clk);
  const char* names[] = {"DFMA", "DADD", "DMUL", "SQRT", "DIV", "DSETP", "ICMP64"};
  for (int blocks_per_sm : {4, 8, 16}) {
  for (int op = 0; op < 7; ++op) {
    const bool eight = op < 3 || op >= 5;
    int iters = eight ? 4096 : 512;
    dim3 grid(sms * blocks_per_sm), block(256);
    cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0);
      switch (op) { case 0: k<0><<<grid,block>>>(d, iters, 0.9999, 1e-3); break; case 1: k<1><<<grid,block>>>(d, iters, 1e-9, 0); break;
        case 2: k<2><<<grid,block>>>(d, iters, 1.0000001, 0); break; case 3: k<3><<<grid,block>>>(d, iters, 1.5, 0); break; case 4: k<4><<<grid,block>>>(d, iters, 1.5, 1.1); break;
        case 5: k<5><<<grid,block>>>(d, iters, 1.5, 0); break; case 6: k<6><<<grid,block>>>(d, iters, 1.5, 0); break; }
      cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
      float ms; cudaEventElapsedTime(&ms, e0, e1);
      double ops = (double)grid.x * block.x * iters * (eight ? 8 : 4);
      const double g = ops / ms / 1e6;
      if (rep == 2 && g > best[op]) best[op] = g;
      if (rep == 2 && !json) printf("bpsm %2d %s: %.3f ms  %.3f Gop/s (lane-ops) %s\n", blocks_per_sm, names[op], ms, g, op==0 ? "(x2 = FLOP)" : "");
    }
  }}
  if (json) printf("{\"sms\": %d, \"clock_khz\": %d, \"dfma_gops\": %.3f, \"dadd_gops\": %.3f, \"dmul_gops\": %.3f, \"sqrt_gops\": %.3f, \"div_gops\": %.3f, \"dsetp_gops\": %.3f, \"icmp64_gops\": %.3f}\n", sms, clk, best[0], best[1], best[2], best[3], best[4], best[5], best[6]);
  return 0;
}
