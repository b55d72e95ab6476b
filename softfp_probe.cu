// Throughput probe of the integer-pipe FP64 arithmetic (pythonmhd_gb300/csrc/softfp.cuh):
// its add/sub, multiply, divide and square root alone and mixed with FP64-pipe multiplies,
// against the FP64 instructions, in lane-operations per second; and a bit-for-bit check of
// every operation against the FP64 instruction on 2 x 1.3 G device-generated operand pairs.
// Blocks of 128 threads, 2 / 4 / 8 resident per SM; each thread runs independent chains.
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -fmad=false -Ipythonmhd_gb300/csrc \
//        softfp_probe.cu -o _build/softfp_probe && _build/softfp_probe
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
#include "softfp.cuh"
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("err %s line %d\n", cudaGetErrorString(e), __LINE__); return 1;}}while(0)

__device__ __forceinline__ uint64_t mix(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// bitwise check: each thread checks `per` pairs; one counter per op
__global__ void k_check(unsigned long long* bad, long long per, int mode) {
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  unsigned long long nb[5] = {0, 0, 0, 0, 0};
  for (long long i = 0; i < per; ++i) {
    const uint64_t r1 = mix(tid * 0x100000001ull + i * 2), r2 = mix(tid * 0x100000001ull + i * 2 + 1);
    uint64_t xb, yb;
    if (mode == 0) { xb = r1; yb = r2; }
    else {  // moderate exponents, close values
      xb = (r1 & 0x800fffffffffffffull) | ((uint64_t)(1000 + (r1 >> 52) % 48) << 52);
      yb = (r2 & 0x800fffffffffffffull) | ((uint64_t)(1000 + (r2 >> 52) % 48) << 52);
      if ((r2 & 7) == 0) yb = (xb ^ 0x8000000000000000ull) ^ (r2 >> 40);
    }
    const double x = __longlong_as_double(xb), y = __longlong_as_double(yb);
    const double s = sfp::add(x, y), d = sfp::sub(x, y), p = sfp::mul(x, y);
    const double hs = __dadd_rn(x, y), hd = __dsub_rn(x, y), hp = __dmul_rn(x, y);
    auto ne = [](double a, double b) { return (a != a) ? (b == b) : (__double_as_longlong(a) != __double_as_longlong(b)); };
    nb[0] += ne(hs, s); nb[1] += ne(hd, d); nb[2] += ne(hp, p);
    nb[3] += ne(__ddiv_rn(x, y), sfp::div(x, y)); nb[4] += ne(__dsqrt_rn(x), sfp::sqrt(x));
  }
  if (nb[0]) atomicAdd(&bad[0], nb[0]);
  if (nb[1]) atomicAdd(&bad[1], nb[1]);
  if (nb[2]) atomicAdd(&bad[2], nb[2]);
  if (nb[3]) atomicAdd(&bad[3], nb[3]);
  if (nb[4]) atomicAdd(&bad[4], nb[4]);
}

// throughput: H chains of FP64-pipe multiplies and S chains of the operation under test per
// iteration (SOP 0 integer-pipe mul, 1 integer-pipe add/sub, 2 FP64 add/sub, 3 integer-pipe
// division, 4 FP64 division, 5 integer-pipe sqrt, 6 FP64 sqrt; the division and sqrt chains
// add one FP64 add per step to keep their operand moving)
template <int H, int S, int SOP>
__global__ void __launch_bounds__(128) k_tp(double* out, int iters, double a, double b) {
  double h[H > 0 ? H : 1], s[S > 0 ? S : 1];
#pragma unroll
  for (int j = 0; j < (H > 0 ? H : 1); ++j) h[j] = 1.0 + threadIdx.x * 1e-3 + j;
#pragma unroll
  for (int j = 0; j < (S > 0 ? S : 1); ++j) s[j] = 1.5 + threadIdx.x * 1e-3 + j;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < H; ++j) h[j] = __dmul_rn(h[j], a);
#pragma unroll
    for (int j = 0; j < S; ++j) {
      if (SOP == 0) s[j] = sfp::mul(s[j], a);
      else if (SOP == 1) s[j] = (j & 1) ? sfp::sub(s[j], b) : sfp::add(s[j], b);
      else if (SOP == 2) s[j] = (j & 1) ? __dsub_rn(s[j], b) : __dadd_rn(s[j], b);
      else if (SOP == 3) s[j] = sfp::div(b, s[j] + a);          // sw div (hw add)
      else if (SOP == 4) s[j] = __ddiv_rn(b, s[j] + a);         // hw div
      else if (SOP == 5) s[j] = sfp::sqrt(s[j] + a);            // sw sqrt
      else s[j] = __dsqrt_rn(s[j] + a);                         // hw sqrt
    }
  }
  double t = 0;
#pragma unroll
  for (int j = 0; j < H; ++j) t += h[j];
#pragma unroll
  for (int j = 0; j < S; ++j) t += s[j];
  if (t == 12345.678) out[0] = t;
}

template <int H, int S, int SOP>
int run(const char* name, int sms, double* d, int bpsm, int iters) {
  dim3 grid(sms * bpsm), block(128);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_tp<H, S, SOP><<<grid, block>>>(d, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  const double lanes = (double)grid.x * block.x * iters;
  const double hw = lanes * H / best / 1e6, sw = lanes * S / best / 1e6;
  printf("%-26s blocks/SM %2d  %8.3f ms  FP64 mul chains %8.1f G/s  tested op %8.1f G/s  total %8.1f G/s\n",
         name, bpsm, best, hw, sw, hw + sw);
  return 0;
}

int main() {
  int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  double* d; CK(cudaMalloc(&d, 8));
  unsigned long long* bad; CK(cudaMalloc(&bad, 5 * sizeof(unsigned long long)));
  for (int mode = 0; mode < 2; ++mode) {
    CK(cudaMemset(bad, 0, 5 * sizeof(unsigned long long)));
    k_check<<<sms * 8, 256>>>(bad, 4096, mode);
    CK(cudaDeviceSynchronize());
    unsigned long long h[5]; CK(cudaMemcpy(h, bad, sizeof h, cudaMemcpyDeviceToHost));
    printf("check mode %d: %llu pairs, mismatches add %llu sub %llu mul %llu div %llu sqrt %llu\n", mode,
           (unsigned long long)sms * 8 * 256 * 4096, h[0], h[1], h[2], h[3], h[4]);
  }
  for (int bpsm : {2, 4, 8}) {
    run<8, 0, 0>("hw mul x8", sms, d, bpsm, 2048);
    run<0, 8, 2>("hw add x8", sms, d, bpsm, 2048);
    run<0, 8, 0>("sw mul x8", sms, d, bpsm, 2048);
    run<0, 8, 1>("sw add/sub x8", sms, d, bpsm, 2048);
    run<8, 4, 0>("hw mul x8 + sw mul x4", sms, d, bpsm, 2048);
    run<8, 8, 0>("hw mul x8 + sw mul x8", sms, d, bpsm, 2048);
    run<8, 16, 0>("hw mul x8 + sw mul x16", sms, d, bpsm, 1024);
    run<8, 4, 1>("hw mul x8 + sw add x4", sms, d, bpsm, 2048);
    run<8, 8, 1>("hw mul x8 + sw add x8", sms, d, bpsm, 2048);
    run<0, 4, 4>("hw div x4", sms, d, bpsm, 512);
    run<0, 4, 3>("sw div x4", sms, d, bpsm, 512);
    run<0, 4, 6>("hw sqrt x4", sms, d, bpsm, 512);
    run<0, 4, 5>("sw sqrt x4", sms, d, bpsm, 512);
    run<8, 2, 3>("hw mul x8 + sw div x2", sms, d, bpsm, 1024);
    run<8, 2, 5>("hw mul x8 + sw sqrt x2", sms, d, bpsm, 1024);
  }
  return 0;
}
