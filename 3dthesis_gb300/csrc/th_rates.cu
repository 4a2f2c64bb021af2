// Issue-rate probe of the device: MUFU.EX2 and FP32 FMA results per SM per clock, measured
// with a throughput-bound kernel, for the roofline the point x node kernels are measured
// against (each FP32 pair costs about ten FP32 lane-operations and one ex2).
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "th_ctx.h"

namespace {

constexpr int kChains = 8;        // independent dependency chains per thread
constexpr int kIters = 4096;      // loop trips per thread (kChains operations each)

// Every thread runs kChains independent chains of kIters dependent ex2.approx (or FMA)
// operations; thread 0 of each block records the SM clocks its block took.  The values
// stay finite (ex2 of a negative argument stays in (0, 1]); the sum keeps them live.
template <bool EX2>
__global__ void __launch_bounds__(256) k_rate(float seed, float* sink, unsigned long long* clocks) {
  float v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) v[c] = seed * (float)(threadIdx.x + c + 1) * 1e-6f;
  __syncthreads();
  const long long c0 = clock64();
  for (int i = 0; i < kIters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
      if (EX2) asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(v[c]) : "f"(-v[c]));
      else v[c] = fmaf(v[c], 0.999f, 1e-7f);
    }
  }
  __syncthreads();
  const long long c1 = clock64();
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += v[c];
  if (s == 12345.f) sink[blockIdx.x] = s;          // practically never; keeps the chains
  if (threadIdx.x == 0) clocks[blockIdx.x] = (unsigned long long)(c1 - c0);
}

// Operations per SM per clock of one probe: blocks_per_sm resident 256-thread blocks on
// every SM (one wave), each block's clocks measured on its own SM.
template <bool EX2>
cudaError_t rate(int sms, int blocks_per_sm, double* out) {
  const int blocks = sms * blocks_per_sm;
  float* sink = nullptr;
  unsigned long long* clk = nullptr;
  cudaError_t e = cudaMalloc(&sink, blocks * sizeof(float));
  if (e != cudaSuccess) return e;
  if ((e = cudaMalloc(&clk, blocks * sizeof(unsigned long long))) != cudaSuccess) { cudaFree(sink); return e; }
  k_rate<EX2><<<blocks, 256>>>(0.5f, sink, clk);          // warm-up
  k_rate<EX2><<<blocks, 256>>>(0.5f, sink, clk);
  e = cudaDeviceSynchronize();
  std::vector<unsigned long long> h(blocks);
  if (e == cudaSuccess) e = cudaMemcpy(h.data(), clk, blocks * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(sink);
  cudaFree(clk);
  if (e != cudaSuccess) return e;
  unsigned long long mx = 0;
  for (unsigned long long c : h) mx = c > mx ? c : mx;   // the slowest block bounds the SM
  const double ops_per_sm = (double)blocks_per_sm * 256.0 * kChains * kIters;
  *out = mx ? ops_per_sm / (double)mx : 0.0;
  return cudaSuccess;
}

}  // namespace

extern "C" th_status th_device_rates(double* out) {
  if (!out) return th_fail(nullptr, TH_ERR_INVALID, "null argument");
  int dev = 0, sms = 0, clk_khz = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, dev);
  if (e != cudaSuccess) return th_cuda_check(nullptr, e, "device attributes");
  double ex2 = 0.0, fma = 0.0;
  // four resident blocks per SM: 32 warps, enough independent chains to cover the latencies
  if ((e = rate<true>(sms, 4, &ex2)) != cudaSuccess) return th_cuda_check(nullptr, e, "ex2 probe");
  if ((e = rate<false>(sms, 4, &fma)) != cudaSuccess) return th_cuda_check(nullptr, e, "fma probe");
  out[0] = sms;
  out[1] = clk_khz * 1e-3;
  out[2] = ex2;
  out[3] = fma;
  return TH_OK;
}
