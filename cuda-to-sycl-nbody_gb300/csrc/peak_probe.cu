// Measured FP32 throughput of the current GPU: a loop of independent packed FP32x2
// fused multiply-adds (FFMA2, 4 flop per instruction per thread), the FP32 pipe's
// best case.  Used as a measured denominator beside the nominal FP32 peak
// (SMs x 128 lanes x 2 flop x clock) when reporting the force kernel's efficiency.
#include <cuda_runtime.h>

#include <cstdint>

#include "nb_kernels.hpp"

namespace nbg {
namespace {

constexpr int kPeakThreads = 256;
constexpr int kPeakChains = 16;  // independent FFMA2 chains per thread

// Each chain has its own multiplier registers: with one shared multiplier the loop
// measured 68 TFLOP/s against 76 with one per chain (register operand bandwidth,
// not the FMA pipe, was the limit), and 16 chains beat 8.
__global__ void __launch_bounds__(kPeakThreads) ffma2_peak_kernel(float2* __restrict__ out,
                                                                  int iters, float2 a, float2 b) {
  float2 c[kPeakChains], m[kPeakChains];
#pragma unroll
  for (int k = 0; k < kPeakChains; ++k) {
    c[k] = make_float2(1e-3f * threadIdx.x + k, 0.5f * k);
    m[k] = make_float2(a.x + 1e-6f * k, a.y - 1e-6f * k);
  }
#pragma unroll 4
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kPeakChains; ++k) c[k] = __ffma2_rn(c[k], m[k], b);  // c <- c*m + b
  }
  float2 s = c[0];
#pragma unroll
  for (int k = 1; k < kPeakChains; ++k) s = __fadd2_rn(s, c[k]);
  out[blockIdx.x * kPeakThreads + threadIdx.x] = s;  // keeps the loop alive
}

}  // namespace

cudaError_t measure_fp32_peak(int sms, float2* scratch, int blocks_per_sm, int iters,
                              int repeats, cudaStream_t stream, double* tflops, float* best_ms) {
  const int grid = sms * blocks_per_sm;
  // c <- ~0.999 c + 0.001 stays in [0, 300): no overflow, no denormals.
  const float2 a = make_float2(0.999f, 0.999f), b = make_float2(1e-3f, 1e-3f);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  // Warm-up: about 50 ms of the same work, so that the SM clock has settled before
  // the timed launches (a first call from an idle GPU read 4 % low after 10 ms).
  for (int r = 0; r < 100 && e == cudaSuccess; ++r) {
    ffma2_peak_kernel<<<grid, kPeakThreads, 0, stream>>>(scratch, iters, a, b);
    e = cudaGetLastError();
  }
  float best = 1e30f;
  for (int r = 0; r <= repeats && e == cudaSuccess; ++r) {  // r = 0 is not counted
    e = cudaEventRecord(e0, stream);
    if (e == cudaSuccess) {
      ffma2_peak_kernel<<<grid, kPeakThreads, 0, stream>>>(scratch, iters, a, b);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && r > 0 && ms < best) best = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return e;
  const double flop = 4.0 * kPeakChains * static_cast<double>(iters) * grid * kPeakThreads;
  *tflops = flop / (best * 1e-3) / 1e12;
  *best_ms = best;
  return cudaSuccess;
}

int fp32_peak_threads() { return kPeakThreads; }

}  // namespace nbg
