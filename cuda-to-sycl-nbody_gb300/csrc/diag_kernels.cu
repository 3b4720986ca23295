// FP64 diagnostics on the GPU: kinetic and potential energy, linear and angular
// momentum, and FP64 accelerations of selected rows.  Pair arithmetic and all
// reductions are double precision; reductions use fixed-order trees and
// per-block partials summed in block order, so results are deterministic.
#include <cuda_runtime.h>

#include <cstdint>

#include "nb_internal.hpp"
#include "nb_kernels.hpp"

namespace nbg {
namespace {

constexpr int kDiagThreads = 256;
constexpr int kDiagVals = 10;  // KE PE px py pz Lx Ly Lz M (unused)

__device__ __forceinline__ double block_sum(double v, double* sh) {
  // Fixed-order tree over the block.
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) sh[t] += sh[t + w];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// Per-particle moments over the padded range [first, last): padding has zero
// mass and velocity, so it contributes nothing.
__global__ void moments_kernel(const float* __restrict__ pos, const float4* __restrict__ vel,
                               int64_t first, int64_t last, double* __restrict__ partial) {
  __shared__ double sh[kDiagThreads];
  double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int64_t g = first + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < last;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double m = pos[pair_index(g, 3)];
    if (m == 0.0) continue;
    const double x = pos[pair_index(g, 0)], y = pos[pair_index(g, 1)], z = pos[pair_index(g, 2)];
    const float4 v = vel[g];
    const double vx = v.x, vy = v.y, vz = v.z;
    acc[0] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
    acc[2] += m * vx;
    acc[3] += m * vy;
    acc[4] += m * vz;
    acc[5] += m * (y * vz - z * vy);
    acc[6] += m * (z * vx - x * vz);
    acc[7] += m * (x * vy - y * vx);
    acc[8] += m;
  }
  for (int k = 0; k < 9; ++k) {
    const double s = block_sum(acc[k], sh);
    if (threadIdx.x == 0) partial[blockIdx.x * kDiagVals + k] = s;
  }
}

// Potential: block b handles i-tile tiles[b] = (system, tile) and all j > i of
// that system.  Writes -G * sum_i m_i sum_{j>i} m_j / sqrt(r^2 + eps) to partial.
__global__ void potential_kernel(const float* __restrict__ pos, const SystemDesc* __restrict__ sys,
                                 const int2* __restrict__ tiles, float eps2, double G,
                                 double* __restrict__ partial) {
  __shared__ double sh[kDiagThreads];
  __shared__ float4 tj[kDiagThreads];
  const int2 tl = tiles[blockIdx.x];
  const SystemDesc sd = sys[tl.x];
  const int li = tl.y * kDiagThreads + threadIdx.x;
  const bool valid = li < sd.n;
  const int64_t gi = sd.offset + (valid ? li : 0);
  const double xi = pos[pair_index(gi, 0)], yi = pos[pair_index(gi, 1)],
               zi = pos[pair_index(gi, 2)], mi = pos[pair_index(gi, 3)];
  double sum = 0.0;
  for (int j0 = tl.y * kDiagThreads; j0 < sd.n; j0 += kDiagThreads) {
    const int lj = j0 + threadIdx.x;
    if (lj < sd.n) {
      const int64_t gj = sd.offset + lj;
      tj[threadIdx.x] = make_float4(pos[pair_index(gj, 0)], pos[pair_index(gj, 1)],
                                    pos[pair_index(gj, 2)], pos[pair_index(gj, 3)]);
    } else {
      tj[threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    const int cnt = min(kDiagThreads, sd.n - j0);
    if (valid) {
      for (int k = 0; k < cnt; ++k) {
        if (j0 + k <= li) continue;
        const float4 q = tj[k];
        const double dx = q.x - xi, dy = q.y - yi, dz = q.z - zi;
        const double d2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, static_cast<double>(eps2))));
        sum = fma(static_cast<double>(q.w), rsqrt(d2), sum);
      }
    }
    __syncthreads();
  }
  const double s = block_sum(valid ? -G * mi * sum : 0.0, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Sum `count` partial records of `stride` doubles, column by column in index order.
__global__ void reduce_partials_kernel(const double* __restrict__ partial, int count, int stride,
                                       int ncols, double* __restrict__ out) {
  const int c = threadIdx.x;
  if (c >= ncols) return;
  double s = 0.0;
  for (int b = 0; b < count; ++b) s += partial[static_cast<int64_t>(b) * stride + c];
  out[c] = s;
}

// FP64 acceleration of row r: G * sum_{j != i} m_j (x_j - x_i) / (|.|^2 + eps)^(3/2).
__global__ void fp64_rows_kernel(const float* __restrict__ pos, const SystemDesc* __restrict__ sys,
                                 const int64_t* __restrict__ rows, const int32_t* __restrict__ rsys,
                                 float eps2, double G, double* __restrict__ out) {
  __shared__ double sh[kDiagThreads];
  const int64_t gi = rows[blockIdx.x];
  const SystemDesc sd = sys[rsys[blockIdx.x]];
  const double xi = pos[pair_index(gi, 0)], yi = pos[pair_index(gi, 1)],
               zi = pos[pair_index(gi, 2)];
  double ax = 0.0, ay = 0.0, az = 0.0;
  for (int j = threadIdx.x; j < sd.n; j += blockDim.x) {
    const int64_t gj = sd.offset + j;
    if (gj == gi) continue;
    const double dx = pos[pair_index(gj, 0)] - xi, dy = pos[pair_index(gj, 1)] - yi,
                 dz = pos[pair_index(gj, 2)] - zi;
    const double d2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, static_cast<double>(eps2))));
    const double inv = rsqrt(d2);
    const double s = static_cast<double>(pos[pair_index(gj, 3)]) * inv * inv * inv;
    ax = fma(dx, s, ax);
    ay = fma(dy, s, ay);
    az = fma(dz, s, az);
  }
  ax = block_sum(ax, sh);
  ay = block_sum(ay, sh);
  az = block_sum(az, sh);
  if (threadIdx.x == 0) {
    out[3 * blockIdx.x + 0] = G * ax;
    out[3 * blockIdx.x + 1] = G * ay;
    out[3 * blockIdx.x + 2] = G * az;
  }
}

}  // namespace

cudaError_t launch_diagnostics(const float* pos, const float4* vel, const SystemDesc* sys_d,
                               const SystemDesc* sys_h, int32_t first_sys, int32_t num_sys,
                               float eps2, float G, bool, double* out10, DiagScratch& scratch,
                               cudaStream_t stream) {
  // Moments.
  const int64_t first = sys_h[first_sys].offset;
  const int64_t last = sys_h[first_sys + num_sys - 1].offset + sys_h[first_sys + num_sys - 1].npad;
  const int mblocks = 1024;
  cudaError_t e = cudaSuccess;
  // Potential tiles.
  int64_t ntiles = 0;
  for (int32_t s = first_sys; s < first_sys + num_sys; ++s)
    ntiles += (sys_h[s].n + kDiagThreads - 1) / kDiagThreads;
  const int64_t need = static_cast<int64_t>(mblocks) * kDiagVals + ntiles + 2 * ntiles + 16;
  if (scratch.max_blocks < need) {
    if (scratch.partial) cudaFree(scratch.partial);
    scratch.partial = nullptr;
    scratch.max_blocks = 0;
    e = cudaMalloc(&scratch.partial, need * sizeof(double));
    if (e != cudaSuccess) return e;
    scratch.max_blocks = static_cast<int32_t>(need);
  }
  double* mom_part = scratch.partial;
  double* pot_part = scratch.partial + static_cast<int64_t>(mblocks) * kDiagVals;
  int2* tiles_d = reinterpret_cast<int2*>(pot_part + ntiles);
  int2* tiles_h = nullptr;
  e = cudaMallocHost(&tiles_h, ntiles * sizeof(int2));
  if (e != cudaSuccess) return e;
  int64_t k = 0;
  for (int32_t s = first_sys; s < first_sys + num_sys; ++s)
    for (int t = 0; t < (sys_h[s].n + kDiagThreads - 1) / kDiagThreads; ++t) tiles_h[k++] = {s, t};
  e = cudaMemcpyAsync(tiles_d, tiles_h, ntiles * sizeof(int2), cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  cudaFreeHost(tiles_h);
  if (e != cudaSuccess) return e;
  moments_kernel<<<mblocks, kDiagThreads, 0, stream>>>(pos, vel, first, last, mom_part);
  potential_kernel<<<static_cast<unsigned>(ntiles), kDiagThreads, 0, stream>>>(pos, sys_d, tiles_d,
                                                                             eps2, G, pot_part);
  reduce_partials_kernel<<<1, 32, 0, stream>>>(mom_part, mblocks, kDiagVals, 9, out10 + 1);
  reduce_partials_kernel<<<1, 32, 0, stream>>>(pot_part, static_cast<int>(ntiles), 1, 1, out10);
  return cudaGetLastError();
}

cudaError_t launch_fp64_rows(const float* pos, const SystemDesc* sys_d, const int64_t* rows_dev,
                             const int32_t* row_sys_dev, int64_t count, float eps2, float G, bool,
                             double* out3, cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  fp64_rows_kernel<<<static_cast<unsigned>(count), kDiagThreads, 0, stream>>>(
      pos, sys_d, rows_dev, row_sys_dev, eps2, G, out3);
  return cudaGetLastError();
}

}  // namespace nbg
