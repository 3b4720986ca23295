// Initial conditions generated on the device, straight into the simulation's
// layout (the reference can only initialise on the host and copy,
// src/simulator.cu:77-103).  The draws are the host generators' counter-based
// SplitMix64 draws (csrc/initial_conditions.cpp), so each particle gets the same
// random numbers as on the host; the transcendental functions are CUDA's double
// versions, so values can differ from the host's by an ulp before rounding to float.
// System k of a simulation uses seed + k.
#include <cuda_runtime.h>

#include <cstdint>

#include "nb_internal.hpp"
#include "nb_kernels.hpp"

namespace nbg {
namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double unit(uint64_t seed, uint64_t particle, uint64_t k) {
  const uint64_t d =
      mix64(seed * 0x9E3779B97F4A7C15ull + mix64(particle * 0xD1B54A32D192ED03ull + k + 1));
  return (static_cast<double>(d >> 11) + 0.5) * 0x1.0p-53;
}

__device__ __forceinline__ void normal2(uint64_t seed, uint64_t particle, uint64_t k, double& a,
                                        double& b) {
  const double u = unit(seed, particle, k), v = unit(seed, particle, k + 1);
  const double rad = sqrt(-2.0 * log(u));
  a = rad * cos(kTwoPi * v);
  b = rad * sin(kTwoPi * v);
}

// One thin-disk particle (nb_ic_thin_disk): float outputs.
__device__ void disk_particle(uint64_t seed, uint64_t n, double eps, uint64_t i, float* o) {
  const double m = 1.0 / static_cast<double>(n);
  const double nm = static_cast<double>(n) * m;
  const double r = sqrt(unit(seed, i, 0));
  const double th = kTwoPi * unit(seed, i, 1);
  double gz, g0, g1, g2;
  normal2(seed, i, 2, gz, g0);
  normal2(seed, i, 4, g1, g2);
  const double r2 = r * r;
  const double vt = r * sqrt(nm * r2 / pow(r2 + eps, 1.5));
  const double c = cos(th), s = sin(th);
  o[0] = static_cast<float>(r * c);
  o[1] = static_cast<float>(r * s);
  o[2] = static_cast<float>(0.01 * gz);
  o[3] = static_cast<float>(-vt * s + 0.01 * g0);
  o[4] = static_cast<float>(vt * c + 0.01 * g1);
  o[5] = static_cast<float>(0.01 * g2);
}

__device__ __forceinline__ void store(float* pos, float4* vel, int64_t g, const float* o,
                                      float m) {
  pos[pair_index(g, 0)] = o[0];
  pos[pair_index(g, 1)] = o[1];
  pos[pair_index(g, 2)] = o[2];
  pos[pair_index(g, 3)] = m;
  vel[g] = make_float4(o[3], o[4], o[5], 0.f);
}

// Thin disks and two-disk collisions: one thread per particle, grid-stride.
__global__ void gen_disks(float* pos, float4* vel, const SystemDesc* sys, const int64_t* first,
                          int32_t nsys, int64_t total, uint64_t seed, double eps, int two) {
  for (int64_t u = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; u < total;
       u += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int32_t lo = 0, hi = nsys - 1;  // system of user index u
    while (lo < hi) {
      const int32_t mid = (lo + hi + 1) / 2;
      if (first[mid] <= u) lo = mid; else hi = mid - 1;
    }
    const SystemDesc sd = sys[lo];
    const uint64_t sk = seed + static_cast<uint64_t>(lo);
    const int64_t i = u - first[lo];
    float o[6];
    float m;
    if (!two) {
      disk_particle(sk, sd.n, eps, i, o);
      m = static_cast<float>(1.0 / static_cast<double>(sd.n));
    } else {
      // nb_ic_two_disks: halves of n/2; the second seeded +0x5bd1e995, tilted 30 deg
      // about x; centres -+2 in x with bulk velocities +-0.3.
      const uint64_t h = sd.n / 2;
      const bool second = static_cast<uint64_t>(i) >= h;
      disk_particle(second ? sk + 0x5bd1e995ull : sk, h, eps, second ? i - h : i, o);
      m = static_cast<float>(1.0 / static_cast<double>(h));
      if (!second) {
        o[0] = static_cast<float>(static_cast<double>(o[0]) - 2.0);
        o[3] = static_cast<float>(static_cast<double>(o[3]) + 0.3);
      } else {
        const double ca = cos(kTwoPi / 12.0), sa = sin(kTwoPi / 12.0);
        const double yy = o[1], zz = o[2], vyy = o[4], vzz = o[5];
        o[1] = static_cast<float>(ca * yy - sa * zz);
        o[2] = static_cast<float>(sa * yy + ca * zz);
        o[4] = static_cast<float>(ca * vyy - sa * vzz);
        o[5] = static_cast<float>(sa * vyy + ca * vzz);
        o[0] = static_cast<float>(static_cast<double>(o[0]) + 2.0);
        o[3] = static_cast<float>(static_cast<double>(o[3]) - 0.3);
      }
    }
    store(pos, vel, sd.offset + i, o, m);
  }
}

// Plummer (nb_ic_plummer), pass 1: per-particle position and velocity in FP64.
__global__ void gen_plummer_raw(double* raw, const SystemDesc* sys, const int64_t* first,
                                int32_t nsys, int64_t total, uint64_t seed) {
  for (int64_t u = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; u < total;
       u += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int32_t lo = 0, hi = nsys - 1;
    while (lo < hi) {
      const int32_t mid = (lo + hi + 1) / 2;
      if (first[mid] <= u) lo = mid; else hi = mid - 1;
    }
    const uint64_t sk = seed + static_cast<uint64_t>(lo);
    const uint64_t i = static_cast<uint64_t>(u - first[lo]);
    uint64_t k = 0;
    double X;
    do {
      X = unit(sk, i, k++);
    } while (X > 0.999 && k < 64);
    const double r = 1.0 / sqrt(pow(X, -2.0 / 3.0) - 1.0);
    const double ct = 1.0 - 2.0 * unit(sk, i, 64);
    const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    const double ph = kTwoPi * unit(sk, i, 65);
    double* o = raw + 6 * u;
    o[0] = r * st * cos(ph);
    o[1] = r * st * sin(ph);
    o[2] = r * ct;
    double q = 0.0;
    uint64_t kk = 128;
    for (int it = 0; it < 20000; ++it) {
      q = unit(sk, i, kk);
      const double g = 0.1 * unit(sk, i, kk + 1);
      kk += 2;
      if (g < q * q * pow(1.0 - q * q, 3.5)) break;
    }
    const double v = q * sqrt(2.0) * pow(1.0 + r * r, -0.25);
    const double cv = 1.0 - 2.0 * unit(sk, i, 66);
    const double sv = sqrt(fmax(0.0, 1.0 - cv * cv));
    const double pv = kTwoPi * unit(sk, i, 67);
    o[3] = v * sv * cos(pv);
    o[4] = v * sv * sin(pv);
    o[5] = v * cv;
  }
}

// Pass 2: per-system mean (one block per system, fixed-order tree), pass 3: subtract.
__global__ void plummer_mean(const double* raw, const int64_t* first, const SystemDesc* sys,
                             double* mean) {
  __shared__ double sh[256][6];
  const int32_t s = blockIdx.x;
  const int64_t f = first[s];
  const int32_t n = sys[s].n;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int32_t i = threadIdx.x; i < n; i += blockDim.x)
    for (int c = 0; c < 6; ++c) acc[c] += raw[6 * (f + i) + c];
  for (int c = 0; c < 6; ++c) sh[threadIdx.x][c] = acc[c];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int c = 0; c < 6; ++c) sh[threadIdx.x][c] += sh[threadIdx.x + w][c];
    __syncthreads();
  }
  if (threadIdx.x < 6) mean[6 * s + threadIdx.x] = sh[0][threadIdx.x] / static_cast<double>(n);
}

__global__ void plummer_store(const double* raw, const double* mean, float* pos, float4* vel,
                              const SystemDesc* sys, const int64_t* first, int32_t nsys,
                              int64_t total) {
  for (int64_t u = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; u < total;
       u += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int32_t lo = 0, hi = nsys - 1;
    while (lo < hi) {
      const int32_t mid = (lo + hi + 1) / 2;
      if (first[mid] <= u) lo = mid; else hi = mid - 1;
    }
    float o[6];
    for (int c = 0; c < 6; ++c) o[c] = static_cast<float>(raw[6 * u + c] - mean[6 * lo + c]);
    store(pos, vel, sys[lo].offset + (u - first[lo]), o,
          static_cast<float>(1.0 / static_cast<double>(sys[lo].n)));
  }
}

int grid_for(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return static_cast<int>(b < 1 ? 1 : (b > 65536 ? 65536 : b));
}

}  // namespace

cudaError_t launch_generate(int kind, float* pos, float4* vel, const SystemDesc* sys_d,
                            const int64_t* first_d, int32_t nsys, int64_t total, uint64_t seed,
                            double eps, double* raw, double* mean, cudaStream_t stream) {
  if (kind == 1 || kind == 3) {
    gen_disks<<<grid_for(total), 256, 0, stream>>>(pos, vel, sys_d, first_d, nsys, total, seed,
                                                    eps, kind == 3);
    return cudaGetLastError();
  }
  gen_plummer_raw<<<grid_for(total), 256, 0, stream>>>(raw, sys_d, first_d, nsys, total, seed);
  plummer_mean<<<nsys, 256, 0, stream>>>(raw, first_d, sys_d, mean);
  plummer_store<<<grid_for(total), 256, 0, stream>>>(raw, mean, pos, vel, sys_d, first_d, nsys,
                                                     total);
  return cudaGetLastError();
}

}  // namespace nbg
