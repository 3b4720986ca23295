// Small kernels around the force step: the reference's PREDICATED variant, and
// moving state between the caller's structure-of-arrays and the device layout.
#include <cuda_runtime.h>

#include <cstdint>

#include "nb_device.cuh"
#include "nb_internal.hpp"
#include "nb_kernels.hpp"

namespace nbg {
namespace {

constexpr int kBlock = 256;

inline int blocks_for(int64_t n) {
  const int64_t b = (n + kBlock - 1) / kBlock;
  return static_cast<int>(b < 1 ? 1 : (b > 65535 * 16 ? 65535 * 16 : b));
}

// particle_interaction<PREDICATED> as shipped (simulator.cu:186-229): the pair
// term is multiplied by (j == i) (:209), so only the self term survives, and it
// is 0 * rsqrt(eps^3) -- zero, or NaN when eps^3 flushes to zero; any other pair
// whose term is not finite also turns the sum into NaN.  One thread per i, the
// reference's loop and operation order (dot(r,r) as nvcc contracts it, :201).
__global__ void predicated_kernel(const ForceArgs a, const SystemDesc sd) {
  const int li = blockIdx.x * blockDim.x + threadIdx.x;
  if (li >= sd.n) return;
  const int64_t gi = sd.offset + li;
  const float xi = a.pos[pair_index(gi, 0)];
  const float yi = a.pos[pair_index(gi, 1)];
  const float zi = a.pos[pair_index(gi, 2)];
  float fx = 0.f, fy = 0.f, fz = 0.f;
  for (int j = 0; j < sd.n; ++j) {
    const int64_t gj = sd.offset + j;
    const float rx = a.pos[pair_index(gj, 0)] - xi;
    const float ry = a.pos[pair_index(gj, 1)] - yi;
    const float rz = a.pos[pair_index(gj, 2)] - zi;
    const float d2 = fmaf(rz, rz, fmaf(rx, rx, ry * ry)) + a.eps2;
    float inv = rsqrtf(d2 * d2 * d2);
    if (!sd.equal_mass) inv *= a.pos[pair_index(gj, 3)];
    const float mask = (j == li) ? 1.f : 0.f;
    fx = fmaf(rx * inv, mask, fx);
    fy = fmaf(ry * inv, mask, fy);
    fz = fmaf(rz * inv, mask, fz);
  }
  finish_particle(a, sd, gi, fx, fy, fz, xi, yi, zi);
}

__global__ void unpack_kernel(const float* __restrict__ soa, int64_t n,
                              const int64_t* __restrict__ map, float* __restrict__ pos,
                              float4* __restrict__ vel, int with_mass) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t g = map ? map[k] : k;
    pos[pair_index(g, 0)] = soa[k];
    pos[pair_index(g, 1)] = soa[n + k];
    pos[pair_index(g, 2)] = soa[2 * n + k];
    if (with_mass) pos[pair_index(g, 3)] = soa[6 * n + k];
    vel[g] = make_float4(soa[3 * n + k], soa[4 * n + k], soa[5 * n + k], 0.f);
  }
}

__global__ void pack_kernel(const float* __restrict__ pos, const float4* __restrict__ vel,
                            int64_t n, const int64_t* __restrict__ map,
                            float* __restrict__ soa) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t g = map ? map[k] : k;
    soa[k] = pos[pair_index(g, 0)];
    soa[n + k] = pos[pair_index(g, 1)];
    soa[2 * n + k] = pos[pair_index(g, 2)];
    const float4 v = vel[g];
    soa[3 * n + k] = v.x;
    soa[4 * n + k] = v.y;
    soa[5 * n + k] = v.z;
  }
}

__global__ void pack_accel_kernel(const float4* __restrict__ acc, int64_t n,
                                  const int64_t* __restrict__ map, float* __restrict__ soa) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t g = map ? map[k] : k;
    const float4 a = acc[g];
    soa[k] = a.x;
    soa[n + k] = a.y;
    soa[2 * n + k] = a.z;
  }
}

__global__ void export_kernel(const float* __restrict__ pos, const float4* __restrict__ vel,
                              int64_t n, const int64_t* __restrict__ map,
                              float4* __restrict__ pos_out, float4* __restrict__ vel_out) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t g = map ? map[k] : k;
    pos_out[k] = make_float4(pos[pair_index(g, 0)], pos[pair_index(g, 1)], pos[pair_index(g, 2)],
                             pos[pair_index(g, 3)]);
    if (vel_out) vel_out[k] = vel[g];
  }
}

__global__ void fill_padding_kernel(float* __restrict__ pos, float4* __restrict__ vel,
                                    int64_t n) {
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < n;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    pos[pair_index(g, 0)] = kFarAway;
    pos[pair_index(g, 1)] = kFarAway;
    pos[pair_index(g, 2)] = kFarAway;
    pos[pair_index(g, 3)] = 0.f;
    vel[g] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

}  // namespace

cudaError_t launch_predicated(const ForceArgs& a, const SystemDesc& sd, int32_t,
                              cudaStream_t stream) {
  const int grid = (sd.n + 127) / 128;
  predicated_kernel<<<grid, 128, 0, stream>>>(a, sd);
  return cudaGetLastError();
}

cudaError_t launch_unpack_state(const float* soa, int64_t n, const int64_t* map, float* pos,
                                float4* vel, bool with_mass, cudaStream_t stream) {
  unpack_kernel<<<blocks_for(n), kBlock, 0, stream>>>(soa, n, map, pos, vel, with_mass ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_pack_state(const float* pos, const float4* vel, int64_t n, const int64_t* map,
                              float* soa, cudaStream_t stream) {
  pack_kernel<<<blocks_for(n), kBlock, 0, stream>>>(pos, vel, n, map, soa);
  return cudaGetLastError();
}

cudaError_t launch_pack_accel(const float4* acc, int64_t n, const int64_t* map, float* soa,
                              cudaStream_t stream) {
  pack_accel_kernel<<<blocks_for(n), kBlock, 0, stream>>>(acc, n, map, soa);
  return cudaGetLastError();
}

cudaError_t launch_export(const float* pos, const float4* vel, int64_t n, const int64_t* map,
                          float4* pos_out, float4* vel_out, cudaStream_t stream) {
  export_kernel<<<blocks_for(n), kBlock, 0, stream>>>(pos, vel, n, map, pos_out, vel_out);
  return cudaGetLastError();
}

cudaError_t launch_fill_padding(float* pos, float4* vel, int64_t n_pad_total,
                                cudaStream_t stream) {
  fill_padding_kernel<<<blocks_for(n_pad_total), kBlock, 0, stream>>>(pos, vel, n_pad_total);
  return cudaGetLastError();
}

}  // namespace nbg
