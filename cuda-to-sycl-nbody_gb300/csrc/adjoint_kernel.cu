// Adjoint (vector-Jacobian product) of one force + integrate iteration.
//
// Forward iteration (src/simulator.cu:193-228, masses and G made explicit):
//   v' = d v + dt G F(x),  x' = x + dt v',
//   F_i(x) = sum_{j != i} m_j r_ij f(|r_ij|^2 + eps),  r_ij = x_j - x_i,  f(s) = s^(-3/2).
// Given the cotangents (lx', lv') of (x', v'):
//   mu = lv' + dt lx',   lv = d mu,   lx = lx' + dt G J(x)^T mu,
// (mu is formed where it is read; lx and lv are written by the combining pass),
// and, with K_ij = s_ij I - 3 q_ij r_ij r_ij^T (s = f, q = s / (r^2 + eps)), which is
// symmetric in i and j,
//   (J^T mu)_i = sum_{j != i} K_ij u_ij,  u_ij = m_i mu_j - m_j mu_i
//              = sum_{j != i} s_ij (u_ij + c_ij r_ij),  c_ij = -3 (r_ij . u_ij) / (r^2 + eps).
// Per pair that is 22 FP32 lane operations and one MUFU rsqrt (equal masses: u = mu_j - mu_i
// and the common mass goes into the final scale), on the packed FP32x2 pipe, with three
// accumulators per i-particle.
//
// Work decomposition: one CTA per (i-tile, j-chunk); each writes its partial sum per
// i-particle, and a second kernel adds the chunks in order (deterministic) and applies
// lx = lx' + dt G (J^T mu).
#include <cuda_runtime.h>

#include <cstdint>

#include "nb_internal.hpp"
#include "nb_kernels.hpp"

namespace nbg {
namespace {

constexpr int kAdjThreads = 128;
constexpr int kAdjR = 4;                      // i-particles per thread
constexpr int kAdjBI = kAdjThreads * kAdjR;   // i-particles per CTA
constexpr int kAdjBJ = 256;                   // j-particles per shared tile

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// Pairs [0, npairs) of one shared tile.  kMask: zero the rsqrt of the self pair and
// of j >= jn (a padding lane at the end of the system).
template <bool kMass, bool kMask>
__device__ __forceinline__ void adj_tile(const float4 (*tile)[4], int npairs, float2 e2,
                                         const float2 (&nx)[kAdjR], const float2 (&ny)[kAdjR],
                                         const float2 (&nz)[kAdjR], const float2 (&wx)[kAdjR],
                                         const float2 (&wy)[kAdjR], const float2 (&wz)[kAdjR],
                                         const float2 (&mi)[kAdjR], float2 (&gx)[kAdjR],
                                         float2 (&gy)[kAdjR], float2 (&gz)[kAdjR], int j_base,
                                         int jn, const int (&li)[kAdjR]) {
  const float2 m3c = f2(-3.f, -3.f);
#pragma unroll 2
  for (int p = 0; p < npairs; ++p) {
    const float4 P0 = tile[p][0], P1 = tile[p][1], M0 = tile[p][2], M1 = tile[p][3];
#pragma unroll
    for (int r = 0; r < kAdjR; ++r) {
      const float2 dx = __fadd2_rn(f2(P0.x, P0.y), nx[r]);
      const float2 dy = __fadd2_rn(f2(P0.z, P0.w), ny[r]);
      const float2 dz = __fadd2_rn(f2(P1.x, P1.y), nz[r]);
      float2 ux, uy, uz;
      if (kMass) {
        const float2 mj = f2(P1.z, P1.w);
        ux = __ffma2_rn(mj, wx[r], __fmul2_rn(mi[r], f2(M0.x, M0.y)));
        uy = __ffma2_rn(mj, wy[r], __fmul2_rn(mi[r], f2(M0.z, M0.w)));
        uz = __ffma2_rn(mj, wz[r], __fmul2_rn(mi[r], f2(M1.x, M1.y)));
      } else {
        ux = __fadd2_rn(f2(M0.x, M0.y), wx[r]);
        uy = __fadd2_rn(f2(M0.z, M0.w), wy[r]);
        uz = __fadd2_rn(f2(M1.x, M1.y), wz[r]);
      }
      float2 d2 = __ffma2_rn(dx, dx, e2);
      d2 = __ffma2_rn(dy, dy, d2);
      d2 = __ffma2_rn(dz, dz, d2);
      float2 inv = f2(rsqrtf(d2.x), rsqrtf(d2.y));
      if (kMask) {
        const int j = j_base + 2 * p;
        if (j == li[r] || j >= jn) inv.x = 0.f;
        if (j + 1 == li[r] || j + 1 >= jn) inv.y = 0.f;
      }
      const float2 inv2 = __fmul2_rn(inv, inv);
      const float2 s = __fmul2_rn(inv2, inv);
      const float2 m3 = __fmul2_rn(inv2, m3c);
      float2 rw = __fmul2_rn(dx, ux);
      rw = __ffma2_rn(dy, uy, rw);
      rw = __ffma2_rn(dz, uz, rw);
      const float2 c = __fmul2_rn(rw, m3);
      gx[r] = __ffma2_rn(s, __ffma2_rn(c, dx, ux), gx[r]);
      gy[r] = __ffma2_rn(s, __ffma2_rn(c, dy, uy), gy[r]);
      gz[r] = __ffma2_rn(s, __ffma2_rn(c, dz, uz), gz[r]);
    }
  }
}

template <bool kMass>
__global__ void __launch_bounds__(kAdjThreads) adjoint_partial_kernel(const AdjointArgs a) {
  // Tile of j-pairs: { x0 x1 y0 y1 } { z0 z1 m0 m1 } { mx0 mx1 my0 my1 } { mz0 mz1 0 0 }
  __shared__ __align__(16) float4 tile[kAdjBJ / 2][4];
  const SystemDesc sd = a.sys[a.tile_sys[blockIdx.x]];
  const int ibase = a.tile_idx[blockIdx.x] * kAdjBI;
  const int split = blockIdx.y;
  const int chunk = ((sd.n + a.num_splits - 1) / a.num_splits + 1) & ~1;
  const int j_lo = split * chunk;
  const int j_hi = min(sd.n, j_lo + chunk);
  const int tid = threadIdx.x;

  float2 nx[kAdjR], ny[kAdjR], nz[kAdjR], wx[kAdjR], wy[kAdjR], wz[kAdjR], mi[kAdjR];
  float2 gx[kAdjR], gy[kAdjR], gz[kAdjR];
  int li[kAdjR];
#pragma unroll
  for (int r = 0; r < kAdjR; ++r) {
    li[r] = ibase + r * kAdjThreads + tid;
    const int64_t g = sd.offset + (li[r] < sd.n ? li[r] : sd.n - 1);
    const float x = a.pos[pair_index(g, 0)], y = a.pos[pair_index(g, 1)],
                z = a.pos[pair_index(g, 2)], m = a.pos[pair_index(g, 3)];
    const float4 lx = a.lam_x[g], lv = a.lam_v[g];  // mu = lv' + dt lx'
    const float4 mu = make_float4(fmaf(a.dt, lx.x, lv.x), fmaf(a.dt, lx.y, lv.y),
                                  fmaf(a.dt, lx.z, lv.z), 0.f);
    nx[r] = f2(-x, -x);
    ny[r] = f2(-y, -y);
    nz[r] = f2(-z, -z);
    wx[r] = f2(-mu.x, -mu.x);
    wy[r] = f2(-mu.y, -mu.y);
    wz[r] = f2(-mu.z, -mu.z);
    mi[r] = f2(m, m);
    gx[r] = gy[r] = gz[r] = f2(0.f, 0.f);
  }
  const float2 e2 = f2(a.eps2, a.eps2);

  for (int j0 = j_lo; j0 < j_hi; j0 += kAdjBJ) {
    const int cnt = min(kAdjBJ, j_hi - j0);
    __syncthreads();
    for (int p = tid; p < kAdjBJ / 2; p += kAdjThreads) {
      float v[2][7];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int lj = j0 + 2 * p + h;
        if (2 * p + h < cnt) {
          const int64_t gj = sd.offset + lj;
          const float4 lx = a.lam_x[gj], lv = a.lam_v[gj];
          const float4 mu = make_float4(fmaf(a.dt, lx.x, lv.x), fmaf(a.dt, lx.y, lv.y),
                                        fmaf(a.dt, lx.z, lv.z), 0.f);
          v[h][0] = a.pos[pair_index(gj, 0)];
          v[h][1] = a.pos[pair_index(gj, 1)];
          v[h][2] = a.pos[pair_index(gj, 2)];
          v[h][3] = a.pos[pair_index(gj, 3)];
          v[h][4] = mu.x;
          v[h][5] = mu.y;
          v[h][6] = mu.z;
        } else {
          // past the chunk: at the origin with zero mass and cotangent (masked below)
          v[h][0] = v[h][1] = v[h][2] = v[h][3] = v[h][4] = v[h][5] = v[h][6] = 0.f;
        }
      }
      tile[p][0] = make_float4(v[0][0], v[1][0], v[0][1], v[1][1]);
      tile[p][1] = make_float4(v[0][2], v[1][2], v[0][3], v[1][3]);
      tile[p][2] = make_float4(v[0][4], v[1][4], v[0][5], v[1][5]);
      tile[p][3] = make_float4(v[0][6], v[1][6], 0.f, 0.f);
    }
    __syncthreads();
    const int npairs = (cnt + 1) / 2;
    const bool diag = a.mask_self && (j0 < ibase + kAdjBI) && (ibase < j0 + cnt);
    if (diag || (cnt & 1)) {
      adj_tile<kMass, true>(tile, npairs, e2, nx, ny, nz, wx, wy, wz, mi, gx, gy, gz, j0,
                            j0 + cnt, li);
    } else {
      adj_tile<kMass, false>(tile, npairs, e2, nx, ny, nz, wx, wy, wz, mi, gx, gy, gz, j0,
                             j0 + cnt, li);
    }
  }

  float4* part = a.partial + static_cast<int64_t>(split) * a.n_pad;
#pragma unroll
  for (int r = 0; r < kAdjR; ++r) {
    if (li[r] >= sd.n) continue;
    part[sd.offset + li[r]] =
        make_float4(gx[r].x + gx[r].y, gy[r].x + gy[r].y, gz[r].x + gz[r].y, 0.f);
  }
}

// lx = lx' + dt * gscale * sum over chunks (in chunk order) and lv = damping * mu,
// real particles only.  One thread per particle, kCombineThreads particles of an
// i-tile per CTA (blockIdx.y picks them); the chunk loop is unrolled so that several
// of its loads are in flight (the additions keep their order).
constexpr int kCombineThreads = 128;
static_assert(kAdjBI % kCombineThreads == 0, "whole i-tiles");

__global__ void __launch_bounds__(kCombineThreads) adjoint_combine_kernel(const AdjointArgs a) {
  const SystemDesc sd = a.sys[a.tile_sys[blockIdx.x]];
  const int ibase = a.tile_idx[blockIdx.x] * kAdjBI;
  const float c = a.dt * sd.gscale;
  const int li = ibase + blockIdx.y * kCombineThreads + threadIdx.x;
  if (li >= sd.n) return;
  const int64_t g = sd.offset + li;
  float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll 8
  for (int s = 0; s < a.num_splits; ++s) {
    const float4 p = a.partial[static_cast<int64_t>(s) * a.n_pad + g];
    sx += p.x;
    sy += p.y;
    sz += p.z;
  }
  const float4 l = a.lam_x[g], v = a.lam_v[g];
  a.lam_x_out[g] = make_float4(fmaf(c, sx, l.x), fmaf(c, sy, l.y), fmaf(c, sz, l.z), 0.f);
  a.lam_v_out[g] = make_float4(a.damping * fmaf(a.dt, l.x, v.x), a.damping * fmaf(a.dt, l.y, v.y),
                               a.damping * fmaf(a.dt, l.z, v.z), 0.f);
}

__global__ void unpack_vec3_kernel(const float* __restrict__ in, int64_t n,
                                   const int64_t* __restrict__ map, float4* __restrict__ out) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t g = map ? map[k] : k;
    out[g] = make_float4(in[3 * k], in[3 * k + 1], in[3 * k + 2], 0.f);
  }
}

__global__ void pack_vec3_kernel(const float4* __restrict__ in, int64_t n,
                                 const int64_t* __restrict__ map, float* __restrict__ out) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t g = map ? map[k] : k;
    const float4 v = in[g];
    out[3 * k] = v.x;
    out[3 * k + 1] = v.y;
    out[3 * k + 2] = v.z;
  }
}

int grid_for(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return static_cast<int>(b < 1 ? 1 : (b > 1 << 20 ? 1 << 20 : b));
}

}  // namespace

int adjoint_tile() { return kAdjBI; }

cudaError_t adjoint_blocks_per_sm(bool per_pair_mass, int* blocks) {
  return per_pair_mass
             ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, adjoint_partial_kernel<true>,
                                                             kAdjThreads, 0)
             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, adjoint_partial_kernel<false>,
                                                             kAdjThreads, 0);
}

cudaError_t launch_adjoint(const AdjointArgs& a, int32_t num_tiles, bool per_pair_mass,
                           cudaStream_t stream) {
  const dim3 grid(num_tiles, a.num_splits);
  if (per_pair_mass)
    adjoint_partial_kernel<true><<<grid, kAdjThreads, 0, stream>>>(a);
  else
    adjoint_partial_kernel<false><<<grid, kAdjThreads, 0, stream>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  adjoint_combine_kernel<<<dim3(num_tiles, kAdjBI / kCombineThreads), kCombineThreads, 0,
                           stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_unpack_vec3(const float* in, int64_t n, const int64_t* map, float4* out,
                               cudaStream_t stream) {
  unpack_vec3_kernel<<<grid_for(n), 256, 0, stream>>>(in, n, map, out);
  return cudaGetLastError();
}

cudaError_t launch_pack_vec3(const float4* in, int64_t n, const int64_t* map, float* out,
                             cudaStream_t stream) {
  pack_vec3_kernel<<<grid_for(n), 256, 0, stream>>>(in, n, map, out);
  return cudaGetLastError();
}

}  // namespace nbg
