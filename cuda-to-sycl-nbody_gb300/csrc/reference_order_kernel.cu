// Reference-order force + integrate step (nb_accumulator NB_ACC_REFERENCE_ORDER).
//
// particle_interaction<BRANCH> (src/simulator.cu:186-229) gives each particle one
// FP32 running sum over j = 0 .. n-1 in index order, skipping j == i (:205-206),
// with the pair term r * rsqrt(d2^3), d2 = dot(r, r) + distEps (:199-202), and then
// v = v * damping + (F * dt) * G, x' = x + v * dt (:213-228), built with
// -use_fast_math (flush-to-zero, contracted multiply-adds, approximate rsqrt).
// This kernel performs the same IEEE operations in the same order for every
// particle, so on the same GPU its results are bit-identical to the reference
// kernel's.  The fast kernel (force_kernel.cuh) sums in another order instead.
//
// GB300 layout: the two lanes of each packed FP32x2 register pair hold two
// different i-particles (each lane its own running sum, so the order per particle
// is untouched), and j-tiles are staged in shared memory already duplicated as
// (x, x, y, y) (z, z, m, m), so one broadcast 16-byte load feeds both lanes.  A
// CTA owns whole i-tiles: an i-particle's sum is never split.  Only the n real
// particles of a system are summed (no padding terms), as in the reference.
// Each CTA prefetches the next j-tile into registers while it computes the
// current one (double-buffered shared memory, no device-side waits).
#include <cuda_runtime.h>

#include <cstdint>

#include "nb_device.cuh"
#include "nb_internal.hpp"
#include "nb_kernels.hpp"

namespace nbg {
namespace {

// Shapes: kRoThreads threads per CTA, kRoPairs i-pairs per thread, so i-tiles of
// kRoThreads * 2 * kRoPairs particles.  A particle's sum cannot be split, so small
// systems need small i-tiles to give every SM work (see the shape table below).
constexpr int kRoBJ = 256;       // j-particles per shared-memory tile
constexpr int kRoRecs = kRoBJ / 2;                // 32-byte pair records per j-tile
constexpr int kRoUnroll = 4;     // j steps per unrolled block

// One j step against all of the thread's i-pairs.  kDiag: the tile overlaps the
// i-tile, so the term of j == i is left out of that lane's sum (the reference's
// `if (i == id) continue;`), by keeping the old value rather than adding zero.
template <int kRoPairs, bool kDiag>
__device__ __forceinline__ void ro_step(const float4 xy, const float4 zm, float2 e2,
                                        const float2 (&nx)[kRoPairs],
                                        const float2 (&ny)[kRoPairs],
                                        const float2 (&nz)[kRoPairs], float2 (&ax)[kRoPairs],
                                        float2 (&ay)[kRoPairs], float2 (&az)[kRoPairs], int j,
                                        const int (&li)[kRoPairs]) {
  const float2 xx = make_float2(xy.x, xy.y);
  const float2 yy = make_float2(xy.z, xy.w);
  const float2 zz = make_float2(zm.x, zm.y);
#pragma unroll
  for (int k = 0; k < kRoPairs; ++k) {
    // r = other_pos - pos (:200)
    const float2 rx = __fadd2_rn(xx, nx[k]);
    const float2 ry = __fadd2_rn(yy, ny[k]);
    const float2 rz = __fadd2_rn(zz, nz[k]);
    // dot(r, r) + distEps (:201) as nvcc contracts the reference's dot():
    // fma(r.z, r.z, fma(r.x, r.x, r.y * r.y)) + distEps.  Of the two ways to fuse
    // the first sum, only this one reproduces the reference kernel's outputs bit for
    // bit (the golden fixtures of its own runs, in the tests).
    float2 d2 = __fmul2_rn(ry, ry);
    d2 = __ffma2_rn(rx, rx, d2);
    d2 = __ffma2_rn(rz, rz, d2);
    d2 = __fadd2_rn(d2, e2);
    // rsqrt(d2 * d2 * d2) (:202)
    float2 t = __fmul2_rn(d2, d2);
    t = __fmul2_rn(t, d2);
    const float2 inv = make_float2(rsqrtf(t.x), rsqrtf(t.y));
    // force += r * inv (:206), contracted
    float2 fx = __ffma2_rn(rx, inv, ax[k]);
    float2 fy = __ffma2_rn(ry, inv, ay[k]);
    float2 fz = __ffma2_rn(rz, inv, az[k]);
    if (kDiag) {
      if (j == li[k]) {
        fx.x = ax[k].x;
        fy.x = ay[k].x;
        fz.x = az[k].x;
      }
      if (j == li[k] + 1) {
        fx.y = ax[k].y;
        fy.y = ay[k].y;
        fz.y = az[k].y;
      }
    }
    ax[k] = fx;
    ay[k] = fy;
    az[k] = fz;
  }
}

// Steps over j = j0 .. j0 + count - 1 of the staged tile, in order.
template <int kRoPairs, bool kDiag>
__device__ __forceinline__ void ro_tile(const float4* __restrict__ tile, int count, int j0,
                                        float2 e2, const float2 (&nx)[kRoPairs],
                                        const float2 (&ny)[kRoPairs],
                                        const float2 (&nz)[kRoPairs], float2 (&ax)[kRoPairs],
                                        float2 (&ay)[kRoPairs], float2 (&az)[kRoPairs],
                                        const int (&li)[kRoPairs]) {
  int jj = 0;
#pragma unroll 1
  for (; jj + kRoUnroll <= count; jj += kRoUnroll) {
#pragma unroll
    for (int u = 0; u < kRoUnroll; ++u)
      ro_step<kRoPairs, kDiag>(tile[2 * (jj + u)], tile[2 * (jj + u) + 1], e2, nx, ny, nz, ax, ay, az,
                     j0 + jj + u, li);
  }
#pragma unroll 1
  for (; jj < count; ++jj)
    ro_step<kRoPairs, kDiag>(tile[2 * jj], tile[2 * jj + 1], e2, nx, ny, nz, ax, ay, az, j0 + jj, li);
}

struct RoTile {
  int32_t sys;
  int32_t itile;
};

template <int kRoThreads, int kRoPairs>
__global__ void __launch_bounds__(kRoThreads) reference_order_kernel(const ForceArgs a,
                                                                      const RoTile* tiles,
                                                                      int32_t num_tiles) {
  constexpr int kRoBI = kRoThreads * 2 * kRoPairs;  // i-particles per tile
  constexpr int kRoRecsPerThread = (kRoRecs + kRoThreads - 1) / kRoThreads;
  static_assert(kRoBI % kPadQuantum == 0, "i-tiles must hold whole padding quanta");
  // [buffer][j][2]: (x, x, y, y), (z, z, m, m)
  __shared__ __align__(16) float4 sm[2][kRoBJ * 2];
  const int tid = threadIdx.x;
  const float4* pos4 = reinterpret_cast<const float4*>(a.pos);
  const float2 e2 = make_float2(a.eps2, a.eps2);

  for (int32_t t = blockIdx.x; t < num_tiles; t += gridDim.x) {
    const RoTile tl = tiles[t];
    const SystemDesc sd = a.sys[tl.sys];
    const int ibase = tl.itile * kRoBI;
    const int64_t rec0 = sd.offset >> 1;  // first pair record of the system
    const int last_rec = (sd.npad >> 1) - 1;

    float2 nx[kRoPairs], ny[kRoPairs], nz[kRoPairs], ax[kRoPairs], ay[kRoPairs], az[kRoPairs];
    int li[kRoPairs];
#pragma unroll
    for (int k = 0; k < kRoPairs; ++k) {
      li[k] = ibase + 2 * (k * kRoThreads + tid);
      const int r = min(li[k] >> 1, last_rec);  // lanes past the system read its last record
      const float4 A = pos4[(rec0 + r) * 2];      // (x0, x1, y0, y1)
      const float4 B = pos4[(rec0 + r) * 2 + 1];  // (z0, z1, m0, m1)
      nx[k] = make_float2(-A.x, -A.y);
      ny[k] = make_float2(-A.z, -A.w);
      nz[k] = make_float2(-B.x, -B.y);
      ax[k] = ay[k] = az[k] = make_float2(0.f, 0.f);
    }

    const int ntiles_j = (sd.n + kRoBJ - 1) / kRoBJ;
    float4 pa[kRoRecsPerThread], pb[kRoRecsPerThread];
    // Stage j-tile jt's records (only those holding real particles) into registers.
    auto fetch = [&](int jt) {
      const int nrec = (min(kRoBJ, sd.n - jt * kRoBJ) + 1) >> 1;
#pragma unroll
      for (int q = 0; q < kRoRecsPerThread; ++q) {
        const int r = q * kRoThreads + tid;
        if (r < nrec) {
          const int64_t g = rec0 + jt * kRoRecs + r;
          pa[q] = pos4[g * 2];
          pb[q] = pos4[g * 2 + 1];
        }
      }
    };
    auto stage = [&](int jt, int buf) {
      const int nrec = (min(kRoBJ, sd.n - jt * kRoBJ) + 1) >> 1;
#pragma unroll
      for (int q = 0; q < kRoRecsPerThread; ++q) {
        const int r = q * kRoThreads + tid;
        if (r < nrec) {
          float4* d = &sm[buf][4 * r];
          d[0] = make_float4(pa[q].x, pa[q].x, pa[q].z, pa[q].z);
          d[1] = make_float4(pb[q].x, pb[q].x, pb[q].z, pb[q].z);
          d[2] = make_float4(pa[q].y, pa[q].y, pa[q].w, pa[q].w);
          d[3] = make_float4(pb[q].y, pb[q].y, pb[q].w, pb[q].w);
        }
      }
    };

    __syncthreads();  // the previous i-tile's last reads of sm[] are done
    fetch(0);
    stage(0, 0);
    __syncthreads();
    for (int jt = 0; jt < ntiles_j; ++jt) {
      const int buf = jt & 1;
      if (jt + 1 < ntiles_j) fetch(jt + 1);
      const int j0 = jt * kRoBJ;
      const int count = min(kRoBJ, sd.n - j0);
      const bool diag = (j0 < ibase + kRoBI) && (ibase < j0 + count);
      if (diag)
        ro_tile<kRoPairs, true>(sm[buf], count, j0, e2, nx, ny, nz, ax, ay, az, li);
      else
        ro_tile<kRoPairs, false>(sm[buf], count, j0, e2, nx, ny, nz, ax, ay, az, li);
      if (jt + 1 < ntiles_j) stage(jt + 1, buf ^ 1);
      __syncthreads();
    }

#pragma unroll
    for (int k = 0; k < kRoPairs; ++k) {
      if (li[k] < sd.n)
        finish_particle(a, sd, sd.offset + li[k], ax[k].x, ay[k].x, az[k].x, -nx[k].x, -ny[k].x,
                        -nz[k].x);
      if (li[k] + 1 < sd.n)
        finish_particle(a, sd, sd.offset + li[k] + 1, ax[k].y, ay[k].y, az[k].y, -nx[k].y,
                        -ny[k].y, -nz[k].y);
    }
  }
}

struct RoShapeEntry {
  int threads;
  int pairs;
  void (*kernel)(const ForceArgs, const RoTile*, int32_t);
};

// Largest i-tiles first.  Measured at N = 1M: 128 x 4 64.4 %, 128 x 2 62.8 % of FP32
// peak; the 64 x 1 shape gives a 25,600-particle system 200 CTAs instead of 25.
const RoShapeEntry kRoShapes[] = {
    {128, 4, reference_order_kernel<128, 4>},
    {128, 2, reference_order_kernel<128, 2>},
    {64, 1, reference_order_kernel<64, 1>},
};
constexpr int kNumRoShapes = sizeof(kRoShapes) / sizeof(kRoShapes[0]);

}  // namespace

int reference_order_num_shapes() { return kNumRoShapes; }

KernelShape reference_order_shape(int index) {
  const RoShapeEntry& e = kRoShapes[index];
  return KernelShape{e.threads, 2 * e.pairs, kRoBJ, 2};
}

cudaError_t reference_order_blocks_per_sm(int index, int* blocks) {
  const RoShapeEntry& e = kRoShapes[index];
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, e.kernel, e.threads, 0);
}

cudaError_t launch_reference_order(int index, const ForceArgs& a, const int32_t* tiles,
                                   int32_t num_tiles, int grid, cudaStream_t stream) {
  if (num_tiles <= 0) return cudaSuccess;
  const RoShapeEntry& e = kRoShapes[index];
  e.kernel<<<grid, e.threads, 0, stream>>>(a, reinterpret_cast<const RoTile*>(tiles), num_tiles);
  return cudaGetLastError();
}

}  // namespace nbg
