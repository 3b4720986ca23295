// All-pairs softened-gravity force + fused integrate step for sm_103a (kernel template;
// force_kernel.cu holds the table of compiled shapes).
//
// Semantics follow the reference kernel particle_interaction<BRANCH>
// (src/simulator.cu:186-229):
//   F_i  = sum_{j != i} m_j r_ij * rsqrt(d2^3),  r_ij = x_j - x_i,
//          d2 = |r_ij|^2 + distEps                        (simulator.cu:197-207)
//   v_i <- v_i * damping + (F_i * dt) * G                 (simulator.cu:214-220)
//   x_i <- x_i + v_i * dt   (written to the next buffer)  (simulator.cu:223-228)
// The reference assumes unit mass; here each system has either equal masses (m
// folded into G outside the pair loop, so the pair loop is the reference's) or
// per-particle masses (one extra multiply per pair).
//
// GB300 design:
//   * Persistent grid (SMs x resident CTAs).  Each CTA walks its slice of a
//     stream-K work list of (system, i-tile, j-tile range) segments built on the
//     host so every CTA gets the same number of pair interactions.  An i-tile
//     whose j-range is cut between CTAs leaves per-part partial sums in a scratch
//     buffer; the last part to arrive (atomic counter) adds the parts in j order,
//     which keeps the result deterministic, and runs the integrate epilogue.
//   * j-tiles are copied global -> shared by cp.async.bulk (the TMA bulk engine)
//     into a STAGES-deep ring, completion tracked by mbarrier transaction counts;
//     thread 0 keeps STAGES-1 tiles in flight.
//   * Each thread holds R i-particles in registers.  The positions are in pair
//     layout, so one 16-byte broadcast shared load gives (x_j0, x_j1, y_j0, y_j1)
//     and the pair math runs on the packed FP32x2 pipe (__fadd2/__ffma2/__fmul2):
//     11 FP32 lane operations and one MUFU rsqrt per pair, half the issue slots of
//     scalar code.
//   * Self pairs contribute exactly zero whenever eps2^3 is a normal float (r = 0),
//     so they are only masked (by index, on tiles that overlap the i-tile) when
//     eps2^3 underflows, where 0 * inf would give NaN; this matches the reference's
//     `if (i == id) continue;`.
//   * Every mbarrier wait is bounded (2 s of %globaltimer); on timeout the CTA sets
//     bit 0 of the error word, drains its own copies (again bounded) and exits.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "nb_device.cuh"
#include "nb_internal.hpp"
#include "nb_kernels.hpp"

namespace nbg {

using LaunchFn = cudaError_t (*)(const ForceArgs&, int, cudaStream_t);
using OccFn = cudaError_t (*)(int*);

// One compiled kernel shape: launchers and occupancy queries indexed by
// [live_slots][compensated][per_pair_mass].
struct ConfigEntry {
  KernelShape shape;
  LaunchFn launch[2][2][2];
  OccFn occ[2][2][2];
};

namespace {


constexpr uint64_t kWaitLimitNs = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Bulk (non-tensor) TMA copy global -> shared; dst, src 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on phase `parity`; false after kWaitLimitNs.
__device__ __noinline__ bool mbar_wait_slow(uint64_t* bar, uint32_t parity) {
  const uint64_t t0 = global_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kWaitLimitNs) return false;
  }
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  return mbar_wait_slow(bar, parity);
}

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// Kahan step on both lanes: (s, c) += t, with s - c the compensated value.
__device__ __forceinline__ void kahan_add2(float2& s, float2& c, float2 t) {
  const float2 y = __fadd2_rn(t, neg2(c));
  const float2 u = __fadd2_rn(s, y);
  c = __fadd2_rn(__fadd2_rn(u, neg2(s)), neg2(y));
  s = u;
}

// Error-free sum of the two lanes plus their compensations -> (hi, lo).
__device__ __forceinline__ void kahan_finish(float2 s, float2 c, float& hi, float& lo) {
  const float a = s.x, b = s.y;
  const float h = a + b;
  const float bb = h - a;
  const float e = (a - (h - bb)) + (b - bb);
  hi = h;
  lo = e - (c.x + c.y);
}

// Pair loop over `npairs` j-pairs of one shared-memory tile (npairs % 8 == 0), U
// j-pairs per unrolled step, for the first RL of the thread's R i-particles (the
// others are past the end of the system and keep their zero sums).
// kMask: zero the term of j == i (tiles overlapping the i-tile when eps2^3 underflows).
template <int RL, int R, int U, bool kMass, bool kMask>
__device__ __forceinline__ void tile_pairs(const float4* __restrict__ tile, int npairs, float2 e2,
                                           const float2 (&nx)[R], const float2 (&ny)[R],
                                           const float2 (&nz)[R], float2 (&ax)[R],
                                           float2 (&ay)[R], float2 (&az)[R], int64_t j_first,
                                           const int64_t (&gi)[R]) {
#pragma unroll 1
  for (int p = 0; p < npairs; p += U) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const float4 A = tile[2 * (p + u)];
      const float4 B = tile[2 * (p + u) + 1];
      const float2 xx = make_float2(A.x, A.y);
      const float2 yy = make_float2(A.z, A.w);
      const float2 zz = make_float2(B.x, B.y);
#pragma unroll
      for (int r = 0; r < RL; ++r) {
        const float2 dx = __fadd2_rn(xx, nx[r]);
        const float2 dy = __fadd2_rn(yy, ny[r]);
        const float2 dz = __fadd2_rn(zz, nz[r]);
        float2 d2 = __ffma2_rn(dx, dx, e2);
        d2 = __ffma2_rn(dy, dy, d2);
        d2 = __ffma2_rn(dz, dz, d2);
        float2 t = __fmul2_rn(d2, d2);
        t = __fmul2_rn(t, d2);
        float2 s = make_float2(rsqrtf(t.x), rsqrtf(t.y));
        if (kMass) s = __fmul2_rn(s, make_float2(B.z, B.w));
        if (kMask) {
          const int64_t j0 = j_first + 2 * (p + u);
          if (j0 == gi[r]) s.x = 0.f;
          if (j0 + 1 == gi[r]) s.y = 0.f;
        }
        ax[r] = __ffma2_rn(dx, s, ax[r]);
        ay[r] = __ffma2_rn(dy, s, ay[r]);
        az[r] = __ffma2_rn(dz, s, az[r]);
      }
    }
  }
}

// tile_pairs over the live register slots: `live` is live_slots() of the i-tile, one
// of 1-4 or R, and only those loop variants are compiled.  Only the kernels built
// with kLive carry these loops: their presence changes how ptxas allocates the full
// loop (236 -> 240 registers for 256 x 4 x 2048, compensated, and 78.5 -> 75.2 % of
// peak at N = 1M), so work lists whose i-tiles are all full keep the kernel without.
template <int R, int U, bool kMass>
__device__ __forceinline__ void tile_pairs_live(int live, const float4* __restrict__ tile,
                                                int npairs, float2 e2, const float2 (&nx)[R],
                                                const float2 (&ny)[R], const float2 (&nz)[R],
                                                float2 (&ax)[R], float2 (&ay)[R], float2 (&az)[R],
                                                int64_t j_first, const int64_t (&gi)[R]) {
  if constexpr (R > 1) {
    if (live == 1) {
      tile_pairs<1, R, U, kMass, false>(tile, npairs, e2, nx, ny, nz, ax, ay, az, j_first, gi);
      return;
    }
  }
  if constexpr (R > 2) {
    if (live == 2) {
      tile_pairs<2, R, U, kMass, false>(tile, npairs, e2, nx, ny, nz, ax, ay, az, j_first, gi);
      return;
    }
  }
  if constexpr (R > 3) {
    if (live == 3) {
      tile_pairs<3, R, U, kMass, false>(tile, npairs, e2, nx, ny, nz, ax, ay, az, j_first, gi);
      return;
    }
  }
  if constexpr (R > 4) {
    if (live == 4) {
      tile_pairs<4, R, U, kMass, false>(tile, npairs, e2, nx, ny, nz, ax, ay, az, j_first, gi);
      return;
    }
  }
  tile_pairs<R, R, U, kMass, false>(tile, npairs, e2, nx, ny, nz, ax, ay, az, j_first, gi);
}

// __launch_bounds__(THREADS, 1): one resident CTA per SM is enough, so ptxas may use up
// to 255 registers per thread for the R i-particles and the unrolled pair loop (with
// the thread bound alone it caps 256-thread shapes at 128 registers, measured 17 %
// slower).
// kLive: skip the register slots past the end of a system in its last i-tile
// (tile_pairs_live); the work list must then be planned with live-slot weights.
template <int THREADS, int R, int BJ, int STAGES, int U, bool kComp, bool kMass, bool kLive>
__global__ void __launch_bounds__(THREADS, 1) force_kernel(const ForceArgs a) {
  constexpr int BI = THREADS * R;
  constexpr int TILE_BYTES = BJ * 16;
  static_assert(BJ % kPadQuantum == 0, "tile must hold whole padding quanta");
  // Every tile (a full one or a system's last, partial one) holds a multiple of
  // kPadQuantum / 2 j-pairs; the pair loop steps U pairs at a time without a
  // remainder, so U must divide that count or the last step reads past the tile.
  static_assert((kPadQuantum / 2) % U == 0, "U must divide the j-pairs of a padding quantum");
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ int s_last;

  const int tid = threadIdx.x;
  const int seg_lo = a.seg_begin[blockIdx.x];
  const int seg_hi = a.seg_begin[blockIdx.x + 1];
  if (seg_lo >= seg_hi) return;

  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < STAGES; ++s) mbar_init(&full_bar[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // Producer cursor (used by thread 0 only): the CTA's flat j-tile sequence.
  int p_seg = seg_lo;
  int p_jt = a.segs[seg_lo].jt0;
  uint32_t issued = 0;
  auto produce = [&]() {
    if (p_seg >= seg_hi) return;
    const Segment& sg = a.segs[p_seg];
    const SystemDesc& sd = a.sys[sg.sys];
    const int count = min(BJ, sd.npad - p_jt * BJ);
    const int64_t first = sd.offset + static_cast<int64_t>(p_jt) * BJ;
    const uint32_t slot = issued % STAGES;
    // Failure-detection test: leave the first tile's barrier without arrival or
    // copy, so the consumers' bounded wait on it runs out.
    if (!(a.inject == kInjectSkipFirstTile && issued == 0)) {
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&full_bar[slot], static_cast<uint32_t>(count) * 16u);
      bulk_g2s(smem + slot * TILE_BYTES, a.pos + first * 4, static_cast<uint32_t>(count) * 16u,
               &full_bar[slot]);
    }
    ++issued;
    if (++p_jt >= sg.jt1) {
      ++p_seg;
      if (p_seg < seg_hi) p_jt = a.segs[p_seg].jt0;
    }
  };
  if (tid == 0) {
#pragma unroll
    for (int k = 0; k < STAGES - 1; ++k) produce();
  }

  const float2 e2 = make_float2(a.eps2, a.eps2);
  uint32_t consumed = 0;
  bool timed_out = false;

  for (int sgi = seg_lo; sgi < seg_hi; ++sgi) {
    const Segment sg = a.segs[sgi];
    const SystemDesc sd = a.sys[sg.sys];
    const int ibase = sd.shard_first + sg.itile * BI;
    const int iend = shard_end(sd);
    const int live = kLive ? live_slots(iend - ibase, THREADS, R) : R;  // slots to run

    float2 nx[R], ny[R], nz[R], ax[R], ay[R], az[R];
    float2 sx[R], sy[R], sz[R], cx[R], cy[R], cz[R];  // compensated running sums
    int64_t gi[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int li = ibase + r * THREADS + tid;
      const int lc = li < iend ? li : iend - 1;
      gi[r] = sd.offset + lc;
      const float xi = a.pos[pair_index(gi[r], 0)];
      const float yi = a.pos[pair_index(gi[r], 1)];
      const float zi = a.pos[pair_index(gi[r], 2)];
      nx[r] = make_float2(-xi, -xi);
      ny[r] = make_float2(-yi, -yi);
      nz[r] = make_float2(-zi, -zi);
      ax[r] = ay[r] = az[r] = make_float2(0.f, 0.f);
      if (kComp) sx[r] = sy[r] = sz[r] = cx[r] = cy[r] = cz[r] = make_float2(0.f, 0.f);
    }

    for (int jt = sg.jt0; jt < sg.jt1; ++jt, ++consumed) {
      if (tid == 0) produce();
      const uint32_t slot = consumed % STAGES;
      if (!mbar_wait(&full_bar[slot], (consumed / STAGES) & 1u)) timed_out = true;
      const float4* tile = reinterpret_cast<const float4*>(smem + slot * TILE_BYTES);
      const int count = min(BJ, sd.npad - jt * BJ);
      const int64_t j_first = sd.offset + static_cast<int64_t>(jt) * BJ;
      const bool diag = a.mask_self && (jt * BJ < ibase + BI) && (ibase < jt * BJ + count);
      if (diag) {
        tile_pairs<R, R, U, kMass, true>(tile, count >> 1, e2, nx, ny, nz, ax, ay, az, j_first, gi);
      } else if constexpr (kLive) {
        tile_pairs_live<R, U, kMass>(live, tile, count >> 1, e2, nx, ny, nz, ax, ay, az, j_first,
                                     gi);
      } else {
        tile_pairs<R, R, U, kMass, false>(tile, count >> 1, e2, nx, ny, nz, ax, ay, az, j_first,
                                          gi);
      }
      if (kComp) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          kahan_add2(sx[r], cx[r], ax[r]);
          kahan_add2(sy[r], cy[r], ay[r]);
          kahan_add2(sz[r], cz[r], az[r]);
          ax[r] = ay[r] = az[r] = make_float2(0.f, 0.f);
        }
      }
      if (__syncthreads_or(timed_out)) {
        // A tile never arrived: flag it, drain what this CTA still has in flight
        // (bounded), and leave without touching the outputs.
        if (tid == 0) {
          atomicOr(a.err, 1);
          for (uint32_t k = consumed; k < issued; ++k)
            (void)mbar_wait(&full_bar[k % STAGES], (k / STAGES) & 1u);
        }
        return;
      }
    }

    // Per-particle totals of this segment (hi, lo): plain mode has lo = 0.
    float hx[R], hy[R], hz[R], lx[R], ly[R], lz[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (kComp) {
        kahan_finish(sx[r], cx[r], hx[r], lx[r]);
        kahan_finish(sy[r], cy[r], hy[r], ly[r]);
        kahan_finish(sz[r], cz[r], hz[r], lz[r]);
      } else {
        hx[r] = ax[r].x + ax[r].y;
        hy[r] = ay[r].x + ay[r].y;
        hz[r] = az[r].x + az[r].y;
        lx[r] = ly[r] = lz[r] = 0.f;
      }
    }

    if (sg.fix < 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int li = ibase + r * THREADS + tid;
        if (li < iend)
          finish_particle(a, sd, gi[r], hx[r] + lx[r], hy[r] + ly[r], hz[r] + lz[r], -nx[r].x,
                          -ny[r].x, -nz[r].x);
      }
      continue;
    }

    // Split i-tile: publish this part, the last part to arrive finishes the tile.
    const Fixup fx = a.fix[sg.fix];
    constexpr int kRec = kComp ? 2 : 1;
    float4* part = a.partials + (static_cast<int64_t>(fx.slot0) + sg.part) * BI * kRec;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int idx = r * THREADS + tid;
      __stcg(&part[idx * kRec], make_float4(hx[r], hy[r], hz[r], 0.f));
      if (kComp) __stcg(&part[idx * kRec + 1], make_float4(lx[r], ly[r], lz[r], 0.f));
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
      const int old = atomicAdd(&a.counters[sg.fix], 1);
      s_last = (old == fx.nparts - 1);
      if (s_last) a.counters[sg.fix] = 0;  // every part has arrived: reset for the next launch
      __threadfence();
    }
    __syncthreads();
    if (s_last) {
      const float4* base = a.partials + static_cast<int64_t>(fx.slot0) * BI * kRec;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int idx = r * THREADS + tid;
        const int li = ibase + idx;
        if (li >= iend) continue;
        float tx = 0.f, ty = 0.f, tz = 0.f;      // running totals
        float ex = 0.f, ey = 0.f, ez = 0.f;      // compensation (compensated mode)
        float qx = 0.f, qy = 0.f, qz = 0.f;      // sum of the parts' low words
        for (int k = 0; k < fx.nparts; ++k) {
          const float4 h = __ldcg(&base[(static_cast<int64_t>(k) * BI + idx) * kRec]);
          if (kComp) {
            const float4 l = __ldcg(&base[(static_cast<int64_t>(k) * BI + idx) * kRec + 1]);
            float y = h.x - ex, u = tx + y;
            ex = (u - tx) - y;
            tx = u;
            y = h.y - ey;
            u = ty + y;
            ey = (u - ty) - y;
            ty = u;
            y = h.z - ez;
            u = tz + y;
            ez = (u - tz) - y;
            tz = u;
            qx += l.x;
            qy += l.y;
            qz += l.z;
          } else {
            tx += h.x;
            ty += h.y;
            tz += h.z;
          }
        }
        if (kComp) {
          tx += qx - ex;
          ty += qy - ey;
          tz += qz - ez;
        }
        finish_particle(a, sd, gi[r], tx, ty, tz, -nx[r].x, -ny[r].x, -nz[r].x);
      }
    }
  }
}

// Shapes whose tile ring needs 48 KB or more of dynamic shared memory opt in to it
// (with the kernel's static shared memory the 48 KB default is exceeded at exactly
// 48 KB). The attribute belongs to the kernel's instance on the current device, so
// the opt-in is made once per device ordinal (ordinals >= 64 opt in on every call).
template <int T, int R, int BJ, int S, int U, bool C, bool M, bool L>
cudaError_t smem_opt_in() {
  constexpr int smem = S * BJ * 16;
  if (smem < 48 * 1024) return cudaSuccess;
  static std::atomic<uint64_t> opted{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = dev >= 0 && dev < 64 ? uint64_t{1} << dev : 0;
  if (bit != 0 && (opted.load(std::memory_order_acquire) & bit) != 0) return cudaSuccess;
  e = cudaFuncSetAttribute(force_kernel<T, R, BJ, S, U, C, M, L>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess && bit != 0) opted.fetch_or(bit, std::memory_order_release);
  return e;
}

template <int T, int R, int BJ, int S, int U, bool C, bool M, bool L>
cudaError_t launch_one(const ForceArgs& a, int grid, cudaStream_t st) {
  constexpr int smem = S * BJ * 16;
  const cudaError_t e = smem_opt_in<T, R, BJ, S, U, C, M, L>();
  if (e != cudaSuccess) return e;
  force_kernel<T, R, BJ, S, U, C, M, L><<<grid, T, smem, st>>>(a);
  return cudaGetLastError();
}

template <int T, int R, int BJ, int S, int U, bool C, bool M, bool L>
cudaError_t occ_one(int* blocks) {
  constexpr int smem = S * BJ * 16;
  const cudaError_t e = smem_opt_in<T, R, BJ, S, U, C, M, L>();
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, force_kernel<T, R, BJ, S, U, C, M, L>,
                                                       T, smem);
}

}  // namespace

// One shape's launchers (NBG_LAUNCH_L) and occupancy queries (NBG_OCC_L) for one
// value of kLive, as [compensated][per_pair_mass].
#define NBG_LAUNCH_L(T, R, BJ, S, U, L)                                                       \
  {{launch_one<T, R, BJ, S, U, false, false, L>, launch_one<T, R, BJ, S, U, false, true, L>}, \
   {launch_one<T, R, BJ, S, U, true, false, L>, launch_one<T, R, BJ, S, U, true, true, L>}}
#define NBG_OCC_L(T, R, BJ, S, U, L)                                                    \
  {{occ_one<T, R, BJ, S, U, false, false, L>, occ_one<T, R, BJ, S, U, false, true, L>}, \
   {occ_one<T, R, BJ, S, U, true, false, L>, occ_one<T, R, BJ, S, U, true, true, L>}}
#define NBG_CONFIG(T, R, BJ, S, U)                                                  \
  ConfigEntry {                                                                    \
    KernelShape{T, R, BJ, S},                                                      \
        {NBG_LAUNCH_L(T, R, BJ, S, U, false), NBG_LAUNCH_L(T, R, BJ, S, U, true)}, \
        {NBG_OCC_L(T, R, BJ, S, U, false), NBG_OCC_L(T, R, BJ, S, U, true)},       \
  }

}  // namespace nbg
