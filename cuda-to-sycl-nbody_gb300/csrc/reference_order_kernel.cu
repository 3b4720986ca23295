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
// GB300 design:
//   * The two lanes of each packed FP32x2 register pair hold two different
//     i-particles (each lane its own running sum, so the order per particle is
//     untouched).  j-particles come from a copy of the positions laid out
//     duplicated, (x, x, y, y) (z, z, m, m) per particle (ro_dup_kernel, one pass
//     per step), so one broadcast 16-byte shared load feeds both lanes.
//   * j-tiles of that copy are staged global -> shared by cp.async.bulk into a
//     three-deep ring in dynamic shared memory with mbarrier completion, like the
//     fast kernel.
//   * Persistent grid with a stream-K work list (worklist.hpp): every CTA gets
//     the same number of pair interactions to within one j-tile, whatever the
//     number of i-tiles, so the last wave is never part-empty.  A particle's sum
//     cannot be split into independently summed parts, so an i-tile whose j-range
//     is cut between CTAs is *handed over* instead: the part over the first
//     j-tiles stores its running sums, and the CTA owning the next part starts
//     from them, in j order -- the same sequence of roundings as one CTA.  Each
//     CTA walks its segments last to first: the part it hands over (its last
//     segment) is done first and the part it continues (its first segment) last,
//     so by the time a CTA needs its predecessor's sums they are long written.
//     The launch is cooperative (all CTAs resident), and every wait -- on an
//     mbarrier or on a predecessor -- is bounded (2 s of %globaltimer); on
//     timeout the CTA sets bit 0 of the error word, drains its own copies and
//     exits.
//   * Only the n real particles of a system are summed (no padding terms), as in
//     the reference.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "nb_device.cuh"
#include "nb_internal.hpp"
#include "nb_kernels.hpp"

namespace nbg {
namespace {

constexpr int kRoStages = 3;   // depth of the tile ring
constexpr uint64_t kRoWaitNs = 2000000000ull;

__device__ __forceinline__ uint32_t ro_smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t ro_global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void ro_mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(ro_smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void ro_fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void ro_fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void ro_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ro_smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Bulk copy global -> shared; both addresses 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void ro_bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          ro_smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(ro_smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool ro_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(ro_smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on phase `parity`; false after kRoWaitNs.
__device__ __noinline__ bool ro_wait_slow(uint64_t* bar, uint32_t parity) {
  const uint64_t t0 = ro_global_ns();
  while (true) {
    if (ro_try_wait(bar, parity)) return true;
    if (ro_global_ns() - t0 > kRoWaitNs) return false;
  }
}

__device__ __forceinline__ bool ro_wait(uint64_t* bar, uint32_t parity) {
  if (ro_try_wait(bar, parity)) return true;
  return ro_wait_slow(bar, parity);
}

// Bounded wait until the hand-over counter reaches `target`; false after kRoWaitNs.
__device__ __noinline__ bool ro_wait_counter(const int32_t* counter, int32_t target) {
  const volatile int32_t* c = counter;
  const uint64_t t0 = ro_global_ns();
  while (*c < target) {
    if (ro_global_ns() - t0 > kRoWaitNs) return false;
    __nanosleep(64);
  }
  __threadfence();
  return true;
}

// One j step against all of the thread's i-pairs.  kDiag: the tile overlaps the
// i-tile, so the term of j == i is left out of that lane's sum (the reference's
// `if (i == id) continue;`), by keeping the old value rather than adding zero.
// kPred: the PREDICATED variant as shipped, force += r * inv * (j == i)
// (simulator.cu:209), contracted to fma(r * inv, mask, force) for every j.
template <int P, bool kDiag, bool kPred>
__device__ __forceinline__ void ro_step(const float4 xy, const float4 zm, float2 e2,
                                        const float2 (&nx)[P], const float2 (&ny)[P],
                                        const float2 (&nz)[P], float2 (&ax)[P],
                                        float2 (&ay)[P], float2 (&az)[P], int j,
                                        const int (&li)[P]) {
  const float2 xx = make_float2(xy.x, xy.y);
  const float2 yy = make_float2(xy.z, xy.w);
  const float2 zz = make_float2(zm.x, zm.y);
#pragma unroll
  for (int k = 0; k < P; ++k) {
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
    if (kPred) {
      const float2 mask = kDiag ? make_float2(j == li[k] ? 1.f : 0.f, j == li[k] + 1 ? 1.f : 0.f)
                                : make_float2(0.f, 0.f);
      ax[k] = __ffma2_rn(__fmul2_rn(rx, inv), mask, ax[k]);
      ay[k] = __ffma2_rn(__fmul2_rn(ry, inv), mask, ay[k]);
      az[k] = __ffma2_rn(__fmul2_rn(rz, inv), mask, az[k]);
      continue;
    }
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
template <int P, bool kDiag, bool kPred, int kRoUnroll>
__device__ __forceinline__ void ro_tile(const float4* __restrict__ tile, int count, int j0,
                                        float2 e2, const float2 (&nx)[P], const float2 (&ny)[P],
                                        const float2 (&nz)[P], float2 (&ax)[P], float2 (&ay)[P],
                                        float2 (&az)[P], const int (&li)[P]) {
  int jj = 0;
#pragma unroll 1
  for (; jj + kRoUnroll <= count; jj += kRoUnroll) {
#pragma unroll
    for (int u = 0; u < kRoUnroll; ++u)
      ro_step<P, kDiag, kPred>(tile[2 * (jj + u)], tile[2 * (jj + u) + 1], e2, nx, ny, nz, ax, ay, az,
                        j0 + jj + u, li);
  }
#pragma unroll 1
  for (; jj < count; ++jj)
    ro_step<P, kDiag, kPred>(tile[2 * jj], tile[2 * jj + 1], e2, nx, ny, nz, ax, ay, az, j0 + jj, li);
}

// The duplicated j-layout from the pair layout: one thread per pair record.
__global__ void ro_dup_kernel(const float4* __restrict__ pos4, int64_t records,
                              float4* __restrict__ dup) {
  for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < records;
       r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const float4 A = pos4[2 * r];      // (x0, x1, y0, y1)
    const float4 B = pos4[2 * r + 1];  // (z0, z1, m0, m1)
    dup[4 * r + 0] = make_float4(A.x, A.x, A.z, A.z);
    dup[4 * r + 1] = make_float4(B.x, B.x, B.z, B.z);
    dup[4 * r + 2] = make_float4(A.y, A.y, A.w, A.w);
    dup[4 * r + 3] = make_float4(B.y, B.y, B.w, B.w);
  }
}

// THREADS threads x P i-pairs per thread (i-tiles of 2 P THREADS particles), j-tiles
// of BJ particles (the ring holds kRoStages of them, BJ x 32 bytes each), U j steps
// per unrolled block, registers budgeted for MINB resident CTAs per SM; kPred: the
// PREDICATED variant's pair term (ro_step).
template <int THREADS, int P, int BJ, int U, int MINB, bool kPred>
__global__ void __launch_bounds__(THREADS, MINB) reference_order_kernel(
    const ForceArgs a, const float4* __restrict__ dup) {
  constexpr int BI = THREADS * 2 * P;  // i-particles per i-tile
  static_assert(BI % kPadQuantum == 0, "i-tiles must hold whole padding quanta");
  extern __shared__ __align__(128) float4 ring_smem[];  // [kRoStages][BJ * 2]
  auto ring = [&](uint32_t slot) { return ring_smem + slot * (BJ * 2); };
  __shared__ __align__(8) uint64_t full_bar[kRoStages];
  __shared__ int s_bail;

  const int tid = threadIdx.x;
  const int seg_lo = a.seg_begin[blockIdx.x];
  const int seg_hi = a.seg_begin[blockIdx.x + 1];
  if (seg_lo >= seg_hi) return;

  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < kRoStages; ++s) ro_mbar_init(&full_bar[s], 1);
    ro_fence_mbar_init();
    s_bail = 0;
  }
  __syncthreads();

  // Producer cursor (thread 0): segments last to first, j-tiles in order within each.
  int p_seg = seg_hi - 1;
  int p_jt = a.segs[p_seg].jt0;
  uint32_t issued = 0;
  auto produce = [&]() {
    if (p_seg < seg_lo) return;
    const Segment& sg = a.segs[p_seg];
    const SystemDesc& sd = a.sys[sg.sys];
    const int count = min(BJ, sd.n - p_jt * BJ);
    const int64_t first = sd.offset + static_cast<int64_t>(p_jt) * BJ;
    const uint32_t slot = issued % kRoStages;
    // Failure-detection test: leave the first tile's barrier without arrival or
    // copy, so the consumers' bounded wait on it runs out.
    if (!(a.inject == kInjectSkipFirstTile && issued == 0)) {
      ro_fence_proxy_async();
      ro_arrive_expect_tx(&full_bar[slot], static_cast<uint32_t>(count) * 32u);
      ro_bulk_g2s(ring(slot), dup + 2 * first, static_cast<uint32_t>(count) * 32u,
                  &full_bar[slot]);
    }
    ++issued;
    if (++p_jt >= sg.jt1) {
      --p_seg;
      if (p_seg >= seg_lo) p_jt = a.segs[p_seg].jt0;
    }
  };
  if (tid == 0) {
#pragma unroll
    for (int k = 0; k < kRoStages - 1; ++k) produce();
  }

  const float4* pos4 = reinterpret_cast<const float4*>(a.pos);
  const float2 e2 = make_float2(a.eps2, a.eps2);
  uint32_t consumed = 0;

  // Give up: flag the error, drain this CTA's copies still in flight (bounded) and
  // leave without touching the outputs.
  auto bail = [&]() {
    if (tid == 0) {
      atomicOr(a.err, 1);
      for (uint32_t k = consumed; k < issued; ++k)
        (void)ro_wait(&full_bar[k % kRoStages], (k / kRoStages) & 1u);
    }
  };

  for (int sgi = seg_hi - 1; sgi >= seg_lo; --sgi) {
    const Segment sg = a.segs[sgi];
    const SystemDesc sd = a.sys[sg.sys];
    const int ibase = sd.shard_first + sg.itile * BI;
    const int iend = shard_end(sd);
    const int64_t rec0 = sd.offset >> 1;  // first pair record of the system
    const int last_rec = (sd.npad >> 1) - 1;
    const bool split = sg.fix >= 0;
    const Fixup fx = split ? a.fix[sg.fix] : Fixup{1, 0};
    float4* slots = a.partials + static_cast<int64_t>(fx.slot0) * BI;

    float2 nx[P], ny[P], nz[P], ax[P], ay[P], az[P];
    int li[P];
#pragma unroll
    for (int k = 0; k < P; ++k) {
      li[k] = ibase + 2 * (k * THREADS + tid);
      const int r = min(li[k] >> 1, last_rec);  // lanes past the system read its last record
      const float4 A = pos4[(rec0 + r) * 2];      // (x0, x1, y0, y1)
      const float4 B = pos4[(rec0 + r) * 2 + 1];  // (z0, z1, m0, m1)
      nx[k] = make_float2(-A.x, -A.y);
      ny[k] = make_float2(-A.z, -A.w);
      nz[k] = make_float2(-B.x, -B.y);
      ax[k] = ay[k] = az[k] = make_float2(0.f, 0.f);
    }

    if (split && sg.part > 0) {
      // Continue the running sums where the previous part of this i-tile stopped.
      if (tid == 0 && !ro_wait_counter(&a.counters[sg.fix], sg.part)) s_bail = 1;
      __syncthreads();
      if (s_bail) {
        bail();
        return;
      }
      const float4* in = slots + static_cast<int64_t>(sg.part - 1) * BI;
#pragma unroll
      for (int k = 0; k < P; ++k) {
        const int idx = k * THREADS + tid;
        const float4 u = __ldcg(&in[2 * idx]);
        const float4 w = __ldcg(&in[2 * idx + 1]);
        ax[k] = make_float2(u.x, u.y);
        ay[k] = make_float2(u.z, u.w);
        az[k] = make_float2(w.x, w.y);
      }
    }

    bool timed_out = false;
    for (int jt = sg.jt0; jt < sg.jt1; ++jt, ++consumed) {
      if (tid == 0) produce();
      const uint32_t slot = consumed % kRoStages;
      if (!ro_wait(&full_bar[slot], (consumed / kRoStages) & 1u)) timed_out = true;
      const int j0 = jt * BJ;
      const int count = min(BJ, sd.n - j0);
      const bool diag = (j0 < ibase + BI) && (ibase < j0 + count);
      if (!timed_out) {
        if (diag)
          ro_tile<P, true, kPred, U>(ring(slot), count, j0, e2, nx, ny, nz, ax, ay, az, li);
        else
          ro_tile<P, false, kPred, U>(ring(slot), count, j0, e2, nx, ny, nz, ax, ay, az, li);
      }
      if (__syncthreads_or(timed_out)) {
        bail();
        return;
      }
    }

    if (split && sg.part < fx.nparts - 1) {
      // Hand the running sums to the CTA that owns the next part.
      float4* out = slots + static_cast<int64_t>(sg.part) * BI;
#pragma unroll
      for (int k = 0; k < P; ++k) {
        const int idx = k * THREADS + tid;
        __stcg(&out[2 * idx], make_float4(ax[k].x, ax[k].y, ay[k].x, ay[k].y));
        __stcg(&out[2 * idx + 1], make_float4(az[k].x, az[k].y, 0.f, 0.f));
      }
      __threadfence();
      __syncthreads();
      // (Failure-detection test: withhold it, so the next part's bounded wait runs out.)
      if (tid == 0 && a.inject != kInjectWithholdHandOver) atomicAdd(&a.counters[sg.fix], 1);
      continue;
    }
    if (split && tid == 0) a.counters[sg.fix] = 0;  // every part has run: reset for the next launch

#pragma unroll
    for (int k = 0; k < P; ++k) {
      if (li[k] < iend)
        finish_particle(a, sd, sd.offset + li[k], ax[k].x, ay[k].x, az[k].x, -nx[k].x, -ny[k].x,
                        -nz[k].x);
      if (li[k] + 1 < iend)
        finish_particle(a, sd, sd.offset + li[k] + 1, ax[k].y, ay[k].y, az[k].y, -nx[k].y,
                        -ny[k].y, -nz[k].y);
    }
  }
}

struct RoShapeEntry {
  int threads;
  int pairs;
  int bj;
  void (*kernel[2])(const ForceArgs, const float4*);  // [BRANCH, PREDICATED]
};

#define RO_SHAPE(T, P, BJ, U, B)                                                   \
  {T, P, BJ, {reference_order_kernel<T, P, BJ, U, B, false>,                       \
              reference_order_kernel<T, P, BJ, U, B, true>}}
// Largest i-tiles first; the default for a system is the first shape whose i-tiles
// give every SM two CTAs (one where only one fits), else the last.  Measured
// (thin disk, ms per step; every variant gave the same bits):
//   * N = 1M and 262,144: 384 x 2 x 1024 (12 warps, one CTA per SM, 4 j-steps per
//     unrolled block) 390.9 / 24.6 ms, 69.8 % of nominal FP32 peak at 1M.  Deeper
//     unrolling (16 j-steps) 398.0 / 25.0; 128 x 2, 256 x 1 and 64 x 1 shapes
//     418-445 / 25.3-27.8; 512 x 2 67.9 % and 256 x 2 66.5 % at 1M; 448 x 2 and
//     320 x 2 (warps not a multiple of the SM's four schedulers) 59 %; 256 x 4,
//     384 x 3 and 256 x 3 68.3-69.4 % at 1M but 51-68 % at 262,144.
//   * Below that, few i-tiles leave each scheduler about one warp, and what hides the
//     pair chain's latency (about 80 cycles from shared load to accumulate) is the
//     number of independent j-steps a thread has in flight: one i-pair per thread,
//     32 j-steps per unrolled block (128 registers).  At 196,608: 256 x 1 x 1024
//     14.2 ms (384 x 2 16.4, 128 x 2 x 256 with 4 j-steps 17.7); at 131,072:
//     128 x 1 x 1024 6.61 (64 x 1 x 1024 6.98, 384 x 2 10.9); at 65,536:
//     64 x 1 x 1024 1.76 (128 x 2 x 256 2.25); at 25,600: 0.418 (64 x 1 x 256 with
//     4 j-steps 0.605); at 2,048: 0.045 (0.057).  2048-particle j-tiles (one CTA
//     per SM) halve the rate of the 64-thread shape.
const RoShapeEntry kRoShapes[] = {
    RO_SHAPE(384, 2, 1024, 4, 1),
    RO_SHAPE(256, 1, 1024, 32, 1),
    RO_SHAPE(128, 1, 1024, 32, 1),
    RO_SHAPE(64, 1, 1024, 32, 1),
};
constexpr int kNumRoShapes = sizeof(kRoShapes) / sizeof(kRoShapes[0]);

size_t ro_smem_bytes(const RoShapeEntry& e) {
  return static_cast<size_t>(kRoStages) * e.bj * 32;
}

// Rings of 48 KB or more opt in to the larger dynamic shared memory, once per
// device ordinal and shape (ordinals >= 64 opt in on every call).
cudaError_t ro_smem_opt_in(int index) {
  static std::atomic<uint64_t> opted[kNumRoShapes];
  const RoShapeEntry& e = kRoShapes[index];
  if (ro_smem_bytes(e) < 48 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  const uint64_t bit = dev >= 0 && dev < 64 ? uint64_t{1} << dev : 0;
  if (bit != 0 && (opted[index].load(std::memory_order_acquire) & bit) != 0) return cudaSuccess;
  for (int v = 0; v < 2 && err == cudaSuccess; ++v)
    err = cudaFuncSetAttribute(e.kernel[v], cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(ro_smem_bytes(e)));
  if (err == cudaSuccess && bit != 0) opted[index].fetch_or(bit, std::memory_order_release);
  return err;
}

}  // namespace

int reference_order_num_shapes() { return kNumRoShapes; }

KernelShape reference_order_shape(int index) {
  const RoShapeEntry& e = kRoShapes[index];
  return KernelShape{e.threads, 2 * e.pairs, e.bj, kRoStages};
}

cudaError_t reference_order_blocks_per_sm(int index, bool predicated, int* blocks) {
  const RoShapeEntry& e = kRoShapes[index];
  const cudaError_t err = ro_smem_opt_in(index);
  if (err != cudaSuccess) return err;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, e.kernel[predicated], e.threads,
                                                       ro_smem_bytes(e));
}

cudaError_t launch_reference_order_dup(const float* pos, int64_t n_pad_total, float4* dup,
                                       cudaStream_t stream) {
  const int64_t records = n_pad_total / 2;
  const int threads = 256;
  const int64_t blocks = (records + threads - 1) / threads;
  ro_dup_kernel<<<static_cast<int>(blocks < 65535 * 16 ? blocks : 65535 * 16), threads, 0,
                  stream>>>(reinterpret_cast<const float4*>(pos), records, dup);
  return cudaGetLastError();
}

cudaError_t launch_reference_order(int index, bool predicated, const ForceArgs& a,
                                   const float4* dup, int grid, cudaStream_t stream) {
  const RoShapeEntry& e = kRoShapes[index];
  const cudaError_t err = ro_smem_opt_in(index);
  if (err != cudaSuccess) return err;
  // Cooperative: every CTA is resident, so a CTA waiting for its predecessor's
  // hand-over always waits on a running CTA.
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(e.threads);
  cfg.dynamicSmemBytes = ro_smem_bytes(e);
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, e.kernel[predicated], a, dup);
}

}  // namespace nbg
