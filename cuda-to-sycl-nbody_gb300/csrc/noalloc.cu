// Accelerations for callers that cannot allocate GPU memory.
//
// Some callers of a physics step own every byte of GPU memory themselves: a
// render engine or plugin host that hands out pre-sized buffers from its own
// pools, a real-time loop that must not hit cudaMalloc's implicit device-wide
// synchronization in the middle of a frame, or a process that reserves its whole
// memory budget up front.  nb_accelerations_noalloc serves them.  They pass
// their own input and output buffers; the library allocates nothing on the
// device and, on success, nothing on the host.
//
// The work the force kernel needs beyond its input and output -- the work list,
// the partial sums of i-tiles whose j-range is split between CTAs, the arrival
// counters, a copy of the positions in the kernel's pair layout, and the error
// word -- lives in one file-scope device array, kScratchBytes (13 MiB) long.
// Every GPU that loads this module keeps that array until the process exits.
// All calls share it and it keeps the last call's contents: each call clears
// what must start at zero (the counters and the error word), and calls whose
// kernels overlap on the GPU (e.g. on two streams) race on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "nb_internal.hpp"
#include "nb_kernels.hpp"
#include "nb_runtime.hpp"
#include "nbody_gb300.h"

namespace nbg {

namespace {

constexpr int kNaConfig = 0;                  // kernel shape: 128 threads x 4 i, 256-particle j-tiles
constexpr int kNaBI = 512;                    // i-particles per CTA of that shape
constexpr int kNaBJ = 256;                    // j-particles per tile of that shape
constexpr int64_t kNaMaxParticles = 1 << 18;  // 262,144
constexpr int kNaMaxGrid = 1024;
constexpr int kNaMaxSegments = 2048;
constexpr int kNaMaxSlots = 1024;
constexpr int kNaMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }

constexpr size_t kOffSys = 0;
constexpr size_t kOffErr = 256;
constexpr size_t kOffCounters = 512;
constexpr size_t kOffFix = align256(kOffCounters + sizeof(int32_t) * kNaMaxGrid);
constexpr size_t kOffBegin = align256(kOffFix + sizeof(Fixup) * kNaMaxGrid);
constexpr size_t kOffSegs = align256(kOffBegin + sizeof(int32_t) * (kNaMaxGrid + 1));
constexpr size_t kOffPos = align256(kOffSegs + sizeof(Segment) * kNaMaxSegments);
constexpr size_t kOffPartials = align256(kOffPos + 16 * kNaMaxParticles);
constexpr size_t kScratchBytes = align256(kOffPartials + sizeof(float4) * kNaBI * kNaMaxSlots);
static_assert(kScratchBytes <= (13u << 20), "no-allocation scratch is stated as 13 MiB");

}  // namespace

// The scratch array.  In host code this name is only a host-side stand-in:
// host code must take the device address with cudaGetSymbolAddress (below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

// Input float4 (x, y, z, m) -> pair layout in the scratch, padding far away.
__global__ void na_to_pair_layout(const float4* __restrict__ in, int64_t n, int64_t npad,
                                  float* __restrict__ pos) {
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < npad;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const float4 v = g < n ? in[g] : make_float4(kFarAway, kFarAway, kFarAway, 0.f);
    pos[pair_index(g, 0)] = v.x;
    pos[pair_index(g, 1)] = v.y;
    pos[pair_index(g, 2)] = v.z;
    pos[pair_index(g, 3)] = v.w;
  }
}

struct DeviceSetup {
  bool ready = false;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
  int grid = 0;
};

std::mutex g_na_mutex;                       // guards the host-side tables below
DeviceSetup g_na_setup[kNaMaxDevices];
Segment g_na_segs[kNaMaxSegments];           // host plan, uploaded every call
int32_t g_na_begin[kNaMaxGrid + 1];
Fixup g_na_fix[kNaMaxGrid];

// Once per device, with that device current: the scratch's device address and
// the persistent grid size.
int na_setup(int dev, DeviceSetup* out) {
  DeviceSetup& d = g_na_setup[dev];
  if (!d.ready) {
    int sms = 0;
    cudaDeviceProp prop;
    NB_TRY(check_device(&sms, &prop));
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(no-allocation scratch)");
    int blocks = 0;
    NB_CUDA(force_blocks_per_sm(kNaConfig, false, true, &blocks));
    const KernelShape sh = force_config_shape(kNaConfig);
    if (sh.bi() != kNaBI || sh.bj != kNaBJ)
      return set_error(NB_ERR_STATE, "no-allocation kernel shape mismatch");
    d.scratch = static_cast<unsigned char*>(p);
    d.grid = blocks * sms < kNaMaxGrid ? blocks * sms : kNaMaxGrid;
    if (d.grid < 1) d.grid = 1;
    d.ready = true;
  }
  *out = d;
  return NB_OK;
}

// The stream-K plan of the force kernel (same rule as plan_worklist) for one
// system, written into the fixed host tables.  Returns false if they are too small.
bool na_plan(int32_t n, int32_t npad, int32_t grid_max, int32_t* grid, int32_t* nseg,
             int32_t* nfix, int32_t* nslots) {
  const int64_t nit = (n + kNaBI - 1) / kNaBI;
  const int64_t njt = (npad + kNaBJ - 1) / kNaBJ;
  const int64_t total = nit * npad;
  const int64_t g = std::max<int64_t>(1, std::min<int64_t>(grid_max, nit * njt));
  int32_t segs = 0, fix = 0, slots = 0;
  int64_t next_cta = 0;
  for (int64_t it = 0; it < nit; ++it) {
    const int64_t c0 = it * npad;
    const int32_t first = segs;
    int64_t t = 0;
    while (t < njt) {
      const int64_t k = std::min<int64_t>(g - 1, ((c0 + t * kNaBJ) * g) / total);
      int64_t t_end = njt;
      if (k + 1 < g) {
        const int64_t need = (k + 1) * total - c0 * g;
        t_end = (need + static_cast<int64_t>(kNaBJ) * g - 1) / (static_cast<int64_t>(kNaBJ) * g);
        t_end = std::min<int64_t>(std::max<int64_t>(t_end, t + 1), njt);
      }
      if (segs >= kNaMaxSegments) return false;
      while (next_cta <= k) g_na_begin[next_cta++] = segs;
      g_na_segs[segs++] = Segment{0, static_cast<int32_t>(it), static_cast<int32_t>(t),
                                  static_cast<int32_t>(t_end), -1, 0};
      t = t_end;
    }
    const int32_t parts = segs - first;
    if (parts > 1) {
      if (fix >= kNaMaxGrid || slots + parts > kNaMaxSlots) return false;
      g_na_fix[fix] = Fixup{parts, slots};
      for (int32_t p = 0; p < parts; ++p) {
        g_na_segs[first + p].fix = fix;
        g_na_segs[first + p].part = p;
      }
      ++fix;
      slots += parts;
    }
  }
  while (next_cta <= g) g_na_begin[next_cta++] = segs;
  *grid = static_cast<int32_t>(g);
  *nseg = segs;
  *nfix = fix;
  *nslots = slots;
  return true;
}

}  // namespace

}  // namespace nbg

using namespace nbg;

extern "C" int nb_accelerations_noalloc(const float* pos_xyzm_device, uint64_t n, float G,
                                        float dist_eps, float* accel_xyzw_device,
                                        void* stream) {
  if (!pos_xyzm_device || !accel_xyzw_device)
    return set_error(NB_ERR_INVALID_ARGUMENT, "NULL device buffer");
  if ((reinterpret_cast<uintptr_t>(pos_xyzm_device) & 15) ||
      (reinterpret_cast<uintptr_t>(accel_xyzw_device) & 15))
    return set_error(NB_ERR_INVALID_ARGUMENT, "device buffers must be 16-byte aligned");
  if (n == 0 || n > static_cast<uint64_t>(kNaMaxParticles))
    return set_error(NB_ERR_INVALID_ARGUMENT,
                     "nb_accelerations_noalloc takes 1 to 262144 particles (its fixed "
                     "13 MiB device scratch); use nb_sim_accelerations for more");
  if (!std::isfinite(G) || !std::isfinite(dist_eps) || dist_eps < 0.f)
    return set_error(NB_ERR_INVALID_ARGUMENT, "G and dist_eps must be finite, dist_eps >= 0");
  int dev = 0;
  NB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNaMaxDevices) return set_error(NB_ERR_NO_DEVICE, "device ordinal");
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  std::lock_guard<std::mutex> lock(g_na_mutex);
  DeviceSetup d;
  NB_TRY(na_setup(dev, &d));
  const int32_t ni = static_cast<int32_t>(n);
  const int32_t npad = (ni + kPadQuantum - 1) / kPadQuantum * kPadQuantum;
  int32_t grid = 0, nseg = 0, nfix = 0, nslots = 0;
  if (!na_plan(ni, npad, d.grid, &grid, &nseg, &nfix, &nslots))
    return set_error(NB_ERR_INVALID_ARGUMENT, "work list exceeds the no-allocation scratch");

  SystemDesc sd{};
  sd.offset = 0;
  sd.n = ni;
  sd.npad = npad;
  sd.gscale = G;  // per-pair masses: each pair term carries m_j
  sd.mass = 0.f;
  sd.equal_mass = 0;
  unsigned char* base = d.scratch;
  // Host sources are pageable: each copy has read them before it returns.
  NB_CUDA(cudaMemcpyAsync(base + kOffSys, &sd, sizeof(sd), cudaMemcpyHostToDevice, st));
  NB_CUDA(cudaMemcpyAsync(base + kOffSegs, g_na_segs, sizeof(Segment) * nseg,
                          cudaMemcpyHostToDevice, st));
  NB_CUDA(cudaMemcpyAsync(base + kOffBegin, g_na_begin, sizeof(int32_t) * (grid + 1),
                          cudaMemcpyHostToDevice, st));
  if (nfix > 0)
    NB_CUDA(cudaMemcpyAsync(base + kOffFix, g_na_fix, sizeof(Fixup) * nfix,
                            cudaMemcpyHostToDevice, st));
  // What must start at zero: the arrival counters and the error word.
  NB_CUDA(cudaMemsetAsync(base + kOffCounters, 0, sizeof(int32_t) * kNaMaxGrid, st));
  NB_CUDA(cudaMemsetAsync(base + kOffErr, 0, sizeof(int32_t), st));
  float* pos = reinterpret_cast<float*>(base + kOffPos);
  na_to_pair_layout<<<(npad + 255) / 256, 256, 0, st>>>(
      reinterpret_cast<const float4*>(pos_xyzm_device), static_cast<int64_t>(n), npad, pos);
  NB_CUDA(cudaGetLastError());

  ForceArgs a{};
  a.pos = pos;
  a.pos_next = nullptr;
  a.vel = nullptr;
  a.accel_out = reinterpret_cast<float4*>(accel_xyzw_device);
  a.sys = reinterpret_cast<const SystemDesc*>(base + kOffSys);
  a.segs = reinterpret_cast<const Segment*>(base + kOffSegs);
  a.seg_begin = reinterpret_cast<const int32_t*>(base + kOffBegin);
  a.fix = reinterpret_cast<const Fixup*>(base + kOffFix);
  a.partials = reinterpret_cast<float4*>(base + kOffPartials);
  a.counters = reinterpret_cast<int32_t*>(base + kOffCounters);
  a.err = reinterpret_cast<int32_t*>(base + kOffErr);
  a.eps2 = dist_eps;
  a.dt = 0.f;
  a.damping = 0.f;
  {
    const float e3 = dist_eps * dist_eps * dist_eps;
    a.mask_self = (e3 >= FLT_MIN) ? 0 : 1;
  }
  a.skip_first_tile = 0;
  NB_CUDA(launch_force(kNaConfig, false, true, a, grid, st));
  int32_t err = 0;
  NB_CUDA(cudaMemcpyAsync(&err, base + kOffErr, sizeof(err), cudaMemcpyDeviceToHost, st));
  NB_CUDA(cudaStreamSynchronize(st));
  if (err != 0)
    return set_error(NB_ERR_DEVICE_TIMEOUT, "a bounded device-side wait timed out");
  return NB_OK;
}
