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
// what must start at zero (the counters and the error word).  Two calls whose
// work overlapped on the GPU would race on it, so each call holds a process-wide
// lock from its first copy until its stream has drained: the calls of one
// process run one after another, whatever streams and threads they come from.
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
#include "worklist.hpp"

namespace nbg {

namespace {

constexpr int kNaConfig = 0;                  // kernel shape: 128 threads x 4 i, 256-particle j-tiles
constexpr int kNaBI = 512;                    // i-particles per CTA of that shape
constexpr int kNaBJ = 256;                    // j-particles per tile of that shape
constexpr int64_t kNaMaxParticles = 1 << 18;  // 262,144
constexpr int kNaMaxItiles = static_cast<int>(kNaMaxParticles / kNaBI);
// Persistent CTAs: the occupancy limit of the shape (two per SM on GB300), capped
// at four per SM of a 152-SM part; a smaller grid only balances less finely.
constexpr int kNaMaxGrid = 608;
// Bounds of a plan over at most kNaMaxItiles i-tiles on at most kNaMaxGrid CTAs
// (worklist.hpp): every CTA boundary inside an i-tile adds one segment, each
// segment of a split i-tile takes one partial-sum slot, and an i-tile is split
// only by a CTA boundary.
constexpr int kNaMaxSegments = kNaMaxItiles + kNaMaxGrid - 1;
constexpr int kNaMaxSlots = kNaMaxSegments;
constexpr int kNaMaxFixups = kNaMaxItiles < kNaMaxGrid - 1 ? kNaMaxItiles : kNaMaxGrid - 1;
constexpr int kNaMaxDevices = 64;
static_assert(kNaMaxParticles % kNaBI == 0, "whole i-tiles at the maximum size");

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }

constexpr size_t kOffSys = 0;
constexpr size_t kOffErr = 256;
constexpr size_t kOffCounters = 512;
constexpr size_t kOffFix = align256(kOffCounters + sizeof(int32_t) * kNaMaxFixups);
constexpr size_t kOffBegin = align256(kOffFix + sizeof(Fixup) * kNaMaxFixups);
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
Fixup g_na_fix[kNaMaxFixups];

// The fixed host tables as the planner's output (worklist.hpp); refuses to grow.
struct FixedTables {
  int64_t grid = 0;
  int64_t nseg = 0;
  int64_t nfix = 0;
  bool set_grid(int64_t g) {
    grid = g;
    return g >= 1 && g <= kNaMaxGrid;
  }
  bool add_segment(const Segment& sg) {
    if (nseg >= kNaMaxSegments) return false;
    g_na_segs[nseg++] = sg;
    return true;
  }
  Segment& segment(int64_t i) { return g_na_segs[i]; }
  int64_t num_segments() const { return nseg; }
  void set_begin(int64_t cta, int64_t first) { g_na_begin[cta] = static_cast<int32_t>(first); }
  bool add_fixup(const Fixup& f) {
    if (nfix >= kNaMaxFixups) return false;
    g_na_fix[nfix++] = f;
    return true;
  }
  int64_t num_fixups() const { return nfix; }
};

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
    NB_CUDA(force_blocks_per_sm(kNaConfig, false, true, false, &blocks));
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

// The force kernel's stream-K plan (plan_work_into, the rule of every other
// launch) for one system, written into the fixed host tables.  The kernel runs
// every register slot here (no live-slot variant), so the plan is unweighted.  The bounds above
// make it fit for every n <= kNaMaxParticles and grid <= kNaMaxGrid; false if not.
bool na_plan(int32_t n, int32_t npad, int32_t grid_max, int32_t* grid, int32_t* nseg,
             int32_t* nfix, int32_t* nslots) {
  SystemDesc sd{};
  sd.n = n;
  sd.npad = npad;
  FixedTables out;
  int32_t split = 0;
  if (!plan_work_into(&sd, 0, 1, kNaBI, kNaBJ, grid_max, out, nslots, &split)) return false;
  if (*nslots > kNaMaxSlots) return false;
  *grid = static_cast<int32_t>(out.grid);
  *nseg = static_cast<int32_t>(out.nseg);
  *nfix = static_cast<int32_t>(out.nfix);
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
  NB_CUDA(cudaMemsetAsync(base + kOffCounters, 0, sizeof(int32_t) * kNaMaxFixups, st));
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
  a.inject = 0;
  NB_CUDA(launch_force(kNaConfig, false, true, false, a, grid, st));
  int32_t err = 0;
  NB_CUDA(cudaMemcpyAsync(&err, base + kOffErr, sizeof(err), cudaMemcpyDeviceToHost, st));
  NB_CUDA(cudaStreamSynchronize(st));
  if (err != 0)
    return set_error(NB_ERR_DEVICE_TIMEOUT, "a bounded device-side wait timed out");
  return NB_OK;
}
