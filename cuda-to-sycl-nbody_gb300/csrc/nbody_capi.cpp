// Host runtime behind the C ABI (include/nbody_gb300.h).
//
// One nb_sim owns the device state of one or more independent systems, a CUDA
// stream, the work lists of the persistent force kernel and the tile table of
// the reference-order kernel (NB_ACC_REFERENCE_ORDER).  All calls are
// stream-ordered on that stream; the calls that return data to the host
// synchronize it.  Errors are returned as nb_status codes with a thread-local
// message; nothing here exits or throws across the ABI (the reference aborts on
// any CUDA error through gpuErrchk, src/simulator.cuh:22-31).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "nb_internal.hpp"
#include "nb_kernels.hpp"
#include "nb_runtime.hpp"
#include "nbody_gb300.h"
#include "worklist.hpp"

using namespace nbg;

namespace nbg {

thread_local std::string t_last_error;
std::atomic<int> g_alloc_failure_countdown{0};

int set_error(int code, const std::string& msg) {
  t_last_error = msg;
  return code;
}

int cuda_error(cudaError_t e, const char* what) {
  const int code = (e == cudaErrorMemoryAllocation) ? NB_ERR_OUT_OF_MEMORY : NB_ERR_CUDA;
  return set_error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

int check_device(int* sms, cudaDeviceProp* out_prop, int* device) {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return set_error(NB_ERR_NO_DEVICE, std::string("no CUDA device: ") +
                                           (e == cudaSuccess ? "device count is 0"
                                                             : cudaGetErrorString(e)));
  }
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDeviceProperties");
  if (device) *device = dev;
  if (prop.major != 10 || prop.minor != 3)
    return set_error(NB_ERR_NO_DEVICE, std::string("device ") + std::to_string(dev) + " (" +
                                           prop.name + ") is sm_" +
                                           std::to_string(prop.major) +
                                           std::to_string(prop.minor) +
                                           "; this library is built for sm_103a only");
  if (sms) *sms = prop.multiProcessorCount;
  if (out_prop) *out_prop = prop;
  return NB_OK;
}

void free_worklist(WorkListDev& w) {
  dev_free(w.segs);
  dev_free(w.seg_begin);
  dev_free(w.fix);
  w = WorkListDev{};
}

static bool finite_params(const nb_params* p) {
  return std::isfinite(p->G) && std::isfinite(p->dt) && std::isfinite(p->damping) &&
         std::isfinite(p->dist_eps);
}

static int validate_params(const nb_params* p) {
  if (!p) return set_error(NB_ERR_INVALID_ARGUMENT, "params is NULL");
  if (!finite_params(p)) return set_error(NB_ERR_INVALID_ARGUMENT, "params must be finite");
  if (p->dist_eps < 0.f) return set_error(NB_ERR_INVALID_ARGUMENT, "dist_eps must be >= 0");
  if (p->calc_method != NB_BRANCH && p->calc_method != NB_PREDICATED)
    return set_error(NB_ERR_INVALID_ARGUMENT, "calc_method must be NB_BRANCH or NB_PREDICATED");
  if (p->accumulator != NB_ACC_PLAIN && p->accumulator != NB_ACC_COMPENSATED &&
      p->accumulator != NB_ACC_REFERENCE_ORDER)
    return set_error(NB_ERR_INVALID_ARGUMENT,
                     "accumulator must be NB_ACC_PLAIN, NB_ACC_COMPENSATED or "
                     "NB_ACC_REFERENCE_ORDER");
  if (p->iters_per_frame < 0) return set_error(NB_ERR_INVALID_ARGUMENT, "iters_per_frame < 0");
  return NB_OK;
}

// Recompute per-system mass mode and G scale from host masses (user order).
constexpr const char* kReferenceOrderMassError =
    "NB_ACC_REFERENCE_ORDER needs equal masses within each system (the reference has unit "
    "masses)";

// True when the masses (user order) are equal within every system, as the
// reference-order kernel needs.
static bool equal_masses_per_system(const nb_sim* s, const float* mass) {
  for (size_t k = 0; k < s->sys_h.size(); ++k) {
    const int64_t u0 = s->user_offset[k];
    for (int32_t i = 1; i < s->sys_h[k].n; ++i)
      if (mass[u0 + i] != mass[u0]) return false;
  }
  return true;
}

static void assign_mass_mode(nb_sim* s, const std::vector<float>& mass) {
  bool all_equal = true;
  for (size_t k = 0; k < s->sys_h.size(); ++k) {
    const int64_t u0 = s->user_offset[k];
    const int32_t n = s->sys_h[k].n;
    bool eq = true;
    for (int32_t i = 1; i < n && eq; ++i) eq = (mass[u0 + i] == mass[u0]);
    s->sys_h[k].equal_mass = eq ? 1 : 0;
    s->sys_h[k].mass = eq ? mass[u0] : 0.f;
    all_equal = all_equal && eq;
  }
  s->per_pair_mass = !all_equal;
  for (auto& d : s->sys_h) d.gscale = s->per_pair_mass ? s->params.G : s->params.G * d.mass;
}

static int upload_systems(nb_sim* s) {
  NB_CUDA(cudaMemcpyAsync(s->sys_d, s->sys_h.data(), s->sys_h.size() * sizeof(SystemDesc),
                          cudaMemcpyHostToDevice, s->stream));
  return NB_OK;
}

int ensure_staging(nb_sim* s) {
  if (!s->staging_d) NB_TRY(dev_alloc(&s->staging_d, 7 * static_cast<size_t>(s->n_real)));
  return NB_OK;
}

int ensure_accel(nb_sim* s) {
  if (!s->acc_d) NB_TRY(dev_alloc(&s->acc_d, static_cast<size_t>(s->n_pad)));
  return NB_OK;
}

// Upload host SoA state (any of the arrays may be NULL: that component is kept).
static int upload_state(nb_sim* s, const float* const arrays[7], bool with_mass) {
  NB_TRY(ensure_staging(s));
  const size_t n = s->n_real;
  bool partial = false;
  for (int c = 0; c < 6; ++c) partial = partial || (arrays[c] == nullptr);
  if (partial) {
    // Start from the current device state so missing components are preserved.
    NB_CUDA(launch_pack_state(s->pos_d[s->cur], s->vel_d, n, s->map_d, s->staging_d, s->stream));
  }
  for (int c = 0; c < 6; ++c)
    if (arrays[c])
      NB_CUDA(cudaMemcpyAsync(s->staging_d + c * n, arrays[c], n * sizeof(float),
                              cudaMemcpyHostToDevice, s->stream));
  if (with_mass)
    NB_CUDA(cudaMemcpyAsync(s->staging_d + 6 * n, arrays[6], n * sizeof(float),
                            cudaMemcpyHostToDevice, s->stream));
  NB_CUDA(launch_unpack_state(s->staging_d, n, s->map_d, s->pos_d[s->cur], s->vel_d, with_mass,
                              s->stream));
  return NB_OK;
}

// Captured graphs bake in the work lists' and the scratch's device addresses:
// whenever either is replaced, the graphs go too (nb_sim_graph_launch then reports
// that none is captured).
static void drop_graphs(nb_sim* s) {
  for (int b = 0; b < 2; ++b) {
    if (s->gexec[b]) cudaGraphExecDestroy(s->gexec[b]);
    if (s->graph[b]) cudaGraphDestroy(s->graph[b]);
    s->gexec[b] = nullptr;
    s->graph[b] = nullptr;
  }
  s->graph_iters = 0;
}

// Shape of work-list config `cfg` (>= 0: tuned kernel; < 0: reference order).
static KernelShape shape_of(int cfg) {
  return cfg >= 0 ? force_config_shape(cfg) : reference_order_shape(-1 - cfg);
}

static int ensure_scratch(nb_sim* s, const WorkListDev& w) {
  const KernelShape sh = shape_of(w.cfg);
  // Partial sums: (hi, lo) records for the compensated tuned kernel, one record
  // otherwise (the reference-order kernel's hand-over holds one float4 per particle).
  const size_t rec = (w.cfg >= 0 && s->params.accumulator == NB_ACC_COMPENSATED) ? 2 : 1;
  const size_t need = static_cast<size_t>(w.slots) * sh.bi() * rec;
  if (need > s->partials_cap || static_cast<size_t>(w.nfix) > s->counters_cap) drop_graphs(s);
  if (need > s->partials_cap) {
    dev_free(s->partials_d);
    NB_TRY(dev_alloc(&s->partials_d, need));
    s->partials_cap = need;
  }
  if (static_cast<size_t>(w.nfix) > s->counters_cap) {
    dev_free(s->counters_d);
    NB_TRY(dev_alloc(&s->counters_d, static_cast<size_t>(w.nfix)));
    NB_CUDA(cudaMemsetAsync(s->counters_d, 0, w.nfix * sizeof(int32_t), s->stream));
    s->counters_cap = w.nfix;
  }
  return NB_OK;
}

static int max_grid_for(nb_sim* s, int cfg, bool live = false) {
  int blocks = 0;
  const bool comp = s->params.accumulator == NB_ACC_COMPENSATED;
  const cudaError_t e =
      cfg >= 0 ? force_blocks_per_sm(cfg, comp, s->per_pair_mass, live, &blocks)
               : reference_order_blocks_per_sm(-1 - cfg, s->params.calc_method == NB_PREDICATED,
                                               &blocks);
  if (e != cudaSuccess || blocks < 1) blocks = 1;
  return blocks * s->sms;
}

static int upload_worklist(nb_sim* s, const WorkListHost& h, int cfg, WorkListDev* out) {
  WorkListDev w;
  w.cfg = cfg;
  w.grid = h.grid;
  w.nseg = static_cast<int32_t>(h.segs.size());
  w.nfix = static_cast<int32_t>(h.fix.size());
  w.slots = h.slots;
  w.split = h.split_tiles;
  int st = dev_alloc(&w.segs, h.segs.size());
  if (st == NB_OK) st = dev_alloc(&w.seg_begin, h.seg_begin.size());
  if (st == NB_OK) st = dev_alloc(&w.fix, std::max<size_t>(1, h.fix.size()));
  if (st != NB_OK) {
    free_worklist(w);
    return st;
  }
  cudaError_t e = cudaMemcpyAsync(w.segs, h.segs.data(), h.segs.size() * sizeof(Segment),
                                  cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(w.seg_begin, h.seg_begin.data(), h.seg_begin.size() * sizeof(int32_t),
                        cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess && !h.fix.empty())
    e = cudaMemcpyAsync(w.fix, h.fix.data(), h.fix.size() * sizeof(Fixup),
                        cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);  // host vectors die on return
  if (e != cudaSuccess) {
    free_worklist(w);
    return cuda_error(e, "upload work list");
  }
  st = ensure_scratch(s, w);
  if (st != NB_OK) {
    free_worklist(w);
    return st;
  }
  *out = w;
  return NB_OK;
}

// Plan systems [first, first + count) for tuned-kernel config `cfg` on at most
// `grid` CTAs (0: the occupancy limit), with the live-slot variant where it pays.
static int plan_tuned(nb_sim* s, int cfg, int32_t first, int32_t count, int grid,
                      WorkListDev* out) {
  const KernelShape sh = force_config_shape(cfg);
  const bool live = live_slots_pay(s->sys_h.data(), first, count, sh.threads, sh.r);
  if (grid <= 0) grid = max_grid_for(s, cfg, live);
  const WorkListHost h = plan_worklist(s->sys_h.data(), first, count, sh.bi(), sh.bj, grid,
                                       live ? sh.threads : 0, sh.r);
  NB_TRY(upload_worklist(s, h, cfg, out));
  out->live = live;
  return NB_OK;
}

// (Re)build the all-systems work list for kernel config `cfg`.
static int build_main_worklist(nb_sim* s, int cfg) {
  WorkListDev w;
  NB_TRY(plan_tuned(s, cfg, 0, static_cast<int32_t>(s->sys_h.size()), 0, &w));
  drop_graphs(s);
  free_worklist(s->wl);
  s->wl = w;
  return NB_OK;
}

static int default_config_for(nb_sim* s, int32_t first, int32_t count);
static int default_reference_order_for(nb_sim* s, int32_t first, int32_t count);

static bool reference_order_mode(const nb_sim* s) {
  return s->params.calc_method == NB_BRANCH && s->params.accumulator == NB_ACC_REFERENCE_ORDER;
}

// The modes that run the sequential-order kernel (reference_order_kernel.cu): the
// reference-order accumulator, and PREDICATED, whose equal-mass systems run that
// kernel with the PREDICATED pair term (per-particle masses keep the one-thread-
// per-particle kernel, aux_kernels.cu).
static bool sequential_order_mode(const nb_sim* s) {
  return reference_order_mode(s) || s->params.calc_method == NB_PREDICATED;
}

// (Re)build the reference-order work list for shape `shape` (all systems).
static int reference_order_grid(nb_sim* s, int shape, int32_t first, int32_t count);

static int build_reference_order_worklist(nb_sim* s, int shape) {
  const int cfg = -1 - shape;
  const KernelShape sh = reference_order_shape(shape);
  const int32_t nsys = static_cast<int32_t>(s->sys_h.size());
  const WorkListHost h = plan_worklist(s->sys_h.data(), 0, nsys, sh.bi(), sh.bj,
                                       reference_order_grid(s, shape, 0, nsys));
  WorkListDev w;
  NB_TRY(upload_worklist(s, h, cfg, &w));
  drop_graphs(s);
  free_worklist(s->ro_wl);
  s->ro_wl = w;
  return NB_OK;
}

// One work list per system for the one-launch-per-system baseline.  Policy
// kPerSystemOwnShape plans each system with the shape it would get as a
// simulation of its own (default_config_for / default_reference_order_for), the
// way a caller launching each system separately would; kPerSystemSimShape gives
// every system the simulation's current shape.
static int build_per_system_worklists(nb_sim* s, int policy) {
  const bool ro = sequential_order_mode(s);
  const int sim_cfg = ro ? -1 - s->ro_shape : s->cfg;
  if (s->wl_sys_policy == policy && (policy == kPerSystemOwnShape || s->wl_sys_cfg == sim_cfg) &&
      s->wl_sys.size() == s->sys_h.size())
    return NB_OK;
  for (auto& w : s->wl_sys) free_worklist(w);
  s->wl_sys.clear();
  s->wl_sys_policy = -1;
  for (int32_t k = 0; k < static_cast<int32_t>(s->sys_h.size()); ++k) {
    int cfg = sim_cfg;
    if (policy == kPerSystemOwnShape)
      cfg = ro ? -1 - default_reference_order_for(s, k, 1) : default_config_for(s, k, 1);
    WorkListDev w;
    if (cfg >= 0) {
      NB_TRY(plan_tuned(s, cfg, k, 1, 0, &w));
    } else {
      const KernelShape sh = shape_of(cfg);
      const WorkListHost h = plan_worklist(s->sys_h.data(), k, 1, sh.bi(), sh.bj,
                                           reference_order_grid(s, -1 - cfg, k, 1));
      NB_TRY(upload_worklist(s, h, cfg, &w));
    }
    s->wl_sys.push_back(w);
  }
  s->wl_sys_policy = policy;
  s->wl_sys_cfg = sim_cfg;
  return NB_OK;
}

// The duplicated j-layout buffer of the reference-order kernel.
static int ensure_reference_order_dup(nb_sim* s) {
  if (!s->ro_dup_d) NB_TRY(dev_alloc(&s->ro_dup_d, 2 * static_cast<size_t>(s->n_pad)));
  return NB_OK;
}

ForceArgs base_args(nb_sim* s) {
  ForceArgs a{};
  a.pos = s->pos_d[s->cur];
  a.pos_next = s->pos_d[s->cur ^ 1];
  a.vel = s->vel_d;
  a.accel_out = nullptr;
  a.sys = s->sys_d;
  a.partials = s->partials_d;
  a.counters = s->counters_d;
  a.err = s->err_d;
  a.eps2 = s->params.dist_eps;
  a.dt = s->params.dt;
  a.damping = s->params.damping;
  a.mask_self = s->mask_self;
  a.inject = 0;
  return a;
}

int launch_with(nb_sim* s, ForceArgs a, const WorkListDev& w) {
  a.inject = s->inject;
  s->inject = 0;
  a.segs = w.segs;
  a.seg_begin = w.seg_begin;
  a.fix = w.fix;
  if (w.cfg < 0) {
    // Sequential order: the duplicated layout of a.pos must have been written.
    NB_CUDA(launch_reference_order(-1 - w.cfg, s->params.calc_method == NB_PREDICATED, a,
                                   s->ro_dup_d, w.grid, s->stream));
    return NB_OK;
  }
  NB_CUDA(launch_force(w.cfg, s->params.accumulator == NB_ACC_COMPENSATED, s->per_pair_mass,
                       w.live, a, w.grid, s->stream));
  return NB_OK;
}

// One force evaluation: integrate into the other buffer (accel_out == nullptr)
// or write accelerations.  `per_system` (kPerSystem*) issues one launch per system.
int force_pass(nb_sim* s, float4* accel_out, int per_system) {
  ForceArgs a = base_args(s);
  a.accel_out = accel_out;
  if (s->params.calc_method == NB_PREDICATED && s->per_pair_mass) {
    for (int32_t k = 0; k < static_cast<int32_t>(s->sys_h.size()); ++k)
      NB_CUDA(launch_predicated(a, s->sys_h[k], k, s->stream));
  } else if (sequential_order_mode(s)) {
    if (s->per_pair_mass) return set_error(NB_ERR_INVALID_ARGUMENT, kReferenceOrderMassError);
    NB_TRY(ensure_reference_order_dup(s));
    NB_CUDA(launch_reference_order_dup(a.pos, s->n_pad, s->ro_dup_d, s->stream));
    if (per_system) {
      NB_TRY(build_per_system_worklists(s, per_system));
      for (const auto& w : s->wl_sys) NB_TRY(launch_with(s, a, w));
    } else {
      NB_TRY(launch_with(s, a, s->ro_wl));
    }
  } else if (per_system) {
    NB_TRY(build_per_system_worklists(s, per_system));
    for (const auto& w : s->wl_sys) NB_TRY(launch_with(s, a, w));
  } else {
    NB_TRY(launch_with(s, a, s->wl));
  }
  if (!accel_out) s->cur ^= 1;  // std::swap(pos_d, pos_next_d), simulator.cu:65
  return NB_OK;
}

int check_error_word(nb_sim* s) {
  int32_t err = 0;
  NB_CUDA(cudaMemcpyAsync(&err, s->err_d, sizeof(err), cudaMemcpyDeviceToHost, s->stream));
  NB_CUDA(cudaStreamSynchronize(s->stream));
  if (err != 0) {
    // CTAs that gave up never arrived on their fixup counters: clear them.
    NB_CUDA(cudaMemsetAsync(s->err_d, 0, sizeof(int32_t), s->stream));
    if (s->counters_d)
      NB_CUDA(cudaMemsetAsync(s->counters_d, 0, s->counters_cap * sizeof(int32_t), s->stream));
    NB_CUDA(cudaStreamSynchronize(s->stream));
    return set_error(NB_ERR_DEVICE_TIMEOUT,
                     "a bounded device-side wait timed out (error word " + std::to_string(err) +
                         "); results of that launch are invalid");
  }
  return NB_OK;
}

// Default kernel shape: the one with the largest tiles whose work list still gives
// every CTA at least 16 (i-tile, j-tile) blocks, so that the stream-K split balances
// to within a few percent; the smallest shape otherwise.  Deterministic (the
// autotuner may pick otherwise, and shapes round differently).  Measured against
// the autotuner's pick: N = 25,600 -> 256 x 2 x 256 (0.24 ms, the 1M shape takes
// 0.32), 65,536 -> 256 x 4 x 1024, 262,144 and 1M -> 256 x 4 x 2048.
// default_config_for judges systems [first, first + count) alone.
static int default_config_for(nb_sim* s, int32_t first, int32_t count) {
  static const int kCandidates[] = {9, 8, 10, 3, 4};  // largest tiles first
  for (const int cfg : kCandidates) {
    const KernelShape sh = force_config_shape(cfg);
    int64_t blocks = 0;
    for (int32_t k = first; k < first + count; ++k) {
      const SystemDesc& d = s->sys_h[k];
      const int64_t i_tiles = (d.n + sh.bi() - 1) / sh.bi();
      blocks += i_tiles * ((d.npad + sh.bj - 1) / sh.bj);
    }
    if (blocks >= 16 * static_cast<int64_t>(max_grid_for(s, cfg))) return cfg;
  }
  return 4;
}

static int default_config(nb_sim* s) {
  return default_config_for(s, 0, static_cast<int32_t>(s->sys_h.size()));
}

// i-tiles of reference-order shape `shape` over systems [first, first + count).
static int64_t reference_order_tiles(const nb_sim* s, int shape, int32_t first, int32_t count) {
  const int bi = reference_order_shape(shape).bi();
  int64_t tiles = 0;
  for (int32_t q = first; q < first + count; ++q) tiles += (s->sys_h[q].n + bi - 1) / bi;
  return tiles;
}

// Grid of the reference-order kernel: one CTA per i-tile while every CTA fits
// on the GPU at once, else the occupancy limit on every SM with the stream-K work
// list.  A CTA's share is then at least one whole i-tile, so a hand-over chain is
// never longer than two parts (a particle's sum is sequential: a longer chain
// would only run its parts one after another).
static int reference_order_grid(nb_sim* s, int shape, int32_t first, int32_t count) {
  const int64_t tiles = reference_order_tiles(s, shape, first, count);
  return static_cast<int>(std::max<int64_t>(
      1, std::min<int64_t>(tiles, max_grid_for(s, -1 - shape))));
}

// Default reference-order shape: the largest i-tiles that still fill the GPU --
// at least two CTAs per SM, or one where a single CTA is all that fits on an SM;
// the smallest shape (the most particles summed at once) when none does.
static int default_reference_order_for(nb_sim* s, int32_t first, int32_t count) {
  const int last = reference_order_num_shapes() - 1;
  for (int k = 0; k < last; ++k) {
    const int64_t per_sm = std::min<int64_t>(2, max_grid_for(s, -1 - k) / s->sms);
    if (reference_order_tiles(s, k, first, count) >= per_sm * s->sms) return k;
  }
  return last;
}

static int create_impl(const nb_params* p, uint32_t num_systems, const uint32_t* sizes,
                       const float* x, const float* y, const float* z, const float* vx,
                       const float* vy, const float* vz, const float* mass, nb_sim** out) {
  if (!out) return set_error(NB_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  NB_TRY(validate_params(p));
  if (num_systems == 0 || !sizes) return set_error(NB_ERR_INVALID_ARGUMENT, "no systems");
  if (!x || !y || !z || !vx || !vy || !vz)
    return set_error(NB_ERR_INVALID_ARGUMENT, "state arrays must not be NULL");
  uint64_t total = 0;
  for (uint32_t k = 0; k < num_systems; ++k) {
    if (sizes[k] == 0) return set_error(NB_ERR_INVALID_ARGUMENT, "a system has 0 particles");
    if (sizes[k] > (1u << 30))
      return set_error(NB_ERR_INVALID_ARGUMENT, "a system has more than 2^30 particles");
    total += sizes[k];
  }
  if (total != p->num_particles)
    return set_error(NB_ERR_INVALID_ARGUMENT,
                     "num_particles (" + std::to_string(p->num_particles) +
                         ") differs from the sum of system sizes (" + std::to_string(total) + ")");
  int sms = 0, device = 0;
  cudaDeviceProp prop;
  NB_TRY(check_device(&sms, &prop, &device));

  nb_sim* s = new (std::nothrow) nb_sim();
  if (!s) return set_error(NB_ERR_OUT_OF_MEMORY, "host allocation failed");
  s->params = *p;
  s->device = device;
  s->sms = sms;
  s->device_name = prop.name;
  s->n_real = total;
  int64_t off = 0, uoff = 0;
  for (uint32_t k = 0; k < num_systems; ++k) {
    SystemDesc d{};
    d.offset = off;
    d.n = static_cast<int32_t>(sizes[k]);
    d.npad = static_cast<int32_t>((sizes[k] + kPadQuantum - 1) / kPadQuantum * kPadQuantum);
    d.shard_first = 0;
    d.shard_count = 0;  // the whole system
    s->sys_h.push_back(d);
    s->user_offset.push_back(uoff);
    off += d.npad;
    uoff += sizes[k];
  }
  s->n_pad = off;
  {
    const float e = p->dist_eps;
    const float e3 = e * e * e;
    s->mask_self = (e3 >= FLT_MIN) ? 0 : 1;  // eps^3 flushes to zero on the device
  }
  std::vector<float> m(total, 1.0f);
  if (mass) std::copy(mass, mass + total, m.begin());
  assign_mass_mode(s, m);
  if (p->accumulator == NB_ACC_REFERENCE_ORDER && s->per_pair_mass) {
    delete s;  // nothing on the device yet
    return set_error(NB_ERR_INVALID_ARGUMENT, kReferenceOrderMassError);
  }

  int st = NB_OK;
  auto fail = [&](int code) {
    nb_sim_destroy(s);
    return code;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(cuda_error(e, "cudaStreamCreate"));
  s->own_stream = true;
  if ((e = cudaEventCreate(&s->ev0)) != cudaSuccess ||
      (e = cudaEventCreate(&s->ev1)) != cudaSuccess)
    return fail(cuda_error(e, "cudaEventCreate"));
  if ((st = dev_alloc(&s->sys_d, s->sys_h.size())) != NB_OK) return fail(st);
  if ((st = dev_alloc(&s->pos_d[0], 4 * static_cast<size_t>(s->n_pad))) != NB_OK) return fail(st);
  if ((st = dev_alloc(&s->pos_d[1], 4 * static_cast<size_t>(s->n_pad))) != NB_OK) return fail(st);
  if ((st = dev_alloc(&s->vel_d, static_cast<size_t>(s->n_pad))) != NB_OK) return fail(st);
  if ((st = dev_alloc(&s->err_d, 1)) != NB_OK) return fail(st);
  if ((e = cudaMemsetAsync(s->err_d, 0, sizeof(int32_t), s->stream)) != cudaSuccess)
    return fail(cuda_error(e, "cudaMemset"));
  if (num_systems > 1) {
    std::vector<int64_t> map(total);
    for (uint32_t k = 0; k < num_systems; ++k)
      for (uint32_t i = 0; i < sizes[k]; ++i)
        map[s->user_offset[k] + i] = s->sys_h[k].offset + i;
    if ((st = dev_alloc(&s->map_d, total)) != NB_OK) return fail(st);
    if ((e = cudaMemcpy(s->map_d, map.data(), total * sizeof(int64_t), cudaMemcpyHostToDevice)) !=
        cudaSuccess)
      return fail(cuda_error(e, "upload map"));
  }
  if ((st = upload_systems(s)) != NB_OK) return fail(st);
  for (int b = 0; b < 2; ++b)
    if ((e = launch_fill_padding(s->pos_d[b], s->vel_d, s->n_pad, s->stream)) != cudaSuccess)
      return fail(cuda_error(e, "fill padding"));
  const float* arrays[7] = {x, y, z, vx, vy, vz, m.data()};
  if ((st = upload_state(s, arrays, true)) != NB_OK) return fail(st);
  // The mass component of the other buffer is rewritten by every step; set it now
  // so that a first accelerations call after a swap sees it too.
  if ((e = cudaMemcpyAsync(s->pos_d[1], s->pos_d[0], 4 * sizeof(float) * s->n_pad,
                           cudaMemcpyDeviceToDevice, s->stream)) != cudaSuccess)
    return fail(cuda_error(e, "copy state"));
  s->cfg = default_config(s);
  if ((st = build_main_worklist(s, s->cfg)) != NB_OK) return fail(st);
  if (sequential_order_mode(s)) {
    s->ro_shape = default_reference_order_for(s, 0, static_cast<int32_t>(s->sys_h.size()));
    if ((st = build_reference_order_worklist(s, s->ro_shape)) != NB_OK) return fail(st);
    if ((st = ensure_reference_order_dup(s)) != NB_OK) return fail(st);
  }
  if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return fail(cuda_error(e, "create"));
  *out = s;
  return NB_OK;
}

}  // namespace nbg

// ============================== C ABI =========================================

extern "C" {

const char* nb_last_error(void) { return t_last_error.c_str(); }

const char* nb_status_string(int status) {
  switch (status) {
    case NB_OK: return "NB_OK";
    case NB_ERR_INVALID_ARGUMENT: return "NB_ERR_INVALID_ARGUMENT";
    case NB_ERR_CUDA: return "NB_ERR_CUDA";
    case NB_ERR_OUT_OF_MEMORY: return "NB_ERR_OUT_OF_MEMORY";
    case NB_ERR_NO_DEVICE: return "NB_ERR_NO_DEVICE";
    case NB_ERR_DEVICE_TIMEOUT: return "NB_ERR_DEVICE_TIMEOUT";
    case NB_ERR_STATE: return "NB_ERR_STATE";
    default: return "unknown status";
  }
}

int nb_abi_version(void) { return NB_ABI_VERSION; }

void nb_params_default(nb_params* p) {
  if (!p) return;
  // SimParam::SimParam (sim_param.cpp:12-22)
  p->G = 2.0f;
  p->dt = 0.005f;
  p->num_particles = 50 * 256;
  p->num_frames = SIZE_MAX;
  p->iters_per_frame = 4;
  p->damping = 0.999998f;
  p->dist_eps = 1.0e-7f;
  p->gw_size = 64;
  p->calc_method = NB_BRANCH;
  p->accumulator = NB_ACC_COMPENSATED;  // faster than plain at the default shape, and ~200x
                                        // more accurate at N = 1M
}

int nb_params_parse_args(nb_params* p, int argc, const char* const* argv) {
  if (!p) return set_error(NB_ERR_INVALID_ARGUMENT, "params is NULL");
  if (argc > 1 && !argv) return set_error(NB_ERR_INVALID_ARGUMENT, "argv is NULL");
  // SimParam::parseArgs (sim_param.cpp:40-67): positional, atoi/atof semantics.
  if (argc >= 2) {
    const long long b = std::atoll(argv[1]);
    if (b < 0) return set_error(NB_ERR_INVALID_ARGUMENT, "number of batches must be >= 0");
    p->num_particles = static_cast<uint64_t>(256 * b);
  }
  if (argc >= 3) p->iters_per_frame = std::atoi(argv[2]);
  if (argc >= 4) p->damping = static_cast<float>(std::atof(argv[3]));
  if (argc >= 5) p->dt = static_cast<float>(std::atof(argv[4]));
  if (argc >= 6) p->dist_eps = static_cast<float>(std::atof(argv[5]));
  if (argc >= 7) p->G = static_cast<float>(std::atof(argv[6]));
  if (argc >= 8) p->num_frames = static_cast<uint64_t>(std::atoll(argv[7]));
  if (argc >= 9) p->gw_size = std::atoi(argv[8]);
  if (argc >= 10) {
    const std::string m = argv[9];
    if (m == "BRANCH")
      p->calc_method = NB_BRANCH;
    else if (m == "PREDICATED")
      p->calc_method = NB_PREDICATED;
    else
      return set_error(NB_ERR_INVALID_ARGUMENT,
                       "Valid calculation methods are BRANCH or PREDICATED");
  }
  return NB_OK;
}

int nb_device_name(char* buf, size_t len) {
  if (!buf || len == 0) return set_error(NB_ERR_INVALID_ARGUMENT, "empty buffer");
  cudaDeviceProp prop;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    // getDeviceName falls back to "Unknown Device" (simulator.cu:41).
    std::snprintf(buf, len, "%s", "Unknown Device");
    return set_error(NB_ERR_NO_DEVICE, "no CUDA device");
  }
  int dev = 0;
  NB_CUDA(cudaGetDevice(&dev));
  NB_CUDA(cudaGetDeviceProperties(&prop, dev));
  std::snprintf(buf, len, "%s", prop.name);
  return NB_OK;
}

int nb_device_fp32_peak_tflops(double* tflops) {
  if (!tflops) return set_error(NB_ERR_INVALID_ARGUMENT, "out is NULL");
  int sms = 0;
  cudaDeviceProp prop;
  NB_TRY(check_device(&sms, &prop));
  int clock_khz = 0, dev = 0;
  NB_CUDA(cudaGetDevice(&dev));
  NB_CUDA(cudaDeviceGetAttribute(&clock_khz, cudaDevAttrClockRate, dev));
  *tflops = static_cast<double>(sms) * 128.0 * 2.0 * clock_khz * 1e3 / 1e12;
  return NB_OK;
}

int nb_measure_fp32_peak_tflops(double* tflops) {
  if (!tflops) return set_error(NB_ERR_INVALID_ARGUMENT, "out is NULL");
  int sms = 0;
  cudaDeviceProp prop;
  NB_TRY(check_device(&sms, &prop));
  constexpr int kBlocksPerSm = 4, kIters = 4096, kRepeats = 20;
  float2* scratch = nullptr;
  NB_TRY(dev_alloc(&scratch, static_cast<size_t>(sms) * kBlocksPerSm * fp32_peak_threads()));
  float ms = 0.f;
  const cudaError_t e =
      measure_fp32_peak(sms, scratch, kBlocksPerSm, kIters, kRepeats, nullptr, tflops, &ms);
  dev_free(scratch);
  if (e != cudaSuccess) return cuda_error(e, "measure_fp32_peak");
  return NB_OK;
}

int nb_sim_create(const nb_params* p, const float* x, const float* y, const float* z,
                  const float* vx, const float* vy, const float* vz, const float* mass,
                  nb_sim** out) {
  if (!p) return set_error(NB_ERR_INVALID_ARGUMENT, "params is NULL");
  if (p->num_particles == 0 || p->num_particles > (1ull << 30))
    return set_error(NB_ERR_INVALID_ARGUMENT, "num_particles must be in [1, 2^30]");
  const uint32_t n = static_cast<uint32_t>(p->num_particles);
  return create_impl(p, 1, &n, x, y, z, vx, vy, vz, mass, out);
}

int nb_sim_create_disk_galaxy(const nb_params* p, nb_sim** out) {
  if (!p) return set_error(NB_ERR_INVALID_ARGUMENT, "params is NULL");
  if (p->num_particles == 0 || p->num_particles > (1ull << 30))
    return set_error(NB_ERR_INVALID_ARGUMENT, "num_particles must be in [1, 2^30]");
  const size_t n = p->num_particles;
  std::vector<float> buf(6 * n);
  float* b = buf.data();
  NB_TRY(nb_ic_reference_disk(n, b, b + n, b + 2 * n, b + 3 * n, b + 4 * n, b + 5 * n));
  return nb_sim_create(p, b, b + n, b + 2 * n, b + 3 * n, b + 4 * n, b + 5 * n, nullptr, out);
}

int nb_ensemble_create(const nb_params* p, uint32_t num_systems, const uint32_t* sizes,
                       const float* x, const float* y, const float* z, const float* vx,
                       const float* vy, const float* vz, const float* mass, nb_sim** out) {
  return create_impl(p, num_systems, sizes, x, y, z, vx, vy, vz, mass, out);
}

int nb_sim_destroy(nb_sim* s) {
  if (!s) return NB_OK;
  DeviceGuard dg_(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (int b = 0; b < 2; ++b) {
    if (s->gexec[b]) cudaGraphExecDestroy(s->gexec[b]);
    if (s->graph[b]) cudaGraphDestroy(s->graph[b]);
  }
  free_worklist(s->wl);
  for (auto& w : s->wl_sys) free_worklist(w);
  dev_free(s->sys_d);
  dev_free(s->map_d);
  dev_free(s->pos_d[0]);
  dev_free(s->pos_d[1]);
  dev_free(s->vel_d);
  dev_free(s->acc_d);
  dev_free(s->staging_d);
  dev_free(s->err_d);
  dev_free(s->partials_d);
  dev_free(s->counters_d);
  free_worklist(s->ro_wl);
  dev_free(s->ro_dup_d);
  release_aux(s);
  release_render_buffers(s);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return NB_OK;
}

int nb_sim_advance(nb_sim* s, int32_t iterations) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  if (iterations < 0) return set_error(NB_ERR_INVALID_ARGUMENT, "iterations < 0");
  for (int32_t k = 0; k < iterations; ++k) NB_TRY(force_pass(s, nullptr, kPerSystemNone));
  return NB_OK;
}

int nb_sim_advance_per_system(nb_sim* s, int32_t iterations) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  if (iterations < 0) return set_error(NB_ERR_INVALID_ARGUMENT, "iterations < 0");
  for (int32_t k = 0; k < iterations; ++k)
    NB_TRY(force_pass(s, nullptr, kPerSystemOwnShape));
  return NB_OK;
}

int nb_inject_alloc_failure(int32_t nth) {
  if (nth < 0) return set_error(NB_ERR_INVALID_ARGUMENT, "nth must be >= 0");
  g_alloc_failure_countdown.store(nth);
  return NB_OK;
}

int nb_sim_synchronize(nb_sim* s) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  NB_CUDA(cudaStreamSynchronize(s->stream));
  return check_error_word(s);
}

int nb_sim_time_iterations(nb_sim* s, int32_t iterations, int32_t per_system, float* ms) {
  if (!s || !ms) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard dg_(s->device);
  if (iterations < 0) return set_error(NB_ERR_INVALID_ARGUMENT, "iterations < 0");
  if (per_system != kPerSystemNone && per_system != kPerSystemOwnShape &&
      per_system != kPerSystemSimShape)
    return set_error(NB_ERR_INVALID_ARGUMENT, "per_system must be 0, 1 or 2");
  if (per_system && s->params.calc_method == NB_BRANCH &&
      s->params.accumulator != NB_ACC_REFERENCE_ORDER)
    NB_TRY(build_per_system_worklists(s, per_system));
  NB_CUDA(cudaEventRecord(s->ev0, s->stream));
  for (int32_t k = 0; k < iterations; ++k) NB_TRY(force_pass(s, nullptr, per_system));
  NB_CUDA(cudaEventRecord(s->ev1, s->stream));
  NB_CUDA(cudaEventSynchronize(s->ev1));
  NB_CUDA(cudaEventElapsedTime(ms, s->ev0, s->ev1));
  return check_error_word(s);
}

int nb_sim_step(nb_sim* s) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  // stepSim (simulator.cu:47-75): the reference times launch-to-sync with a host
  // clock; here the same region is timed with CUDA events on the stream.
  float ms = 0.f;
  NB_TRY(nb_sim_time_iterations(s, s->params.iters_per_frame, 0, &ms));
  s->last_ms = ms;
  return NB_OK;
}

int nb_sim_get_state(nb_sim* s, float* x, float* y, float* z, float* vx, float* vy, float* vz) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  NB_TRY(ensure_staging(s));
  const size_t n = s->n_real;
  NB_CUDA(launch_pack_state(s->pos_d[s->cur], s->vel_d, n, s->map_d, s->staging_d, s->stream));
  float* outs[6] = {x, y, z, vx, vy, vz};
  for (int c = 0; c < 6; ++c)
    if (outs[c])
      NB_CUDA(cudaMemcpyAsync(outs[c], s->staging_d + c * n, n * sizeof(float),
                              cudaMemcpyDeviceToHost, s->stream));
  NB_CUDA(cudaStreamSynchronize(s->stream));
  return check_error_word(s);
}

int nb_sim_set_state(nb_sim* s, const float* x, const float* y, const float* z, const float* vx,
                     const float* vy, const float* vz, const float* mass) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  if (mass && s->params.accumulator == NB_ACC_REFERENCE_ORDER &&
      !equal_masses_per_system(s, mass))
    return set_error(NB_ERR_INVALID_ARGUMENT, kReferenceOrderMassError);  // state unchanged
  if (mass) {
    std::vector<float> m(mass, mass + s->n_real);
    assign_mass_mode(s, m);
    NB_TRY(upload_systems(s));
  }
  const float* arrays[7] = {x, y, z, vx, vy, vz, mass};
  NB_TRY(upload_state(s, arrays, mass != nullptr));
  if (mass) {
    // Both buffers carry the masses (the step copies them forward).
    NB_CUDA(cudaMemcpyAsync(s->pos_d[s->cur ^ 1], s->pos_d[s->cur],
                            4 * sizeof(float) * s->n_pad, cudaMemcpyDeviceToDevice, s->stream));
  }
  NB_CUDA(cudaStreamSynchronize(s->stream));
  return NB_OK;
}

int nb_sim_accelerations(nb_sim* s, float* ax, float* ay, float* az) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  NB_TRY(ensure_accel(s));
  NB_TRY(ensure_staging(s));
  NB_TRY(force_pass(s, s->acc_d, kPerSystemNone));
  const size_t n = s->n_real;
  NB_CUDA(launch_pack_accel(s->acc_d, n, s->map_d, s->staging_d, s->stream));
  float* outs[3] = {ax, ay, az};
  for (int c = 0; c < 3; ++c)
    if (outs[c])
      NB_CUDA(cudaMemcpyAsync(outs[c], s->staging_d + c * n, n * sizeof(float),
                              cudaMemcpyDeviceToHost, s->stream));
  NB_CUDA(cudaStreamSynchronize(s->stream));
  return check_error_word(s);
}

int nb_sim_num_particles(const nb_sim* s, uint64_t* n) {
  if (!s || !n) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = s->n_real;
  return NB_OK;
}

int nb_sim_num_systems(const nb_sim* s, uint32_t* n) {
  if (!s || !n) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = static_cast<uint32_t>(s->sys_h.size());
  return NB_OK;
}

int nb_sim_last_step_ms(const nb_sim* s, float* ms) {
  if (!s || !ms) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  *ms = s->last_ms;
  return NB_OK;
}

int nb_sim_gw_size(const nb_sim* s, int32_t* gw) {
  if (!s || !gw) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  *gw = s->params.gw_size;
  return NB_OK;
}

int nb_sim_calc_method(const nb_sim* s, int32_t* method) {
  if (!s || !method) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  *method = s->params.calc_method;
  return NB_OK;
}

int nb_sim_set_stream(nb_sim* s, void* stream) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  NB_CUDA(cudaStreamSynchronize(s->stream));
  if (s->own_stream) cudaStreamDestroy(s->stream);
  s->own_stream = false;
  s->stream = static_cast<cudaStream_t>(stream);
  return NB_OK;
}

int nb_sim_export_device(nb_sim* s, float* pos_xyzm_device, float* vel_xyzw_device) {
  if (!s || !pos_xyzm_device) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard dg_(s->device);
  if ((reinterpret_cast<uintptr_t>(pos_xyzm_device) & 15) ||
      (reinterpret_cast<uintptr_t>(vel_xyzw_device) & 15))
    return set_error(NB_ERR_INVALID_ARGUMENT, "device buffers must be 16-byte aligned");
  NB_CUDA(launch_export(s->pos_d[s->cur], s->vel_d, s->n_real, s->map_d,
                        reinterpret_cast<float4*>(pos_xyzm_device),
                        reinterpret_cast<float4*>(vel_xyzw_device), s->stream));
  return NB_OK;
}

int nb_num_kernel_configs(void) { return num_force_configs(); }

int nb_kernel_config_info(int32_t index, nb_kernel_info* info) {
  if (!info || index < -reference_order_num_shapes() || index >= num_force_configs())
    return set_error(NB_ERR_INVALID_ARGUMENT, "bad config index");
  const KernelShape sh = index >= 0 ? force_config_shape(index) : reference_order_shape(-1 - index);
  *info = nb_kernel_info{index, sh.threads, sh.r, sh.bj, sh.stages, 0, 0, 0, 0};
  return NB_OK;
}

int nb_sim_set_kernel_config(nb_sim* s, int32_t index) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  if (sequential_order_mode(s)) {
    // The reference-order kernel's shapes: index 0 .. reference-order shapes - 1.
    if (index < -1 || index >= reference_order_num_shapes())
      return set_error(NB_ERR_INVALID_ARGUMENT, "bad reference-order shape index");
    const int shape =
        index < 0 ? default_reference_order_for(s, 0, static_cast<int32_t>(s->sys_h.size()))
                  : index;
    NB_TRY(build_reference_order_worklist(s, shape));
    s->ro_shape = shape;
    return NB_OK;
  }
  if (index < -1 || index >= num_force_configs())
    return set_error(NB_ERR_INVALID_ARGUMENT, "bad config index");
  const int cfg = index < 0 ? default_config(s) : index;
  NB_TRY(build_main_worklist(s, cfg));
  s->cfg = cfg;
  return NB_OK;
}

int nb_sim_kernel_info(const nb_sim* s, nb_kernel_info* info) {
  if (!s || !info) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  if (sequential_order_mode(s)) {
    const KernelShape sh = reference_order_shape(s->ro_shape);
    *info = nb_kernel_info{-1 - s->ro_shape, sh.threads, sh.r, sh.bj, sh.stages,
                           s->ro_wl.grid, s->ro_wl.nseg, s->ro_wl.split, 0};
    return NB_OK;
  }
  const KernelShape sh = force_config_shape(s->cfg);
  *info = nb_kernel_info{s->cfg, sh.threads, sh.r, sh.bj, sh.stages,
                         s->wl.grid, s->wl.nseg, s->wl.split, s->wl.live ? 1 : 0};
  return NB_OK;
}

int nb_sim_autotune(nb_sim* s, int32_t* chosen) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  if (s->params.calc_method == NB_PREDICATED) {
    // The compatibility mode keeps its default shape: nothing to choose.
    if (chosen) *chosen = -1 - s->ro_shape;
    return NB_OK;
  }
  NB_TRY(ensure_accel(s));
  if (s->params.accumulator == NB_ACC_REFERENCE_ORDER) {
    // Time the reference-order shapes (accelerations only; every shape gives the
    // same bits) and keep the fastest.
    int best = s->ro_shape;
    float best_ms = 1e30f;
    for (int k = 0; k < reference_order_num_shapes(); ++k) {
      s->ro_shape = k;
      NB_TRY(build_reference_order_worklist(s, k));
      NB_TRY(force_pass(s, s->acc_d, kPerSystemNone));  // warm-up
      NB_CUDA(cudaEventRecord(s->ev0, s->stream));
      NB_TRY(force_pass(s, s->acc_d, kPerSystemNone));
      NB_CUDA(cudaEventRecord(s->ev1, s->stream));
      NB_CUDA(cudaEventSynchronize(s->ev1));
      float ms = 0.f;
      NB_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
      if (ms < best_ms) {
        best_ms = ms;
        best = k;
      }
    }
    s->ro_shape = best;
    NB_TRY(build_reference_order_worklist(s, best));
    if (chosen) *chosen = -1 - best;
    return NB_OK;
  }
  int best = s->cfg;
  float best_ms = 1e30f;
  for (int c = 0; c < num_force_configs(); ++c) {
    NB_TRY(build_main_worklist(s, c));
    s->cfg = c;
    NB_TRY(force_pass(s, s->acc_d, kPerSystemNone));  // warm-up
    NB_CUDA(cudaEventRecord(s->ev0, s->stream));
    NB_TRY(force_pass(s, s->acc_d, kPerSystemNone));
    NB_CUDA(cudaEventRecord(s->ev1, s->stream));
    NB_CUDA(cudaEventSynchronize(s->ev1));
    float ms = 0.f;
    NB_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    int reps = ms < 2.f ? 5 : (ms < 50.f ? 2 : 0);
    if (reps > 0) {
      NB_CUDA(cudaEventRecord(s->ev0, s->stream));
      for (int r = 0; r < reps; ++r) NB_TRY(force_pass(s, s->acc_d, kPerSystemNone));
      NB_CUDA(cudaEventRecord(s->ev1, s->stream));
      NB_CUDA(cudaEventSynchronize(s->ev1));
      NB_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
      ms /= reps;
    }
    NB_TRY(check_error_word(s));
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  NB_TRY(build_main_worklist(s, best));
  s->cfg = best;
  if (chosen) *chosen = best;
  return NB_OK;
}

int nb_plan_work(uint32_t num_systems, const uint32_t* sizes, int32_t config_index,
                 int32_t max_grid, nb_segment* segments, int32_t max_segments,
                 int32_t* seg_begin, int32_t* grid, int32_t* num_segments, int32_t* num_fixups,
                 int32_t* num_partial_slots) {
  static_assert(sizeof(nb_segment) == sizeof(Segment), "nb_segment mirrors Segment");
  if (num_systems == 0 || !sizes) return set_error(NB_ERR_INVALID_ARGUMENT, "no systems");
  if (config_index < -reference_order_num_shapes() || config_index >= num_force_configs())
    return set_error(NB_ERR_INVALID_ARGUMENT, "bad config index");
  if (max_grid < 1) return set_error(NB_ERR_INVALID_ARGUMENT, "max_grid must be >= 1");
  std::vector<SystemDesc> sys(num_systems);
  int64_t off = 0;
  for (uint32_t k = 0; k < num_systems; ++k) {
    if (sizes[k] == 0 || sizes[k] > (1u << 30))
      return set_error(NB_ERR_INVALID_ARGUMENT, "system size must be in [1, 2^30]");
    sys[k].offset = off;
    sys[k].n = static_cast<int32_t>(sizes[k]);
    sys[k].npad = static_cast<int32_t>((sizes[k] + kPadQuantum - 1) / kPadQuantum * kPadQuantum);
    off += sys[k].npad;
  }
  const bool tuned = config_index >= 0;
  const KernelShape sh =
      tuned ? force_config_shape(config_index) : reference_order_shape(-1 - config_index);
  // The rule of every launch: the tuned kernel's live-slot variant where it pays.
  const bool live = tuned && live_slots_pay(sys.data(), 0, static_cast<int32_t>(num_systems),
                                            sh.threads, sh.r);
  const WorkListHost h = plan_worklist(sys.data(), 0, static_cast<int32_t>(num_systems), sh.bi(),
                                       sh.bj, max_grid, live ? sh.threads : 0, sh.r);
  if (grid) *grid = h.grid;
  if (num_segments) *num_segments = static_cast<int32_t>(h.segs.size());
  if (num_fixups) *num_fixups = static_cast<int32_t>(h.fix.size());
  if (num_partial_slots) *num_partial_slots = h.slots;
  if (segments) {
    if (max_segments < static_cast<int32_t>(h.segs.size()))
      return set_error(NB_ERR_INVALID_ARGUMENT, "segments buffer too small");
    std::memcpy(segments, h.segs.data(), h.segs.size() * sizeof(Segment));
  }
  if (seg_begin) std::memcpy(seg_begin, h.seg_begin.data(), h.seg_begin.size() * sizeof(int32_t));
  return NB_OK;
}

int nb_sim_set_shard(nb_sim* s, uint64_t first, uint64_t count) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  if (s->sys_h.size() != 1)
    return set_error(NB_ERR_INVALID_ARGUMENT, "a shard splits a simulation of one system");
  if (s->params.calc_method != NB_BRANCH)
    return set_error(NB_ERR_INVALID_ARGUMENT, "shards need the BRANCH method");
  SystemDesc& d = s->sys_h[0];
  const uint64_t n = static_cast<uint64_t>(d.n);
  if (count == 0) {
    first = 0;
    count = n;
  }
  if (first % kPadQuantum || first >= n || count > n - first)
    return set_error(NB_ERR_INVALID_ARGUMENT,
                     "a shard is [first, first + count) within the system, first a multiple of 16");
  if (first + count != n && count % kPadQuantum)
    return set_error(NB_ERR_INVALID_ARGUMENT,
                     "a shard's count is a multiple of 16 unless the shard ends the system");
  d.shard_first = static_cast<int32_t>(first);
  d.shard_count = (first == 0 && count == n) ? 0 : static_cast<int32_t>(count);
  NB_TRY(upload_systems(s));
  NB_TRY(build_main_worklist(s, s->cfg));
  if (reference_order_mode(s)) NB_TRY(build_reference_order_worklist(s, s->ro_shape));
  for (auto& w : s->wl_sys) free_worklist(w);
  s->wl_sys.clear();
  s->wl_sys_policy = -1;
  s->adj.valid = false;
  NB_CUDA(cudaStreamSynchronize(s->stream));
  return NB_OK;
}

// Byte range of particles [first, first + count) of a one-system simulation's
// state arrays (16 bytes per particle in both the position and the velocity
// buffer); a block that ends the system runs to its padded end.
static int state_block(const nb_sim* s, uint64_t first, uint64_t count, int32_t what,
                       size_t* offset, size_t* bytes) {
  if (s->sys_h.size() != 1)
    return set_error(NB_ERR_INVALID_ARGUMENT, "state blocks address a simulation of one system");
  if (what != NB_BLOCK_POSITIONS && what != NB_BLOCK_VELOCITIES)
    return set_error(NB_ERR_INVALID_ARGUMENT, "what must be NB_BLOCK_POSITIONS or _VELOCITIES");
  const SystemDesc& d = s->sys_h[0];
  const uint64_t n = static_cast<uint64_t>(d.n);
  if (count == 0 || first % kPadQuantum || first >= n || count > n - first)
    return set_error(NB_ERR_INVALID_ARGUMENT,
                     "a block is [first, first + count) within the system, first a multiple of 16");
  const uint64_t end = (first + count == n) ? static_cast<uint64_t>(d.npad) : first + count;
  if (end % kPadQuantum)
    return set_error(NB_ERR_INVALID_ARGUMENT,
                     "a block's count is a multiple of 16 unless the block ends the system");
  *offset = 16 * first;
  *bytes = 16 * (end - first);
  return NB_OK;
}

int nb_sim_state_block_bytes(const nb_sim* s, uint64_t first, uint64_t count, int32_t what,
                             uint64_t* bytes) {
  if (!s || !bytes) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  size_t off = 0, b = 0;
  NB_TRY(state_block(s, first, count, what, &off, &b));
  *bytes = b;
  return NB_OK;
}

int nb_sim_copy_state_block(nb_sim* s, uint64_t first, uint64_t count, int32_t what,
                            void* dst_device) {
  if (!s || !dst_device) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard dg_(s->device);
  size_t off = 0, bytes = 0;
  NB_TRY(state_block(s, first, count, what, &off, &bytes));
  const unsigned char* src = what == NB_BLOCK_POSITIONS
                                 ? reinterpret_cast<const unsigned char*>(s->pos_d[s->cur])
                                 : reinterpret_cast<const unsigned char*>(s->vel_d);
  NB_CUDA(cudaMemcpyAsync(dst_device, src + off, bytes, cudaMemcpyDeviceToDevice, s->stream));
  return NB_OK;
}

int nb_sim_load_state_block(nb_sim* s, uint64_t first, uint64_t count, int32_t what,
                            const void* src_device) {
  if (!s || !src_device) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard dg_(s->device);
  size_t off = 0, bytes = 0;
  NB_TRY(state_block(s, first, count, what, &off, &bytes));
  unsigned char* dst = what == NB_BLOCK_POSITIONS
                           ? reinterpret_cast<unsigned char*>(s->pos_d[s->cur])
                           : reinterpret_cast<unsigned char*>(s->vel_d);
  NB_CUDA(cudaMemcpyAsync(dst + off, src_device, bytes, cudaMemcpyDeviceToDevice, s->stream));
  return NB_OK;
}

int nb_sim_generate(nb_sim* s, int32_t kind, uint64_t seed) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  if (kind != NB_IC_THIN_DISK && kind != NB_IC_PLUMMER && kind != NB_IC_TWO_DISKS)
    return set_error(NB_ERR_INVALID_ARGUMENT, "unknown initial-condition kind");
  const int32_t nsys = static_cast<int32_t>(s->sys_h.size());
  std::vector<float> m(s->n_real);
  for (int32_t k = 0; k < nsys; ++k) {
    const int32_t n = s->sys_h[k].n;
    if (kind == NB_IC_TWO_DISKS && (n < 2 || n % 2))
      return set_error(NB_ERR_INVALID_ARGUMENT, "two-disk systems need an even size");
    const double per = kind == NB_IC_TWO_DISKS ? 1.0 / (n / 2) : 1.0 / n;
    std::fill(m.begin() + s->user_offset[k], m.begin() + s->user_offset[k] + n,
              static_cast<float>(per));
  }
  int64_t* first_d = nullptr;
  double* raw = nullptr;
  double* mean = nullptr;
  int st = dev_alloc(&first_d, static_cast<size_t>(nsys));
  if (st == NB_OK && kind == NB_IC_PLUMMER) st = dev_alloc(&raw, 6 * s->n_real);
  if (st == NB_OK && kind == NB_IC_PLUMMER) st = dev_alloc(&mean, 6 * static_cast<size_t>(nsys));
  cudaError_t e = cudaSuccess;
  if (st == NB_OK) {
    e = cudaMemcpyAsync(first_d, s->user_offset.data(), nsys * sizeof(int64_t),
                        cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
      e = launch_generate(kind, s->pos_d[s->cur], s->vel_d, s->sys_d, first_d, nsys,
                          static_cast<int64_t>(s->n_real), seed, s->params.dist_eps, raw, mean,
                          s->stream);
    // Both buffers carry the masses.
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->pos_d[s->cur ^ 1], s->pos_d[s->cur], 4 * sizeof(float) * s->n_pad,
                          cudaMemcpyDeviceToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  }
  dev_free(first_d);
  dev_free(raw);
  dev_free(mean);
  if (st != NB_OK) return st;
  if (e != cudaSuccess) return cuda_error(e, "generate initial conditions");
  assign_mass_mode(s, m);
  return upload_systems(s) == NB_OK ? check_error_word(s) : NB_ERR_CUDA;
}

int nb_sim_inject_wait_timeout(nb_sim* s) {
  return nb_sim_inject_failure(s, NB_INJECT_TILE_NEVER_COPIED);
}

int nb_sim_inject_failure(nb_sim* s, int32_t kind) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  if (kind != NB_INJECT_TILE_NEVER_COPIED && kind != NB_INJECT_HAND_OVER_WITHHELD)
    return set_error(NB_ERR_INVALID_ARGUMENT, "unknown failure kind");
  if (s->params.calc_method != NB_BRANCH)
    return set_error(NB_ERR_STATE, "the failure hooks cover the BRANCH kernels only");
  if (kind == NB_INJECT_HAND_OVER_WITHHELD && !reference_order_mode(s))
    return set_error(NB_ERR_STATE, "hand-overs exist in NB_ACC_REFERENCE_ORDER only");
  s->inject = kind == NB_INJECT_TILE_NEVER_COPIED ? kInjectSkipFirstTile : kInjectWithholdHandOver;
  return NB_OK;
}

int nb_sim_graph_capture(nb_sim* s, int32_t iterations) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  if (iterations <= 0) return set_error(NB_ERR_INVALID_ARGUMENT, "iterations must be > 0");
  if (s->stream == nullptr)
    return set_error(NB_ERR_STATE, "graph capture needs a non-default stream");
  if (s->params.calc_method == NB_PREDICATED &&
      static_cast<int64_t>(s->sys_h.size()) * iterations > 65536)
    return set_error(NB_ERR_INVALID_ARGUMENT, "too many launches to capture");
  drop_graphs(s);
  // The launches bake in the buffer pointers, so keep one graph per starting buffer.
  const int cur0 = s->cur;
  for (int b = 0; b < 2; ++b) {
    s->cur = b;
    cudaError_t e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      s->cur = cur0;
      return cuda_error(e, "cudaStreamBeginCapture");
    }
    int st = NB_OK;
    for (int32_t k = 0; k < iterations && st == NB_OK; ++k) st = force_pass(s, nullptr, kPerSystemNone);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(s->stream, &g);
    s->cur = cur0;  // nothing ran
    if (st != NB_OK || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return st != NB_OK ? st : cuda_error(e, "cudaStreamEndCapture");
    }
    s->graph[b] = g;
    NB_CUDA(cudaGraphInstantiate(&s->gexec[b], g, 0));
  }
  s->graph_iters = iterations;
  return NB_OK;
}

int nb_sim_graph_launch(nb_sim* s) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  if (!s->gexec[s->cur]) return set_error(NB_ERR_STATE, "no graph captured");
  NB_CUDA(cudaGraphLaunch(s->gexec[s->cur], s->stream));
  s->cur ^= (s->graph_iters & 1);
  return NB_OK;
}

}  // extern "C"
