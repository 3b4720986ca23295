// The simulation object behind the opaque nb_sim handle, and runtime helpers
// shared by the host translation units.
#pragma once

#include <cuda_runtime.h>

#include <atomic>

#include <cstdint>
#include <string>
#include <vector>

#include "nb_internal.hpp"
#include "nb_kernels.hpp"
#include "nb_render.hpp"
#include "nbody_gb300.h"

namespace nbg {

// A work list on the device.  cfg >= 0: a shape of the tuned force kernel;
// cfg < 0: reference-order shape -1 - cfg.
struct WorkListDev {
  int32_t cfg = -1;
  bool live = false;  // the force kernel's live-slot variant (planned with its weights)
  int32_t grid = 0;
  int32_t nseg = 0;
  int32_t nfix = 0;
  int32_t slots = 0;
  int32_t split = 0;
  Segment* segs = nullptr;
  int32_t* seg_begin = nullptr;
  Fixup* fix = nullptr;
};

// Checkpoints and work buffers of the adjoint (allocated on first use).
struct AdjointState {
  int32_t T = 0;
  int32_t every = 0;
  int32_t count = 0;                // number of checkpoints stored
  int32_t start_cur = 0;
  std::vector<float*> ckpt_pos;     // pair layout, n_pad * 4 floats each
  std::vector<float4*> ckpt_vel;
  std::vector<float*> seg_pos;      // positions of one recomputed segment
  float4* lam_x = nullptr;
  float4* lam_v = nullptr;
  float4* mu = nullptr;
  float4* tmp = nullptr;
  float4* vel = nullptr;            // velocities of the recomputed segment
  int32_t* tile_sys = nullptr;
  int32_t* tile_idx = nullptr;
  int32_t num_tiles = 0;
  int32_t num_splits = 1;
  float4* partial = nullptr;        // [num_splits][n_pad]
  bool valid = false;
};

}  // namespace nbg

struct nb_sim {
  nb_params params{};
  int device = 0;  // the CUDA device current when the simulation was created
  int sms = 0;
  std::string device_name;
  cudaStream_t stream = nullptr;
  bool own_stream = false;

  std::vector<nbg::SystemDesc> sys_h;
  std::vector<int64_t> user_offset;  // first user index of each system
  uint64_t n_real = 0;
  int64_t n_pad = 0;
  nbg::SystemDesc* sys_d = nullptr;
  int64_t* map_d = nullptr;  // user index -> padded index (NULL: identity, one system)

  float* pos_d[2] = {nullptr, nullptr};  // pair layout, double-buffered
  int cur = 0;
  float4* vel_d = nullptr;
  float4* acc_d = nullptr;
  float* staging_d = nullptr;  // [7][n_real]
  int32_t* err_d = nullptr;
  bool per_pair_mass = false;
  int32_t mask_self = 0;
  int32_t inject = 0;  // one-shot failure-detection hook for the next force launch (kInject*)

  int cfg = 0;
  nbg::WorkListDev wl;
  std::vector<nbg::WorkListDev> wl_sys;
  int wl_sys_policy = -1;  // how wl_sys was planned (kPerSystem*), -1: not yet
  int wl_sys_cfg = 0;      // and with which shape, for kPerSystemSimShape
  float4* partials_d = nullptr;
  size_t partials_cap = 0;
  int32_t* counters_d = nullptr;
  size_t counters_cap = 0;

  // NB_ACC_REFERENCE_ORDER: the reference-order kernel's shape, its work list
  // (config index -1 - shape) and the duplicated j-layout of the positions.
  int ro_shape = 0;
  nbg::WorkListDev ro_wl;
  float4* ro_dup_d = nullptr;  // [2 * n_pad]

  cudaEvent_t ev0 = nullptr;
  cudaEvent_t ev1 = nullptr;
  float last_ms = 0.f;

  cudaGraph_t graph[2] = {nullptr, nullptr};        // indexed by starting buffer
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  int32_t graph_iters = 0;

  nbg::DiagScratch diag{};
  double* diag_out_d = nullptr;
  nbg::AdjointState adj;
  nbg::RenderBuffers render;
};

namespace nbg {

extern thread_local std::string t_last_error;
// Failure-detection hook (nb_inject_alloc_failure): while positive, each device
// allocation counts it down, and the one that brings it to zero fails.
extern std::atomic<int> g_alloc_failure_countdown;
int set_error(int code, const std::string& msg);
int cuda_error(cudaError_t e, const char* what);
// Properties of the current device; NB_ERR_NO_DEVICE unless it is an sm_103 GPU.
int check_device(int* sms, cudaDeviceProp* prop, int* device = nullptr);

// Makes `dev` current for the lifetime of the guard and restores the caller's
// device afterwards, so that a simulation always runs on the device it was created
// on whatever device the calling thread has selected since.
class DeviceGuard {
 public:
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev_) == cudaSuccess && prev_ != dev && cudaSetDevice(dev) == cudaSuccess)
      switched_ = true;
  }
  ~DeviceGuard() {
    if (switched_) cudaSetDevice(prev_);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;

 private:
  int prev_ = 0;
  bool switched_ = false;
};
void free_worklist(WorkListDev& w);
// Free the diagnostics and adjoint buffers of a simulation.
void release_aux(nb_sim* s);
void release_render_buffers(nb_sim* s);

template <class T>
int dev_alloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) return NB_OK;
  if (g_alloc_failure_countdown.load(std::memory_order_relaxed) > 0 &&
      g_alloc_failure_countdown.fetch_sub(1) == 1)
    return set_error(NB_ERR_OUT_OF_MEMORY, "injected allocation failure (nb_inject_alloc_failure)");
  const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_error(e, "cudaMalloc");
  }
  return NB_OK;
}

template <class T>
void dev_free(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

// Shared by the host translation units (nbody_capi.cpp).
ForceArgs base_args(nb_sim* s);
// How force_pass launches an ensemble: one persistent launch over every system,
// or one launch per system, each planned with the shape the system would get as a
// simulation of its own, or each with the simulation's current shape.
constexpr int kPerSystemNone = 0;
constexpr int kPerSystemOwnShape = 1;
constexpr int kPerSystemSimShape = 2;
// One force evaluation over all systems: integrate into the other position
// buffer and swap (accel_out == nullptr), or write accelerations.
int force_pass(nb_sim* s, float4* accel_out, int per_system);
int check_error_word(nb_sim* s);
int ensure_staging(nb_sim* s);
int ensure_accel(nb_sim* s);
// Launch the force kernel with arguments `a` over work list `w`.
int launch_with(nb_sim* s, ForceArgs a, const WorkListDev& w);

#define NB_TRY(expr)            \
  do {                          \
    const int s_ = (expr);      \
    if (s_ != NB_OK) return s_; \
  } while (0)
#define NB_CUDA(expr)                                          \
  do {                                                         \
    const cudaError_t e_ = (expr);                             \
    if (e_ != cudaSuccess) return ::nbg::cuda_error(e_, #expr); \
  } while (0)

}  // namespace nbg
