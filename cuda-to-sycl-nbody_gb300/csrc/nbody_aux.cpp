// C ABI: FP64 diagnostics and the adjoint of the step (host side).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "nb_internal.hpp"
#include "nb_kernels.hpp"
#include "nb_runtime.hpp"
#include "nbody_gb300.h"

using namespace nbg;

namespace nbg {

void release_aux(nb_sim* s) {
  if (s->diag.partial) cudaFree(s->diag.partial);
  s->diag = DiagScratch{};
  dev_free(s->diag_out_d);
  AdjointState& a = s->adj;
  for (auto* p : a.ckpt_pos) cudaFree(p);
  for (auto* p : a.ckpt_vel) cudaFree(p);
  for (auto* p : a.seg_pos) cudaFree(p);
  dev_free(a.lam_x);
  dev_free(a.lam_v);
  dev_free(a.mu);
  dev_free(a.tmp);
  dev_free(a.vel);
  dev_free(a.tile_sys);
  dev_free(a.tile_idx);
  dev_free(a.partial);
  a = AdjointState{};
}

}  // namespace nbg

namespace {

int ensure_adjoint_buffers(nb_sim* s, int32_t ncp, int32_t every) {
  AdjointState& a = s->adj;
  const size_t np = static_cast<size_t>(s->n_pad);
  while (static_cast<int32_t>(a.ckpt_pos.size()) < ncp) {
    float* p = nullptr;
    float4* v = nullptr;
    NB_TRY(dev_alloc(&p, 4 * np));
    a.ckpt_pos.push_back(p);
    NB_TRY(dev_alloc(&v, np));
    a.ckpt_vel.push_back(v);
  }
  if (!a.vel) NB_TRY(dev_alloc(&a.vel, np));
  while (static_cast<int32_t>(a.seg_pos.size()) < every) {
    float* p = nullptr;
    NB_TRY(dev_alloc(&p, 4 * np));
    // Padding particles must sit far away with zero mass in every buffer the
    // force kernel reads; the kernel writes only real particles.
    NB_CUDA(launch_fill_padding(p, a.vel, s->n_pad, s->stream));
    a.seg_pos.push_back(p);
  }
  if (!a.lam_x) {
    NB_TRY(dev_alloc(&a.lam_x, np));
    NB_TRY(dev_alloc(&a.lam_v, np));
    NB_TRY(dev_alloc(&a.mu, np));
    NB_TRY(dev_alloc(&a.tmp, np));
  }
  if (!a.tile_sys) {
    std::vector<int32_t> ts, ti;
    const int bi = adjoint_tile();
    for (int32_t k = 0; k < static_cast<int32_t>(s->sys_h.size()); ++k)
      for (int32_t t = 0; t < (s->sys_h[k].n + bi - 1) / bi; ++t) {
        ts.push_back(k);
        ti.push_back(t);
      }
    a.num_tiles = static_cast<int32_t>(ts.size());
    // j-chunks per i-tile: one full wave of resident CTAs (i-tiles x chunks = SMs x
    // resident CTAs per SM, rounded up), the chunk sums reduced in order afterwards.
    int per_sm = 1;
    if (adjoint_blocks_per_sm(s->per_pair_mass, &per_sm) != cudaSuccess || per_sm < 1) per_sm = 1;
    const int32_t target = per_sm * s->sms;
    a.num_splits = std::max(1, std::min(64, (target + a.num_tiles - 1) / a.num_tiles));
    NB_TRY(dev_alloc(&a.partial, static_cast<size_t>(a.num_splits) * np));
    NB_TRY(dev_alloc(&a.tile_sys, ts.size()));
    NB_TRY(dev_alloc(&a.tile_idx, ti.size()));
    NB_CUDA(cudaMemcpy(a.tile_sys, ts.data(), ts.size() * sizeof(int32_t),
                       cudaMemcpyHostToDevice));
    NB_CUDA(cudaMemcpy(a.tile_idx, ti.data(), ti.size() * sizeof(int32_t),
                       cudaMemcpyHostToDevice));
  }
  return NB_OK;
}

}  // namespace

extern "C" {

int nb_sim_diagnostics(nb_sim* s, int32_t system, nb_diagnostics* out) {
  if (!s || !out) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard dg_(s->device);
  const int32_t nsys = static_cast<int32_t>(s->sys_h.size());
  if (system < -1 || system >= nsys) return set_error(NB_ERR_INVALID_ARGUMENT, "bad system");
  if (!s->diag_out_d) NB_TRY(dev_alloc(&s->diag_out_d, 10));
  const int32_t first = system < 0 ? 0 : system;
  const int32_t count = system < 0 ? nsys : 1;
  NB_CUDA(launch_diagnostics(s->pos_d[s->cur], s->vel_d, s->sys_d, s->sys_h.data(), first, count,
                             s->params.dist_eps, s->params.G, s->per_pair_mass, s->diag_out_d,
                             s->diag, s->stream));
  double h[10];
  NB_CUDA(cudaMemcpyAsync(h, s->diag_out_d, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
  NB_CUDA(cudaStreamSynchronize(s->stream));
  out->potential = h[0];
  out->kinetic = h[1];
  out->total = h[0] + h[1];
  out->momentum[0] = h[3];
  out->momentum[1] = h[4];
  out->momentum[2] = h[5];
  out->angular_momentum[0] = h[6];
  out->angular_momentum[1] = h[7];
  out->angular_momentum[2] = h[8];
  out->mass = h[9];
  return NB_OK;
}

int nb_sim_fp64_accelerations(nb_sim* s, const uint64_t* rows, uint64_t count, double* ax,
                              double* ay, double* az) {
  if (!s || (count && (!rows || !ax || !ay || !az)))
    return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard dg_(s->device);
  if (count == 0) return NB_OK;
  if (count > (1u << 24)) return set_error(NB_ERR_INVALID_ARGUMENT, "too many rows");
  std::vector<int64_t> g(count);
  std::vector<int32_t> sy(count);
  for (uint64_t k = 0; k < count; ++k) {
    if (rows[k] >= s->n_real) return set_error(NB_ERR_INVALID_ARGUMENT, "row out of range");
    const auto it = std::upper_bound(s->user_offset.begin(), s->user_offset.end(),
                                     static_cast<int64_t>(rows[k]));
    const int32_t sys = static_cast<int32_t>(it - s->user_offset.begin()) - 1;
    sy[k] = sys;
    g[k] = s->sys_h[sys].offset + (static_cast<int64_t>(rows[k]) - s->user_offset[sys]);
  }
  int64_t* g_d = nullptr;
  int32_t* s_d = nullptr;
  double* o_d = nullptr;
  int st = dev_alloc(&g_d, count);
  if (st == NB_OK) st = dev_alloc(&s_d, count);
  if (st == NB_OK) st = dev_alloc(&o_d, 3 * count);
  std::vector<double> o(3 * count);
  cudaError_t e = cudaSuccess;
  if (st == NB_OK) {
    e = cudaMemcpyAsync(g_d, g.data(), count * sizeof(int64_t), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s_d, sy.data(), count * sizeof(int32_t), cudaMemcpyHostToDevice,
                          s->stream);
    if (e == cudaSuccess)
      e = launch_fp64_rows(s->pos_d[s->cur], s->sys_d, g_d, s_d, static_cast<int64_t>(count),
                           s->params.dist_eps, s->params.G, s->per_pair_mass, o_d, s->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(o.data(), o_d, 3 * count * sizeof(double), cudaMemcpyDeviceToHost,
                          s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  }
  dev_free(g_d);
  dev_free(s_d);
  dev_free(o_d);
  if (st != NB_OK) return st;
  if (e != cudaSuccess) return cuda_error(e, "fp64 accelerations");
  for (uint64_t k = 0; k < count; ++k) {
    ax[k] = o[3 * k];
    ay[k] = o[3 * k + 1];
    az[k] = o[3 * k + 2];
  }
  return NB_OK;
}

int nb_sim_adjoint_forward(nb_sim* s, int32_t T, int32_t checkpoint_every) {
  if (!s) return set_error(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
  DeviceGuard dg_(s->device);
  if (T < 1 || checkpoint_every < 1)
    return set_error(NB_ERR_INVALID_ARGUMENT, "T and checkpoint_every must be >= 1");
  if (s->params.calc_method != NB_BRANCH)
    return set_error(NB_ERR_STATE, "the adjoint is defined for the BRANCH method only");
  for (const SystemDesc& d : s->sys_h)
    if (d.shard_first != 0 || d.shard_count != 0)
      return set_error(NB_ERR_STATE, "the adjoint needs the whole system, not a shard");
  const int32_t every = std::min(checkpoint_every, T);
  const int32_t ncp = (T + every - 1) / every;
  s->adj.valid = false;
  NB_TRY(ensure_adjoint_buffers(s, ncp, every));
  const size_t np = static_cast<size_t>(s->n_pad);
  for (int32_t k = 0; k < ncp; ++k) {
    NB_CUDA(cudaMemcpyAsync(s->adj.ckpt_pos[k], s->pos_d[s->cur], 4 * np * sizeof(float),
                            cudaMemcpyDeviceToDevice, s->stream));
    NB_CUDA(cudaMemcpyAsync(s->adj.ckpt_vel[k], s->vel_d, np * sizeof(float4),
                            cudaMemcpyDeviceToDevice, s->stream));
    NB_TRY(nb_sim_advance(s, std::min(every, T - k * every)));
  }
  NB_TRY(nb_sim_synchronize(s));
  s->adj.T = T;
  s->adj.every = every;
  s->adj.count = ncp;
  s->adj.valid = true;
  return NB_OK;
}

// The backward sweep, stream-ordered on the simulation's stream, from device
// gradients dL/dx_T, dL/dv_T (n x 3, xyz-interleaved; gv_T may be NULL) to device
// dL/dx_0, dL/dv_0.  The outputs may alias the inputs: the inputs are read first.
static int adjoint_backward_stream(nb_sim* s, const float* gx_T, const float* gv_T, float* gx_0,
                                   float* gv_0) {
  AdjointState& a = s->adj;
  const size_t n = s->n_real;
  const size_t np = static_cast<size_t>(s->n_pad);
  NB_CUDA(cudaMemsetAsync(a.lam_x, 0, np * sizeof(float4), s->stream));
  NB_CUDA(cudaMemsetAsync(a.lam_v, 0, np * sizeof(float4), s->stream));
  NB_CUDA(cudaMemsetAsync(a.tmp, 0, np * sizeof(float4), s->stream));
  NB_CUDA(cudaMemsetAsync(a.mu, 0, np * sizeof(float4), s->stream));
  NB_CUDA(launch_unpack_vec3(gx_T, n, s->map_d, a.lam_x, s->stream));
  if (gv_T) NB_CUDA(launch_unpack_vec3(gv_T, n, s->map_d, a.lam_v, s->stream));
  const float dt = s->params.dt;
  for (int32_t k = a.count - 1; k >= 0; --k) {
    const int32_t t0 = k * a.every;
    const int32_t L = std::min(a.every, a.T - t0);
    // Recompute the positions x_{t0} .. x_{t0+L-1} from the checkpoint.
    NB_CUDA(cudaMemcpyAsync(a.seg_pos[0], a.ckpt_pos[k], 4 * np * sizeof(float),
                            cudaMemcpyDeviceToDevice, s->stream));
    NB_CUDA(cudaMemcpyAsync(a.vel, a.ckpt_vel[k], np * sizeof(float4), cudaMemcpyDeviceToDevice,
                            s->stream));
    for (int32_t t = 0; t + 1 < L; ++t) {
      ForceArgs fa = base_args(s);
      fa.pos = a.seg_pos[t];
      fa.pos_next = a.seg_pos[t + 1];
      fa.vel = a.vel;
      NB_TRY(launch_with(s, fa, s->wl));
    }
    // Reverse through the segment.
    for (int32_t t = L - 1; t >= 0; --t) {
      AdjointArgs aa{};
      aa.pos = a.seg_pos[t];
      aa.lam_x = a.lam_x;
      aa.lam_v = a.lam_v;
      aa.lam_x_out = a.tmp;
      aa.lam_v_out = a.mu;  // second buffer pair: (tmp, mu) <- (lam_x, lam_v)
      aa.sys = s->sys_d;
      aa.tile_sys = a.tile_sys;
      aa.tile_idx = a.tile_idx;
      aa.partial = a.partial;
      aa.n_pad = s->n_pad;
      aa.num_splits = a.num_splits;
      aa.eps2 = s->params.dist_eps;
      aa.dt = dt;
      aa.damping = s->params.damping;
      aa.mask_self = s->mask_self;
      NB_CUDA(launch_adjoint(aa, a.num_tiles, s->per_pair_mass, s->stream));
      std::swap(a.lam_x, a.tmp);
      std::swap(a.lam_v, a.mu);
    }
  }
  NB_CUDA(launch_pack_vec3(a.lam_x, n, s->map_d, gx_0, s->stream));
  NB_CUDA(launch_pack_vec3(a.lam_v, n, s->map_d, gv_0, s->stream));
  return NB_OK;
}

int nb_sim_adjoint_backward(nb_sim* s, const float* gx_T, const float* gv_T, float* gx_0,
                            float* gv_0) {
  if (!s || !gx_T || !gx_0 || !gv_0) return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard dg_(s->device);
  AdjointState& a = s->adj;
  if (!a.valid) return set_error(NB_ERR_STATE, "call nb_sim_adjoint_forward first");
  NB_TRY(ensure_staging(s));
  const size_t n = s->n_real;
  float* stage = s->staging_d;  // 7n floats: the two n x 3 arrays in and out
  NB_CUDA(cudaMemcpyAsync(stage, gx_T, 3 * n * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  if (gv_T)
    NB_CUDA(cudaMemcpyAsync(stage + 3 * n, gv_T, 3 * n * sizeof(float), cudaMemcpyHostToDevice,
                            s->stream));
  NB_TRY(adjoint_backward_stream(s, stage, gv_T ? stage + 3 * n : nullptr, stage, stage + 3 * n));
  NB_CUDA(cudaMemcpyAsync(gx_0, stage, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  NB_CUDA(cudaMemcpyAsync(gv_0, stage + 3 * n, 3 * n * sizeof(float), cudaMemcpyDeviceToHost,
                          s->stream));
  NB_CUDA(cudaStreamSynchronize(s->stream));
  return check_error_word(s);
}

int nb_sim_adjoint_backward_device(nb_sim* s, const float* gx_T_device, const float* gv_T_device,
                                   float* gx_0_device, float* gv_0_device) {
  if (!s || !gx_T_device || !gx_0_device || !gv_0_device)
    return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard dg_(s->device);
  if (!s->adj.valid) return set_error(NB_ERR_STATE, "call nb_sim_adjoint_forward first");
  return adjoint_backward_stream(s, gx_T_device, gv_T_device, gx_0_device, gv_0_device);
}

}  // extern "C"
