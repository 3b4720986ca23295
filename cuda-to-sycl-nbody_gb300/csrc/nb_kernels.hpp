// Host-callable launchers of the device kernels (implemented in the .cu files).
#pragma once

#include <cuda_runtime.h>

#include "nb_internal.hpp"

namespace nbg {

// ---- force + integrate (force_kernel.cu) ----------------------------------------
int num_force_configs();
KernelShape force_config_shape(int index);
// Launch the tuned force kernel of shape `index`.  `compensated` selects the Kahan
// accumulator, `per_pair_mass` multiplies each pair term by m_j, `live` the variant
// that skips the register slots past the end of a system (its work list is planned
// with live-slot weights, live_slots_pay in worklist.hpp).
cudaError_t launch_force(int index, bool compensated, bool per_pair_mass, bool live,
                         const ForceArgs& a, int grid, cudaStream_t stream);
cudaError_t force_blocks_per_sm(int index, bool compensated, bool per_pair_mass, bool live,
                                int* blocks);

// ---- compatibility kernel (aux_kernels.cu) ------------------------------------------
// The reference's PREDICATED variant as shipped, one thread per i-particle over one
// system (simulator.cu:186-229 with the (i == id) mask of :208-209).
cudaError_t launch_predicated(const ForceArgs& a, const SystemDesc& sd, int32_t sys_index,
                              cudaStream_t stream);

// ---- reference-order force + integrate (reference_order_kernel.cu) -------------------
// particle_interaction<BRANCH> with the reference's per-particle summation order
// and arithmetic (bit-identical results on the same GPU), equal masses per system;
// `predicated` selects particle_interaction<PREDICATED>'s pair term instead.
// Shapes are indexed largest i-tile first.  The kernel walks a stream-K work list
// (ForceArgs segs / seg_begin / fix) of reference_order_shape(index) tiles; split
// i-tiles hand their running sums over through `partials` and `counters`.  `dup` is
// the duplicated j-layout of a.pos (2 float4 per padded particle) written by
// launch_reference_order_dup.  The launch is cooperative: grid <= blocks per SM x SMs.
int reference_order_num_shapes();
KernelShape reference_order_shape(int index);  // threads, i-particles per thread, j-tile, stages
cudaError_t reference_order_blocks_per_sm(int index, bool predicated, int* blocks);
cudaError_t launch_reference_order_dup(const float* pos, int64_t n_pad_total, float4* dup,
                                       cudaStream_t stream);
cudaError_t launch_reference_order(int index, bool predicated, const ForceArgs& a,
                                   const float4* dup, int grid, cudaStream_t stream);

// ---- measured FP32 throughput (peak_probe.cu) ----------------------------------------
// Time `repeats` launches (after one warm-up) of an FFMA2 loop over sms x blocks_per_sm
// CTAs; `scratch` holds sms * blocks_per_sm * fp32_peak_threads() float2.
cudaError_t measure_fp32_peak(int sms, float2* scratch, int blocks_per_sm, int iters,
                              int repeats, cudaStream_t stream, double* tflops, float* best_ms);
int fp32_peak_threads();

// ---- state movement (aux_kernels.cu) ------------------------------------------------
// Device SoA staging <-> simulation layout.  `map` holds, for each of the n real
// particles in user order, its padded device index.
cudaError_t launch_unpack_state(const float* soa /*[7][n]: x y z vx vy vz m*/, int64_t n,
                                const int64_t* map, float* pos, float4* vel, bool with_mass,
                                cudaStream_t stream);
cudaError_t launch_pack_state(const float* pos, const float4* vel, int64_t n, const int64_t* map,
                              float* soa /*[6][n]*/, cudaStream_t stream);
cudaError_t launch_pack_accel(const float4* acc, int64_t n, const int64_t* map,
                              float* soa /*[3][n]*/, cudaStream_t stream);
cudaError_t launch_export(const float* pos, const float4* vel, int64_t n, const int64_t* map,
                          float4* pos_out, float4* vel_out, cudaStream_t stream);
cudaError_t launch_fill_padding(float* pos, float4* vel, int64_t n_pad_total, cudaStream_t stream);

// ---- FP64 diagnostics (diag_kernels.cu) ---------------------------------------------
struct DiagScratch {
  double* partial;   // [max_blocks][10]
  int32_t max_blocks;
};
cudaError_t launch_diagnostics(const float* pos, const float4* vel, const SystemDesc* sys_d,
                               const SystemDesc* sys_h, int32_t first_sys, int32_t num_sys,
                               float eps2, float G, bool per_pair_mass, double* out10,
                               DiagScratch& scratch, cudaStream_t stream);
cudaError_t launch_fp64_rows(const float* pos, const SystemDesc* sys_d, const int64_t* rows_dev,
                             const int32_t* row_sys_dev, int64_t count, float eps2, float G,
                             bool per_pair_mass, double* out3, cudaStream_t stream);

// ---- adjoint (adjoint_kernel.cu) ----------------------------------------------------
struct AdjointArgs {
  const float* pos;       // pair layout, positions x_t at which the Jacobian is taken
  const float4* lam_x;    // [n_pad] lam_x' (cotangent of x')
  const float4* lam_v;    // [n_pad] lam_v' (cotangent of v')
  float4* lam_x_out;      // [n_pad] lam_x = lam_x' + dt * G * J^T mu, mu = lam_v' + dt lam_x'
  float4* lam_v_out;      // [n_pad] lam_v = damping * mu
  const SystemDesc* sys;
  const int32_t* tile_sys;  // [tiles] system of each i-tile
  const int32_t* tile_idx;  // [tiles] i-tile index within its system
  float4* partial;          // [num_splits][n_pad] per-chunk partial sums
  int64_t n_pad;
  int32_t num_splits;       // j-chunks per i-tile
  float eps2;
  float dt;
  float damping;
  int32_t mask_self;
};
cudaError_t launch_adjoint(const AdjointArgs& a, int32_t num_tiles, bool per_pair_mass,
                           cudaStream_t stream);
int adjoint_tile();  // i-particles per adjoint CTA
cudaError_t adjoint_blocks_per_sm(bool per_pair_mass, int* blocks);
// n x 3 interleaved (user order) <-> padded float4.
cudaError_t launch_unpack_vec3(const float* in, int64_t n, const int64_t* map, float4* out,
                               cudaStream_t stream);
cudaError_t launch_pack_vec3(const float4* in, int64_t n, const int64_t* map, float* out,
                             cudaStream_t stream);

// ---- initial conditions on the device (initgen.cu) ------------------------------------
// kind 1: thin disks, 2: Plummer (needs raw [6 * total] and mean [6 * nsys] FP64
// scratch), 3: two-disk collisions.  first_d[k] = first user index of system k.
cudaError_t launch_generate(int kind, float* pos, float4* vel, const SystemDesc* sys_d,
                            const int64_t* first_d, int32_t nsys, int64_t total, uint64_t seed,
                            double eps, double* raw, double* mean, cudaStream_t stream);

}  // namespace nbg
