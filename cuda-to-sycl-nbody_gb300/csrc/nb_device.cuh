// Device helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>

#include "nb_internal.hpp"

namespace nbg {

// Integrate (or write accelerations for) one real particle.
__device__ __forceinline__ void finish_particle(const ForceArgs& a, const SystemDesc& sd,
                                                int64_t gi, float fx, float fy, float fz,
                                                float xi, float yi, float zi) {
  const float g = sd.gscale;
  if (a.accel_out != nullptr) {
    a.accel_out[gi] = make_float4(fx * g, fy * g, fz * g, 0.f);
    return;
  }
  float4 v = a.vel[gi];
  // v = v * damping; v += (F * dt) * G   (simulator.cu:214-216)
  v.x = fmaf(fx * a.dt, g, v.x * a.damping);
  v.y = fmaf(fy * a.dt, g, v.y * a.damping);
  v.z = fmaf(fz * a.dt, g, v.z * a.damping);
  a.vel[gi] = v;
  // x' = x + v * dt   (simulator.cu:223-228)
  a.pos_next[pair_index(gi, 0)] = fmaf(v.x, a.dt, xi);
  a.pos_next[pair_index(gi, 1)] = fmaf(v.y, a.dt, yi);
  a.pos_next[pair_index(gi, 2)] = fmaf(v.z, a.dt, zi);
  a.pos_next[pair_index(gi, 3)] = a.pos[pair_index(gi, 3)];
}

}  // namespace nbg
