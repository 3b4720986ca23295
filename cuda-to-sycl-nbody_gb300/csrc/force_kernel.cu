// Table of the compiled shapes of the force kernel (force_kernel.cuh).  Each
// force_shapes_*.cu file instantiates a few shapes so that they compile in parallel.
#include <cuda_runtime.h>

#include "force_kernel.cuh"

namespace nbg {

extern const ConfigEntry kForceShapesA[];
extern const int kNumForceShapesA;
extern const ConfigEntry kForceShapesB[];
extern const int kNumForceShapesB;
extern const ConfigEntry kForceShapesC[];
extern const int kNumForceShapesC;

namespace {

const ConfigEntry& entry(int index) {
  if (index < kNumForceShapesA) return kForceShapesA[index];
  index -= kNumForceShapesA;
  if (index < kNumForceShapesB) return kForceShapesB[index];
  return kForceShapesC[index - kNumForceShapesB];
}

}  // namespace

int num_force_configs() { return kNumForceShapesA + kNumForceShapesB + kNumForceShapesC; }

KernelShape force_config_shape(int index) { return entry(index).shape; }

cudaError_t launch_force(int index, bool compensated, bool per_pair_mass, bool live,
                         const ForceArgs& a, int grid, cudaStream_t stream) {
  return entry(index).launch[live][compensated][per_pair_mass](a, grid, stream);
}

cudaError_t force_blocks_per_sm(int index, bool compensated, bool per_pair_mass, bool live,
                                int* blocks) {
  return entry(index).occ[live][compensated][per_pair_mass](blocks);
}

}  // namespace nbg
