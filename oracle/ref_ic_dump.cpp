// Dump the reference's own initial state: construct the reference's
// simulation::DiskGalaxySimulator (src/simulator.cuh:129-160) from a SimParam with
// numParticles = 256 * nBatches, as its main does (src/nbody.cpp:33-36), and write
// getParticlePos() and getParticleVel() as raw float32 arrays x, y, z, vx, vy, vz.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.sh from the reference's
// unmodified src/simulator.cu and src/sim_param.cpp, with oracle/ref_ic_host.cpp
// standing in for the CUDA runtime on a host without a GPU.
//
//   ref_ic_dump OUT_FILE NBATCHES
#include <cstdio>
#include <cstdlib>

#include "simulator.cuh"

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s OUT_FILE NBATCHES\n", argv[0]);
    return 2;
  }
  SimParam params;
  params.numParticles = 256 * static_cast<size_t>(std::atoll(argv[2]));
  simulation::DiskGalaxySimulator sim(params);
  const simulation::ParticleData& pos = sim.getParticlePos();
  const simulation::ParticleData& vel = sim.getParticleVel();
  std::FILE* f = std::fopen(argv[1], "wb");
  if (!f) return 1;
  bool ok = true;
  for (const auto* a : {&pos.x, &pos.y, &pos.z, &vel.x, &vel.y, &vel.z})
    ok = ok && std::fwrite(a->data(), sizeof(float), a->size(), f) == a->size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? 0 : 1;
}
