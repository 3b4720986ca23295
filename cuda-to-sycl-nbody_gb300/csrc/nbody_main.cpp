// Headless driver: the reference's no_render main (src/nbody.cpp:31-36 construction,
// :83-123 the DISABLE_GL frame loop) on the GB300 simulator.  Same positional arguments
// (nBatches iters damping dt distEps G numFrames gwSize calcMethod) and the same
// per-step line on stdout.
//
// Two environment variables that the reference does not have:
//   NBODY_GB300_ACCUMULATOR   plain | compensated | reference_order (default
//                             compensated);
//                             reference_order gives the reference kernel's results bit
//                             for bit
//   NBODY_GB300_STATE_OUT     file that receives the final state as raw float32
//                             arrays x, y, z, vx, vy, vz (numParticles each)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "simulator.hpp"

using namespace simulation;

namespace {

int accumulator_from_env(int fallback) {
  const char* v = std::getenv("NBODY_GB300_ACCUMULATOR");
  if (!v || !*v) return fallback;
  if (!std::strcmp(v, "plain")) return NB_ACC_PLAIN;
  if (!std::strcmp(v, "compensated")) return NB_ACC_COMPENSATED;
  if (!std::strcmp(v, "reference_order")) return NB_ACC_REFERENCE_ORDER;
  throw std::invalid_argument(std::string("NBODY_GB300_ACCUMULATOR must be plain, compensated or "
                                          "reference_order, not ") + v);
}

void write_state(const char* path, const ParticleData& pos, const ParticleData& vel) {
  FILE* f = std::fopen(path, "wb");
  if (!f) throw std::runtime_error(std::string("cannot open ") + path);
  bool ok = true;
  for (const std::vector<coords_t>* a : {&pos.x, &pos.y, &pos.z, &vel.x, &vel.y, &vel.z})
    ok = ok && std::fwrite(a->data(), sizeof(coords_t), a->size(), f) == a->size();
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) throw std::runtime_error(std::string("cannot write ") + path);
}

}  // namespace

int main(int argc, char** argv) {
  try {
    SimParam params;
    params.parseArgs(argc, argv);
    params.accumulator = accumulator_from_env(params.accumulator);
    DiskGalaxySimulator nbodySim(params);

    std::vector<float> stepTimes;
    size_t step = 0;
    while (step < params.numFrames) {
      nbodySim.stepSim();
      step++;
      const size_t warmSteps = 2;
      if (step > warmSteps) {
        stepTimes.push_back(nbodySim.getLastStepTime());
        // The same arithmetic as src/nbody.cpp:110-118: the sum is taken in double
        // (initial value 0.0) and stored as float; each squared deviation comes
        // from std::pow in double and is added into a float.
        const float cum = std::accumulate(stepTimes.begin(), stepTimes.end(), 0.0);
        const float mean = cum / stepTimes.size();
        float acc = 0.0f;
        for (const float t : stepTimes) acc += std::pow(t - mean, 2);
        const float sd = std::pow(acc / stepTimes.size(), 0.5);
        std::cout << "At step " << step << " kernel time is " << stepTimes.back()
                  << " and mean is " << mean << " and stddev is: " << sd << "\n";
      }
    }
    if (const char* out = std::getenv("NBODY_GB300_STATE_OUT"))
      if (*out) write_state(out, nbodySim.getParticlePos(), nbodySim.getParticleVel());
  } catch (const std::exception& e) {
    std::cerr << "nbody_gb300: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
