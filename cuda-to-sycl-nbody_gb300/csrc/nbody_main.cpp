// Headless driver: the reference's no_render main loop (src/nbody.cpp:138-248 with
// DISABLE_GL) on the GB300 simulator.  Same positional arguments
// (nBatches iters damping dt distEps G numFrames gwSize calcMethod) and the same
// per-step line on stdout.
#include <cmath>
#include <cstdio>
#include <iostream>
#include <numeric>
#include <stdexcept>
#include <vector>

#include "simulator.hpp"

using namespace simulation;

int main(int argc, char** argv) {
  try {
    SimParam params;
    params.parseArgs(argc, argv);
    DiskGalaxySimulator nbodySim(params);

    std::vector<float> stepTimes;
    size_t step = 0;
    while (step < params.numFrames) {
      nbodySim.stepSim();
      step++;
      const size_t warmSteps = 2;
      if (step > warmSteps) {
        stepTimes.push_back(nbodySim.getLastStepTime());
        const float cum = std::accumulate(stepTimes.begin(), stepTimes.end(), 0.0f);
        const float mean = cum / stepTimes.size();
        float acc = 0.0f;
        for (float t : stepTimes) acc += (t - mean) * (t - mean);
        const float sd = std::sqrt(acc / stepTimes.size());
        std::cout << "At step " << step << " kernel time is " << stepTimes.back()
                  << " and mean is " << mean << " and stddev is: " << sd << "\n";
      }
    }
  } catch (const std::exception& e) {
    std::cerr << "nbody_gb300: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
