// C++ mirror of the reference's simulator interface, implemented over the C ABI.
//
//   SimParam                      src/sim_param.hpp:16-40, src/sim_param.cpp:12-67
//   simulation::ParticleData      src/simulator.cuh:75-84
//   simulation::Simulator         src/simulator.cuh:107-116
//   simulation::DiskGalaxySimulator src/simulator.cuh:129-160
//
// Same names, members and meaning, so code written against the reference's
// headers compiles against this one.  Differences: errors raise
// std::runtime_error instead of exit() (the reference's gpuErrchk,
// simulator.cuh:22-31); stepSim times with CUDA events; the current positions
// are also available on the device (devicePositions) so a renderer need not
// copy through the host.
#pragma once

#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "nbody_gb300.h"

enum class CalculationMethod { BRANCH, PREDICATED };

class SimParam {
 public:
  SimParam();
  void parseArgs(int argc, char** argv);

  float G;
  float dt;
  size_t numParticles;
  size_t numFrames;
  int simIterationsPerFrame;
  float damping;
  float distEps;
  int gwSize;
  CalculationMethod calcMethod;
  // Not in the reference: how each particle's force is summed (nb_accumulator;
  // NB_ACC_REFERENCE_ORDER reproduces the reference kernel bit for bit).
  int accumulator;

  nb_params toC() const;
};

namespace simulation {

typedef float coords_t;

struct ParticleData {
  std::vector<coords_t> x;
  std::vector<coords_t> y;
  std::vector<coords_t> z;

  ParticleData(std::vector<coords_t> x_, std::vector<coords_t> y_, std::vector<coords_t> z_)
      : x(std::move(x_)), y(std::move(y_)), z(std::move(z_)) {}
  explicit ParticleData(size_t n) : x(n, 0.0f), y(n, 0.0f), z(n, 0.0f) {}
};

class Simulator {
 public:
  virtual ~Simulator() = default;
  virtual void stepSim() = 0;
  virtual size_t getNumParticles() = 0;
  virtual const ParticleData& getParticlePos() = 0;
  virtual const ParticleData& getParticleVel() = 0;
  virtual float getLastStepTime() = 0;
  virtual const std::string* getDeviceName() = 0;
  virtual int getGwSize() = 0;
};

class DiskGalaxySimulator : public Simulator {
 public:
  // The reference's constructor: its default-seeded disk (simulator.cu:24-34).
  explicit DiskGalaxySimulator(SimParam params_);
  // The same simulator from caller-provided state (mass may be empty: unit masses).
  DiskGalaxySimulator(SimParam params_, const ParticleData& pos_, const ParticleData& vel_,
                      const std::vector<coords_t>& mass = {});
  ~DiskGalaxySimulator() override;
  DiskGalaxySimulator(const DiskGalaxySimulator&) = delete;
  DiskGalaxySimulator& operator=(const DiskGalaxySimulator&) = delete;

  void stepSim() override;
  float getLastStepTime() override { return lastStepTime; }
  size_t getNumParticles() override { return params.numParticles; }
  const ParticleData& getParticlePos() override { return pos; }
  const ParticleData& getParticleVel() override { return vel; }
  const std::string* getDeviceName() override;
  int getGwSize() override { return params.gwSize; }
  CalculationMethod getCM() { return params.calcMethod; }

  // Device hand-off: current positions as float4 (x, y, z, m) into device memory.
  void devicePositions(float* xyzm_device, float* vel_xyzw_device = nullptr);
  nb_sim* handle() { return sim; }

 private:
  SimParam params;
  std::string devName;
  float lastStepTime{0.0f};
  ParticleData pos;
  ParticleData vel;
  nb_sim* sim = nullptr;

  void recvFromDevice();
};

}  // namespace simulation
