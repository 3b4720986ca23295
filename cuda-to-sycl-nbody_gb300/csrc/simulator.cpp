// simulation::DiskGalaxySimulator over the C ABI.
#include "simulator.hpp"

#include <string>

namespace {

void check(int status, const char* what) {
  if (status != NB_OK)
    throw std::runtime_error(std::string(what) + ": " + nb_status_string(status) + ": " +
                             nb_last_error());
}

}  // namespace

SimParam::SimParam() {
  nb_params p;
  nb_params_default(&p);
  G = p.G;
  dt = p.dt;
  numParticles = p.num_particles;
  numFrames = p.num_frames;
  simIterationsPerFrame = p.iters_per_frame;
  damping = p.damping;
  distEps = p.dist_eps;
  gwSize = p.gw_size;
  calcMethod = CalculationMethod::BRANCH;
  accumulator = p.accumulator;
}

void SimParam::parseArgs(int argc, char** argv) {
  nb_params p = toC();
  const int st = nb_params_parse_args(&p, argc, argv);
  if (st == NB_ERR_INVALID_ARGUMENT && argc >= 10)
    throw std::invalid_argument(nb_last_error());  // sim_param.cpp:36
  check(st, "SimParam::parseArgs");
  G = p.G;
  dt = p.dt;
  numParticles = p.num_particles;
  numFrames = p.num_frames;
  simIterationsPerFrame = p.iters_per_frame;
  damping = p.damping;
  distEps = p.dist_eps;
  gwSize = p.gw_size;
  calcMethod = p.calc_method == NB_PREDICATED ? CalculationMethod::PREDICATED
                                              : CalculationMethod::BRANCH;
}

nb_params SimParam::toC() const {
  nb_params p;
  nb_params_default(&p);
  p.G = G;
  p.dt = dt;
  p.num_particles = numParticles;
  p.num_frames = numFrames;
  p.iters_per_frame = simIterationsPerFrame;
  p.damping = damping;
  p.dist_eps = distEps;
  p.gw_size = gwSize;
  p.calc_method = calcMethod == CalculationMethod::PREDICATED ? NB_PREDICATED : NB_BRANCH;
  p.accumulator = accumulator;
  return p;
}

namespace simulation {

DiskGalaxySimulator::DiskGalaxySimulator(SimParam params_)
    : params(params_), pos(params_.numParticles), vel(params_.numParticles) {
  const nb_params p = params.toC();
  check(nb_sim_create_disk_galaxy(&p, &sim), "DiskGalaxySimulator");
  recvFromDevice();
}

DiskGalaxySimulator::DiskGalaxySimulator(SimParam params_, const ParticleData& pos_,
                                         const ParticleData& vel_,
                                         const std::vector<coords_t>& mass)
    : params(params_), pos(pos_), vel(vel_) {
  const nb_params p = params.toC();
  check(nb_sim_create(&p, pos.x.data(), pos.y.data(), pos.z.data(), vel.x.data(), vel.y.data(),
                      vel.z.data(), mass.empty() ? nullptr : mass.data(), &sim),
        "DiskGalaxySimulator");
}

DiskGalaxySimulator::~DiskGalaxySimulator() { nb_sim_destroy(sim); }

void DiskGalaxySimulator::stepSim() {
  check(nb_sim_step(sim), "stepSim");
  check(nb_sim_last_step_ms(sim, &lastStepTime), "stepSim");
  recvFromDevice();  // the reference copies the state back every step (simulator.cu:74)
}

const std::string* DiskGalaxySimulator::getDeviceName() {
  if (devName.empty()) {
    char buf[256];
    devName = nb_device_name(buf, sizeof(buf)) == NB_OK ? buf : "Unknown Device";
  }
  return &devName;
}

void DiskGalaxySimulator::devicePositions(float* xyzm_device, float* vel_xyzw_device) {
  check(nb_sim_export_device(sim, xyzm_device, vel_xyzw_device), "devicePositions");
}

void DiskGalaxySimulator::recvFromDevice() {
  check(nb_sim_get_state(sim, pos.x.data(), pos.y.data(), pos.z.data(), vel.x.data(),
                         vel.y.data(), vel.z.data()),
        "recvFromDevice");
}

}  // namespace simulation
