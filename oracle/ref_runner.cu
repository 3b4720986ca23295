// ref_runner.cu -- runs the reference's own CUDA kernel on the GPU.
//
// TEST INFRASTRUCTURE ONLY (parity pin for the oracle and the library).
//
// oracle/build_ref.sh compiles the reference's src/simulator.cu, unmodified, into
// oracle/_ref/simulator_sm103a.cubin with the reference's release flag
// -use_fast_math (src/CMakeLists.txt:51).  This runner loads that cubin with the
// CUDA runtime's library API, finds particle_interaction<BRANCH|PREDICATED>
// (src/simulator.cu:186-229) by name, and drives it the way
// DiskGalaxySimulator::stepSim does (src/simulator.cu:47-75): grid
// ceil(N / gwSize) x gwSize, `iters` launches with a position-buffer swap after
// each, on SoA float arrays.
//
// The two structs below restate the kernel's by-value parameter types so that
// the argument bytes match: ParticleData_d holds three device pointers
// (src/simulator.cuh:87-98) and SimParam is the POD of src/sim_param.hpp:30-39
// (CalculationMethod is an int-sized enum class, sim_param.hpp:8-11).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>

namespace {

struct RefParticleData {
  float* x;
  float* y;
  float* z;
};

struct RefSimParam {
  float G;
  float dt;
  size_t numParticles;
  size_t numFrames;
  int simIterationsPerFrame;
  float damping;
  float distEps;
  int gwSize;
  int calcMethod;
};
static_assert(sizeof(RefSimParam) == 48, "SimParam layout");

void put_err(char* err, int len, const char* what, cudaError_t e) {
  if (err && len > 0) std::snprintf(err, len, "%s: %s", what, cudaGetErrorString(e));
}

}  // namespace

extern "C" int ref_run(const char* cubin, int method, int64_t n, float* x, float* y, float* z,
                       float* vx, float* vy, float* vz, int iters, float G, float dt,
                       float damping, float dist_eps, int gw_size, float* ms_out, char* err,
                       int errlen) {
#define CK(call)                 \
  do {                           \
    cudaError_t e_ = (call);     \
    if (e_ != cudaSuccess) {     \
      put_err(err, errlen, #call, e_); \
      return 1;                  \
    }                            \
  } while (0)
  if (n <= 0 || gw_size <= 0 || iters < 0) {
    if (err && errlen > 0) std::snprintf(err, errlen, "bad arguments");
    return 1;
  }
  cudaLibrary_t lib;
  CK(cudaLibraryLoadFromFile(&lib, cubin, nullptr, nullptr, 0, nullptr, nullptr, 0));
  unsigned count = 0;
  CK(cudaLibraryGetKernelCount(&count, lib));
  cudaKernel_t kernels[16];
  if (count > 16) count = 16;
  CK(cudaLibraryEnumerateKernels(kernels, count, lib));
  const char* want = method == 0 ? "CalculationMethod0E" : "CalculationMethod1E";
  cudaKernel_t k = nullptr;
  for (unsigned i = 0; i < count; ++i) {
    const char* name = nullptr;
    if (cudaFuncGetName(&name, reinterpret_cast<const void*>(kernels[i])) != cudaSuccess) continue;
    if (name && std::strstr(name, "particle_interaction") && std::strstr(name, want)) k = kernels[i];
  }
  if (!k) {
    if (err && errlen > 0) std::snprintf(err, errlen, "particle_interaction not found in cubin");
    cudaLibraryUnload(lib);
    return 1;
  }
  const size_t bytes = sizeof(float) * static_cast<size_t>(n);
  RefParticleData pos{}, next{}, vel{};
  float** bufs[9] = {&pos.x, &pos.y, &pos.z, &next.x, &next.y, &next.z, &vel.x, &vel.y, &vel.z};
  for (auto* b : bufs) CK(cudaMalloc(reinterpret_cast<void**>(b), bytes));
  CK(cudaMemcpy(pos.x, x, bytes, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(pos.y, y, bytes, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(pos.z, z, bytes, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(vel.x, vx, bytes, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(vel.y, vy, bytes, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(vel.z, vz, bytes, cudaMemcpyHostToDevice));
  RefSimParam p{};
  p.G = G;
  p.dt = dt;
  p.numParticles = static_cast<size_t>(n);
  p.numFrames = 1;
  p.simIterationsPerFrame = iters;
  p.damping = damping;
  p.distEps = dist_eps;
  p.gwSize = gw_size;
  p.calcMethod = method;
  const unsigned grid = static_cast<unsigned>((n - 1) / gw_size + 1);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0));
  for (int it = 0; it < iters; ++it) {
    void* args[4] = {&pos, &next, &vel, &p};
    CK(cudaLaunchKernel(reinterpret_cast<const void*>(k), dim3(grid), dim3(gw_size), args, 0,
                        nullptr));
    const RefParticleData t = pos;
    pos = next;
    next = t;
  }
  CK(cudaEventRecord(e1));
  CK(cudaEventSynchronize(e1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  if (ms_out) *ms_out = ms;
  CK(cudaMemcpy(x, pos.x, bytes, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(y, pos.y, bytes, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(z, pos.z, bytes, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(vx, vel.x, bytes, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(vy, vel.y, bytes, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(vz, vel.z, bytes, cudaMemcpyDeviceToHost));
  for (auto* b : bufs) cudaFree(*b);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaLibraryUnload(lib);
  return 0;
#undef CK
}
