// Host-only stand-in for the CUDA runtime calls that the reference's
// DiskGalaxySimulator constructor makes, so that the reference's own initial-state
// code (src/simulator.cu:24-34 -> randomParticlePos, initialParticleVel,
// sendToDevice; :79-103, :131-158) runs unmodified on a machine without a GPU.
//
// TEST INFRASTRUCTURE ONLY: linked into oracle/_ref/ref_ic_dump (oracle/build_ref.sh),
// never into the library.  cudaMalloc and cudaMemcpy become host malloc and memcpy,
// so "device" buffers are host memory; registration of the reference's kernels is
// accepted and ignored; launching a kernel is refused (the constructor launches
// none).  Only names and signatures come from the CUDA headers.
#include <cuda.h>
#include <cuda_runtime_api.h>

#include <cstdlib>
#include <cstring>

extern "C" {

cudaError_t CUDARTAPI cudaMalloc(void** devPtr, size_t size) {
  *devPtr = std::malloc(size ? size : 1);
  return *devPtr ? cudaSuccess : cudaErrorMemoryAllocation;
}

cudaError_t CUDARTAPI cudaMemcpy(void* dst, const void* src, size_t count, enum cudaMemcpyKind) {
  std::memmove(dst, src, count);
  return cudaSuccess;
}

cudaError_t CUDARTAPI cudaDeviceSynchronize(void) { return cudaSuccess; }

const char* CUDARTAPI cudaGetErrorString(cudaError_t error) {
  return error == cudaSuccess ? "no error" : "host stand-in: not supported";
}

CUresult CUDAAPI cuDeviceGetName(char* name, int len, CUdevice) {
  if (name && len > 0) name[0] = '\0';
  return CUDA_ERROR_NO_DEVICE;
}

// Kernel registration (emitted by nvcc into every .cu object) and launches.
static void* g_handle = nullptr;
void** CUDARTAPI __cudaRegisterFatBinary(void*) { return &g_handle; }
void CUDARTAPI __cudaRegisterFatBinaryEnd(void**) {}
void CUDARTAPI __cudaUnregisterFatBinary(void**) {}
char CUDARTAPI __cudaInitModule(void**) { return 0; }
void CUDARTAPI __cudaRegisterFunction(void**, const char*, char*, const char*, int, uint3*,
                                      uint3*, dim3*, dim3*, int*) {}
unsigned CUDARTAPI __cudaPushCallConfiguration(dim3, dim3, size_t, struct CUstream_st*) {
  return 0;
}
cudaError_t CUDARTAPI __cudaPopCallConfiguration(dim3*, dim3*, size_t*, void*) {
  return cudaErrorNotSupported;
}
cudaError_t CUDARTAPI __cudaGetKernel(cudaKernel_t*, const void*) { return cudaErrorNotSupported; }
cudaError_t CUDARTAPI __cudaLaunchKernel(cudaKernel_t, dim3, dim3, void**, size_t, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // extern "C"
