/* Host-only stand-in for <cuda_runtime.h>, used solely to compile the
 * reference's ReadAndInitialOptions.cpp into the golden-vector generator.
 * That file's checkGPUMem/getGPUInfo diagnostics are never called (the
 * reference never calls them either) and read cudaDeviceProp fields that the
 * CUDA 13 headers no longer have; these stubs only let the file link. */
#ifndef ORACLE_REF_SHIM_CUDA_RUNTIME_H
#define ORACLE_REF_SHIM_CUDA_RUNTIME_H
#include <stddef.h>
typedef int cudaError_t;
struct cudaDeviceProp {
  char name[256];
  size_t totalGlobalMem, sharedMemPerBlock, totalConstMem, memPitch, texturePitchAlignment;
  int regsPerBlock, warpSize, maxThreadsPerBlock, maxThreadsDim[3], maxGridSize[3];
  int clockRate, memoryClockRate, memoryBusWidth, major, minor, multiProcessorCount, maxThreadsPerMultiProcessor;
};
static inline cudaError_t cudaSetDevice(int) { return 1; }
static inline cudaError_t cudaMemGetInfo(size_t* a, size_t* t) { *a = 0; *t = 0; return 1; }
static inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp*, int) { return 1; }
static inline cudaError_t cudaDriverGetVersion(int* v) { *v = 0; return 1; }
static inline cudaError_t cudaRuntimeGetVersion(int* v) { *v = 0; return 1; }
#endif
