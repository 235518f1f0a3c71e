// ref_pin_shim.h -- force-included when oracle/ref_pin.cu is compiled against
// the reference's own include/ directory (test infrastructure only).
//
// It lets the reference's HOST code (graph_loader::ReadGraphGR and
// csr_tocsc) build with CUDA 13 and run on a machine without a GPU:
//   * CUDA 13 removed two cudaDeviceProp fields read by the dead
//     query_device_prop (include/intrinsics.cuh:41,48,50); they are mapped
//     onto a field that still exists;
//   * CUDA 13 takes a cudaMemLocation in cudaMemPrefetchAsync/cudaMemAdvise;
//     the int-device overloads used by Set_Mem_Policy (include/graph.cuh:175-248)
//     forward to them (compiled, never executed by the pin);
//   * cudaMallocManaged is redirected to zeroed host memory, so the loader's
//     "managed" arrays live on the host (zeroed like fresh managed pages, which
//     the reference relies on for xadj[0], graph_loader.cuh:114-119).
#pragma once
#include <cuda_runtime.h>
#include <cstdlib>

#define deviceOverlap memoryBusWidth
#define memoryClockRate memoryBusWidth

static inline cudaError_t cudaMemPrefetchAsync(const void *p, size_t n, int dev,
                                               cudaStream_t s) {
  cudaMemLocation loc{};
  loc.type = cudaMemLocationTypeDevice;
  loc.id = dev;
  return cudaMemPrefetchAsync(p, n, loc, 0u, s);
}
static inline cudaError_t cudaMemAdvise(const void *p, size_t n,
                                        cudaMemoryAdvise a, int dev) {
  cudaMemLocation loc{};
  loc.type = cudaMemLocationTypeDevice;
  loc.id = dev;
  return cudaMemAdvise(p, n, a, loc);
}

template <typename T>
static inline cudaError_t grus_pin_host_managed(T **p, size_t bytes,
                                                unsigned = 0) {
  *p = (T *)std::calloc(bytes ? bytes : 1, 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
#define cudaMallocManaged grus_pin_host_managed
