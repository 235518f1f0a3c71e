// intrinsics.cuh -- drop-in for the reference's include/intrinsics.cuh:
// atomicAggInc (one atomic per group of converged lanes), wtime, dArrayInit
// and a device summary printer.  The reference's x86 rdtsc helpers are not
// provided (the GB300 host is aarch64); query_device_prop prints only fields
// that still exist in CUDA 13.
#ifndef GRUS_MGG_INTRINSICS_CUH
#define GRUS_MGG_INTRINSICS_CUH

#include <cooperative_groups.h>
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>

#include <chrono>

using namespace cooperative_groups;

namespace intrinsics {

inline void query_device_prop(int nDevices) {
  for (int i = 0; i < nDevices; i++) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, i) != cudaSuccess) continue;
    printf("Device Number: %d\n Device name: %s\n Device Capability: %d.%d\n", i, prop.name,
           prop.major, prop.minor);
    printf(" Total Global Memory (GB): %.2f\n SMs: %d\n L2 (MB): %.1f\n", prop.totalGlobalMem / 1073741824.0,
           prop.multiProcessorCount, prop.l2CacheSize / 1048576.0);
  }
}

inline double wtime() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static __global__ void dArrayInit(unsigned *ctr, unsigned n, unsigned k = 0) {
  for (unsigned tid = blockDim.x * blockIdx.x + threadIdx.x; tid < n; tid += blockDim.x * gridDim.x)
    ctr[tid] = k;
}

// One atomicAdd per group of lanes that arrive together; each lane gets its
// own slot (the reference's include/intrinsics.cuh:96-103 contract).
__device__ __forceinline__ unsigned atomicAggInc(unsigned *ctr) {
  coalesced_group g = coalesced_threads();
  unsigned base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(ctr, g.size());
  return g.shfl(base, 0) + g.thread_rank();
}

}  // namespace intrinsics
#endif
