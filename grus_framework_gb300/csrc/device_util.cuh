// device_util.cuh -- device-side building blocks shared by libgrus and the
// header-only mgg drop-in: lane helpers, L2-only loads for data other SMs
// write during a persistent launch, bitmap tests, warp-aggregated
// reservation, block sums, and a grid barrier whose waits end after a time
// limit with an error bit instead of spinning forever.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace grus {

// Device-side error bits, OR-ed into a workspace word and turned into a
// status code by the host after the launch completes.
enum : uint32_t {
  kErrTimeout = 1u << 0,   // a grid-barrier wait ran past its limit
  kErrOverflow = 1u << 1,  // a queue or chunk list would have overflowed
  kErrLevels = 1u << 2,    // level counter passed its bound
  kErrAborted = 1u << 3,   // a CTA left a grid barrier because another CTA's
                           // wait had run past its limit
};

// ---- device helpers ------------------------------------------------------
__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// L2-only load (ld.global.cg): for data written by other SMs in the same
// persistent launch, where an L1 line could be stale.
__device__ __forceinline__ uint32_t ld_cg(const uint32_t *p) { return __ldcg(p); }

__device__ __forceinline__ bool test_bit(const uint32_t *bm, uint32_t v) {
  return (__ldcg(bm + (v >> 5)) >> (v & 31u)) & 1u;
}

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint64_t ld_acquire_u64(const unsigned long long *p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Warp-aggregated append: one atomicAdd per group of lanes that reach the
// call together (coalesced_threads), the same idea as the reference's
// atomicAggInc (include/intrinsics.cuh:96-103).
__device__ __forceinline__ uint32_t agg_reserve(uint32_t *counter) {
  namespace cg = cooperative_groups;
  cg::coalesced_group g = cg::coalesced_threads();
  uint32_t base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(counter, g.size());
  return g.shfl(base, 0) + g.thread_rank();
}

// Grid barrier for cooperative (co-resident) launches.  Every wait is
// bounded: past `timeout_ns` the waiting CTA raises the shared abort flag and
// kErrTimeout, and every CTA then returns false so the kernel exits cleanly;
// a CTA that leaves because it saw the flag adds kErrAborted, so a launch cut
// short never reads as a success.  A launch that timed out leaves the flag
// and a stale arrival count behind, so the host clears the barrier and the
// error word in the launch's stream before every launch on them (a stale
// count would otherwise let a later episode complete early).
// The arrival counter sits alone on one 128-byte line and the generation and
// abort words on the next: the CTAs polling the generation then do not queue
// behind the arrivals' atomics at the same L2 line (measured with 1,216
// CTAs: 5.1 -> 3.5 us per barrier; 608 CTAs: 3.2 -> 2.7 us).  Control blocks
// place it on a 128-byte boundary.
struct GridBarrier {
  uint32_t count;
  uint32_t pad0[31];
  uint32_t gen;
  uint32_t abort;
  uint32_t pad1[30];
};
static_assert(sizeof(GridBarrier) == 256, "grid barrier spans two 128-byte lines");

__device__ __forceinline__ bool grid_sync(GridBarrier *bar, uint32_t *err,
                                          uint64_t timeout_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const uint32_t gen = ld_acquire_u32(&bar->gen);
    __threadfence();
    const uint32_t arrived = atomicAdd(&bar->count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(&bar->count, 0u);
      __threadfence();
      atomicAdd(&bar->gen, 1u);
    } else {
      const uint64_t t0 = global_timer_ns();
      uint32_t spins = 0;
      while (ld_acquire_u32(&bar->gen) == gen) {
        if (ld_acquire_u32(&bar->abort)) {
          atomicOr(err, kErrAborted);
          ok = 0;
          break;
        }
        __nanosleep(40);
        if ((++spins & 255u) == 0 && global_timer_ns() - t0 > timeout_ns) {
          atomicExch(&bar->abort, 1u);
          atomicOr(err, kErrTimeout);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Block-wide sum of a per-thread 64-bit value; result valid in thread 0.
template <int kBlock>
__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v) {
  __shared__ unsigned long long s_part[kBlock / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane_id() == 0) s_part[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned long long t = 0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < kBlock / 32 ? s_part[threadIdx.x] : 0ull;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;
}

// Block-wide exclusive scan of one value per thread; *total gets the sum.
// Must be called by every thread of the block.
template <int kBlock>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t s_warp[kBlock / 32];
  __shared__ uint32_t s_total;
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if ((int)lane >= o) incl += t;
  }
  __syncthreads();
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kBlock / 32 ? s_warp[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if ((int)lane >= o) wi += t;
    }
    if (lane < kBlock / 32) s_warp[lane] = wi - w;
    if (lane == 31) s_total = wi;
  }
  __syncthreads();
  *total = s_total;
  return s_warp[warp] + incl - v;
}

}  // namespace grus
