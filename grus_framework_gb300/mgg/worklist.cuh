// worklist.cuh -- drop-in for the reference's include/worklist.cuh.
//
// Worklist: a device vertex queue (data, count) with the reference's
// interface (include/worklist.cuh:15-85): append (one atomic per item),
// warp_append (one atomic per converged group), host get_sz/reset/add_item/
// initFull.  Differences, all invisible to the samples: `data` is device
// memory rather than managed memory, and the host methods are defined in
// mgg/worklist.cu (compiled in place of the reference's src/worklist.cu).
// The compaction kernels read the byte map as 16-byte vectors and reserve
// queue slots once per warp (ballot/popc), see worklist.cu.
#ifndef GRUS_MGG_WORKLIST_CUH
#define GRUS_MGG_WORKLIST_CUH

#include "common.cuh"
#include "intrinsics.cuh"

using namespace intrinsics;
#define WARP_SIZE 32

namespace mgg {
namespace worklist {

class Worklist {
 public:
  vtx_t *data = nullptr;
  vtx_t *count = nullptr;
  vtx_t c_count = 0;
  vtx_t capacity = 0;

  __host__ Worklist(vtx_t capacity_p) { init(capacity_p); }
  __host__ Worklist() {}
  __host__ void init(vtx_t capacity_p, cudaStream_t stream = NULL);
  __host__ void free();
  __host__ void initFull(vtx_t n);
  __host__ vtx_t get_sz();
  __host__ vtx_t get_sz(cudaStream_t stream);
  __host__ void reset();
  __host__ void add_item(vtx_t item, cudaStream_t stream);
  __host__ void creset() { c_count = 0; }
  // Enlarges the buffer (keeping its contents) to at least `cap` items.
  __host__ void grow(size_t cap);

  __device__ __forceinline__ void append(const vtx_t &item) {
    const vtx_t at = atomicAdd((vtx_t *)count, 1u);
    if (at < capacity) data[at] = item;
  }
  __device__ __forceinline__ void warp_append(const vtx_t &item) {
    const vtx_t at = atomicAggInc((vtx_t *)count);
    if (at < capacity) data[at] = item;
  }
  __device__ __forceinline__ void append_all(vtx_t *cache, const vtx_t length) {
    const vtx_t at = atomicAdd((vtx_t *)count, length);
    for (vtx_t i = 0; i < length && at + i < capacity; i++) data[at + i] = cache[i];
  }
  __device__ __forceinline__ void reset_d() const { *count = 0; }
  __device__ __forceinline__ vtx_t read(vtx_t i) const { return data[i]; }
  __device__ __forceinline__ vtx_t size() const { return min(*count, capacity); }
  __device__ __forceinline__ void assign(vtx_t i, vtx_t t) const { data[i] = t; }
};

// Kernels of the reference's src/worklist.cu, same signatures.
__global__ void flag_to_wl(Worklist wl, char *flag1, vtx_t size);
__global__ void wl_to_flag(Worklist wl, char *flag1, vtx_t size);
__global__ void flag_to_wl_remote_local(Worklist wl_remote, Worklist wl_local, char *flag_local,
                                        char *flag_active, vtx_t size);
__global__ void compute_lookup_buffer(vtx_t *vtx, vtx_t *vtx_ptr, vtx_t *xadj,
                                      uint *lookup_buffer, uint *outDegree, vtx_t size);
__global__ void get_flag_num(char *flag1, vtx_t size, vtx_t *num);

// Byte map -> queue, 16 flags per thread, one reservation per warp; when
// `clear` is set the words read are zeroed (the map is ready for the next
// level without a separate memset).  `nvec` counts 16-byte vectors.
__global__ void compact_bytemap(char *flag, size_t nvec, vtx_t *out, vtx_t *count,
                                vtx_t capacity, int clear);

// Bytes of a byte map for n vertices, rounded up to whole 16-byte vectors.
inline size_t bytemap_bytes(size_t n) { return (n + 15) / 16 * 16 + 16; }

}  // namespace worklist
}  // namespace mgg
#endif
