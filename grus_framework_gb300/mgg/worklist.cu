// worklist.cu -- host methods and helper kernels of the mgg drop-in worklist.
// Compile this file in place of the reference's src/worklist.cu.
#include "worklist.cuh"

namespace mgg {
namespace worklist {

__global__ void worklist_add(Worklist wl, vtx_t item) {
  if (blockDim.x * blockIdx.x + threadIdx.x == 0) wl.append(item);
}

__global__ void worklist_init_full(Worklist wl, vtx_t n) {
  for (size_t id = blockDim.x * (size_t)blockIdx.x + threadIdx.x; id < n;
       id += (size_t)gridDim.x * blockDim.x)
    wl.data[id] = (vtx_t)id;
  if (blockIdx.x == 0 && threadIdx.x == 0) *wl.count = n;
}

void Worklist::init(vtx_t capacity_p, cudaStream_t stream) {
  capacity = capacity_p;
  c_count = 0;
  H_ERR(cudaMalloc(&data, (size_t)(capacity ? capacity : 1) * sizeof(vtx_t)));
  H_ERR(cudaMalloc(&count, sizeof(vtx_t)));
  H_ERR(cudaMemsetAsync(count, 0, sizeof(vtx_t), stream));
}

void Worklist::free() {
  H_ERR(cudaFree(data));
  H_ERR(cudaFree(count));
  data = count = nullptr;
}

void Worklist::initFull(vtx_t n) {
  worklist_init_full<<<n / BLOCK_SIZE + 1, BLOCK_SIZE>>>(*this, n);
  c_count = n;
}

// The device count keeps growing when appends overflow (they are dropped, not
// written), so every host read is clamped to the capacity.
vtx_t Worklist::get_sz() {
  H_ERR(cudaMemcpy(&c_count, count, sizeof(vtx_t), cudaMemcpyDeviceToHost));
  if (c_count > capacity) c_count = capacity;
  return c_count;
}

vtx_t Worklist::get_sz(cudaStream_t stream) {
  H_ERR(cudaMemcpyAsync(&c_count, count, sizeof(vtx_t), cudaMemcpyDeviceToHost, stream));
  H_ERR(cudaStreamSynchronize(stream));
  if (c_count > capacity) c_count = capacity;
  return c_count;
}

void Worklist::grow(size_t cap) {
  if (cap <= capacity) return;
  vtx_t *fresh = nullptr;
  H_ERR(cudaMalloc(&fresh, cap * sizeof(vtx_t)));
  H_ERR(cudaMemcpy(fresh, data, (size_t)capacity * sizeof(vtx_t), cudaMemcpyDeviceToDevice));
  H_ERR(cudaFree(data));
  data = fresh;
  capacity = (vtx_t)cap;
}

void Worklist::reset() {
  H_ERR(cudaMemsetAsync(count, 0, sizeof(vtx_t)));
  creset();
}

void Worklist::add_item(vtx_t item, cudaStream_t stream) {
  worklist_add<<<1, 32, 0, stream>>>(*this, item);
}

__global__ void flag_to_wl(Worklist wl, char *flag1, vtx_t size) {
  const size_t tid = blockDim.x * (size_t)blockIdx.x + threadIdx.x;
  const bool set = tid < size && flag1[tid];
  const unsigned mask = __ballot_sync(0xffffffffu, set);
  if (!mask) return;
  const unsigned lane = threadIdx.x & 31u;
  unsigned base = 0;
  if (lane == 0) base = atomicAdd(wl.count, (vtx_t)__popc(mask));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (set) {
    const unsigned at = base + __popc(mask & ((1u << lane) - 1u));
    if (at < wl.capacity) wl.data[at] = (vtx_t)tid;
  }
}

// Bounds are the queue length (the reference bounds by n, src/worklist.cu:94-100).
__global__ void wl_to_flag(Worklist wl, char *flag1, vtx_t size) {
  const size_t tid = blockDim.x * (size_t)blockIdx.x + threadIdx.x;
  const vtx_t len = min(*wl.count, wl.capacity);
  if (tid < size && tid < len) flag1[wl.data[tid]] = 1;
}

__global__ void flag_to_wl_remote_local(Worklist wl_remote, Worklist wl_local, char *flag_local,
                                        char *flag_active, vtx_t size) {
  const size_t tid = blockDim.x * (size_t)blockIdx.x + threadIdx.x;
  if (tid < size && flag_active[tid]) {
    if (flag_local[tid]) wl_local.warp_append((vtx_t)tid);
    else wl_remote.warp_append((vtx_t)tid);
  }
}

__global__ void compute_lookup_buffer(vtx_t *vtx, vtx_t *vtx_ptr, vtx_t *xadj,
                                      uint *lookup_buffer, uint *outDegree, vtx_t size) {
  const size_t tid = blockDim.x * (size_t)blockIdx.x + threadIdx.x;
  if (tid < size) {
    lookup_buffer[vtx[tid]] = (uint)tid;
    outDegree[tid] = xadj[vtx[tid] + 1] - xadj[vtx[tid]];
  }
}

__global__ void get_flag_num(char *flag1, vtx_t size, vtx_t *num) {
  const size_t tid = blockDim.x * (size_t)blockIdx.x + threadIdx.x;
  const unsigned mask = __ballot_sync(0xffffffffu, tid < size && flag1[tid]);
  if ((threadIdx.x & 31u) == 0 && mask) atomicAdd(num, (vtx_t)__popc(mask));
}

// 16 flags per thread: the 4 words' nonzero bytes give a 16-bit mask, a warp
// exclusive scan of the popcounts places each thread's indices, and lane 0
// reserves the warp's total with one atomicAdd.
__global__ void compact_bytemap(char *flag, size_t nvec, vtx_t *out, vtx_t *count,
                                vtx_t capacity, int clear) {
  uint4 *vec = reinterpret_cast<uint4 *>(flag);
  const unsigned lane = threadIdx.x & 31u;
  const size_t warp = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t base = warp * 32; base < nvec; base += nwarps * 32) {
    const size_t i = base + lane;
    uint4 q = make_uint4(0, 0, 0, 0);
    if (i < nvec) q = vec[i];
    const unsigned w[4] = {q.x, q.y, q.z, q.w};
    unsigned m16 = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const unsigned ne = __vcmpne4(w[k], 0u);  // 0xFF per nonzero byte
      m16 |= (((ne >> 7) & 1u) | ((ne >> 14) & 2u) | ((ne >> 21) & 4u) | ((ne >> 28) & 8u)) << (4 * k);
    }
    const unsigned c = __popc(m16);
    unsigned incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)lane >= o) incl += t;
    }
    const unsigned total = __shfl_sync(0xffffffffu, incl, 31);
    if (!total) continue;
    unsigned wbase = 0;
    if (lane == 0) wbase = atomicAdd(count, total);
    wbase = __shfl_sync(0xffffffffu, wbase, 0);
    unsigned at = wbase + incl - c;
    unsigned mm = m16;
    while (mm) {
      const int b = __ffs(mm) - 1;
      mm &= mm - 1;
      if (at < capacity) out[at] = (vtx_t)(i * 16 + b);
      ++at;
    }
    if (clear && m16) vec[i] = make_uint4(0, 0, 0, 0);
  }
}

}  // namespace worklist
}  // namespace mgg
