// frontier.cuh -- drop-in for the reference's include/frontier.cuh.
//
// The user's generator writes the next frontier into a char byte map, so the
// byte maps stay; what changes is the level step:
//   Frontier<BDF>  (all push samples): current = queue, next = byte map.
//      Next() compacts the byte map into the queue with 16 flags per thread and
//      one queue reservation per warp, zeroing the map as it reads it, and
//      copies the count back once.  The reference pays a reset kernel, an n-
//      thread flag_to_wl, a memset and three blocking 4-byte copies per level
//      (src/worklist.cu:64-68,87-93; include/frontier.cuh:64-70).
//   Frontier<BITMAP> (pull samples): byte maps flag1/flag2 + finished flag, as
//      in the reference (include/frontier.cuh:77-127).
//   Frontier<BDF_AUTO>: queue or byte map by frontier size (th1, th2), with
//      the kernel dispatch fixed (the reference's switch falls through,
//      include/kernel.cuh:186-201).
//   Frontier<WL>: two queues.
// Byte maps are padded to whole 16-byte vectors (worklist::bytemap_bytes)
// and the padding is never set.  A Frontier is copied by value into kernel
// functors, so state that must be shared by every copy (the hub chunk list,
// pinned count) sits behind the `aux` pointer.
#ifndef GRUS_MGG_FRONTIER_CUH
#define GRUS_MGG_FRONTIER_CUH

#include <gflags/gflags.h>

#include <algorithm>

#include "common.cuh"
#include "print.cuh"
#include "timer.cuh"
#include "worklist.cuh"

DECLARE_double(wl_th);

namespace mgg {
namespace frontier {
using namespace intrinsics;
using namespace worklist;

// Shared by all copies of a frontier: the list of 4096-edge pieces of hub
// vertices produced by one expansion and consumed by the next launch.
struct FrontierAux {
  uint4 *chunks = nullptr;
  uint32_t chunk_cap = 0;
  vtx_t *ccount = nullptr;

  void ensure(uint64_t m, uint32_t huge, uint32_t piece) {
    const uint64_t need = m / piece + m / huge + 2;
    if (need <= chunk_cap) return;
    if (chunks) H_ERR(cudaFree(chunks));
    H_ERR(cudaMalloc(&chunks, need * sizeof(uint4)));
    chunk_cap = (uint32_t)need;
  }
};

inline char *alloc_bytemap(vtx_t n, int value) {
  char *p = nullptr;
  const size_t bytes = bytemap_bytes(n);
  H_ERR(cudaMalloc(&p, bytes));
  H_ERR(cudaMemsetAsync(p, 0, bytes, NULL));
  if (value) H_ERR(cudaMemsetAsync(p, value, n, NULL));
  return p;
}

inline FrontierAux *new_aux() {
  FrontierAux *a = new FrontierAux();
  H_ERR(cudaMalloc(&a->ccount, sizeof(vtx_t)));
  H_ERR(cudaMemsetAsync(a->ccount, 0, sizeof(vtx_t), NULL));
  return a;
}

inline int compact_grid(size_t nvec) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t warps = (nvec + 31) / 32;
  return (int)std::max<size_t>(1, std::min<size_t>((warps + 7) / 8, (size_t)sms * 8));
}

template <frontierType type>
class Frontier {
 public:
  Frontier();
  ~Frontier();
  void Init();
  void Next();
  __host__ vtx_t get_work_size_h();
};

template <>
class Frontier<BDF> {
 public:
  vtx_t numNode = 0;
  Worklist wl1, wl2;
  Worklist *wl_c = nullptr, *wl_n = nullptr;
  char *flag1 = nullptr, *flag2 = nullptr;
  vtx_t src = 0;
  vtx_t wl_sz = 1;
  vtx_t *flag_sz = nullptr;
  float active_perct = 0;
  float switch_th = 1.0;
  char *finished_d = nullptr;
  bool current_wl = true;
  FrontierAux *aux = nullptr;

  Frontier() {}
  ~Frontier() {}
  void Init(vtx_t _numNode, vtx_t _src = 0, int gpu_id = 0, float size_threshold = 1.0,
            bool _full = false) {
    numNode = _numNode;
    src = _src;
    switch_th = FLAGS_wl_th;
    (void)size_threshold;  // the queue always holds n (a level can activate every vertex)
    H_ERR(cudaSetDevice(gpu_id));
    flag2 = alloc_bytemap(numNode, 0);
    wl1.init(numNode);
    wl_c = &wl1;
    wl_n = &wl1;
    aux = new_aux();
    if (_full) {
      wl1.initFull(numNode);
      wl_sz = numNode;
    } else {
      wl1.add_item(src, 0);
      wl_sz = 1;
    }
  }
  void Next() {
    H_ERR(cudaMemsetAsync(wl1.count, 0, sizeof(vtx_t), NULL));
    const size_t nvec = bytemap_bytes(numNode) / 16;
    compact_bytemap<<<compact_grid(nvec), 256>>>(flag2, nvec, wl1.data, wl1.count, wl1.capacity, 1);
    H_ERR(cudaMemcpy(&wl_sz, wl1.count, sizeof(vtx_t), cudaMemcpyDeviceToHost));
    wl1.c_count = wl_sz;
  }
  __device__ vtx_t get_work_item(vtx_t id) { return wl1.data[id]; }
  __device__ vtx_t get_work_size() { return *wl1.count; }
  __host__ vtx_t get_work_size_h() { return wl_sz; }
  __device__ void add_work_item(vtx_t id) { wl1.append(id); }
  __host__ bool finish() { return wl_sz == 0; }
};

template <>
class Frontier<BITMAP> {
 public:
  vtx_t numNode = 0;
  char *flag1 = nullptr, *flag2 = nullptr;
  Worklist *wl_c = nullptr, *wl_n = nullptr;
  vtx_t src = 0;
  vtx_t wl_sz = 1;
  vtx_t *flag_sz = nullptr;
  float active_perct = 0;
  char *finished_d = nullptr, finished = false;
  FrontierAux *aux = nullptr;

  Frontier() {}
  ~Frontier() {}
  void Init(vtx_t _numNode, vtx_t _src = 0, int gpu_id = 0, float size_threshold = 1.0,
            bool _full = false) {
    (void)size_threshold;
    numNode = _numNode;
    src = _src;
    H_ERR(cudaSetDevice(gpu_id));
    flag1 = alloc_bytemap(numNode, _full ? 1 : 0);
    flag2 = alloc_bytemap(numNode, 0);
    if (!_full) H_ERR(cudaMemsetAsync(flag1 + src, 1, 1, NULL));
    H_ERR(cudaMalloc(&finished_d, 1));
    H_ERR(cudaMemset(finished_d, 1, 1));
    aux = new_aux();
  }
  void Next() {
    H_ERR(cudaMemcpy(&finished, finished_d, 1, cudaMemcpyDeviceToHost));
    H_ERR(cudaMemset(finished_d, 1, 1));
    std::swap(flag2, flag1);
    if (!finished) H_ERR(cudaMemsetAsync(flag2, 0, bytemap_bytes(numNode), NULL));
  }
  __host__ vtx_t get_work_size_h() { return finished ? 0 : 1; }
  __host__ bool finish() { return finished; }
};

template <>
class Frontier<WL> {
 public:
  vtx_t numNode = 0;
  Worklist wl1, wl2;
  Worklist *wl_c = nullptr, *wl_n = nullptr;
  char *flag = nullptr;
  vtx_t src = 0;
  vtx_t wl_sz = 1;
  vtx_t *flag_sz = nullptr;
  float active_perct = 0;
  char *finished_d = nullptr;
  FrontierAux *aux = nullptr;

  Frontier() {}
  ~Frontier() {}
  void Init(vtx_t _numNode, vtx_t _src = 0, int gpu_id = 0, float size_threshold = 1.0,
            bool _full = false) {
    (void)size_threshold;
    numNode = _numNode;
    src = _src;
    H_ERR(cudaSetDevice(gpu_id));
    wl1.init(numNode);
    wl2.init(numNode);
    wl_c = &wl1;
    wl_n = &wl2;
    aux = new_aux();
    if (_full) {
      wl1.initFull(numNode);
      wl_sz = numNode;
    } else {
      wl_c->add_item(src, 0);
      wl_sz = 1;
    }
  }
  // The push kernel appends to wl_n with the user's generator; a vertex may be
  // appended more than once (the reference's semantics, generator-defined).
  void Next() {
    std::swap(wl_c, wl_n);
    wl_n->reset();
    wl_sz = wl_c->get_sz();
  }
  __device__ vtx_t get_work_item(vtx_t id) { return wl_c->data[id]; }
  __host__ vtx_t get_work_size_h() { return wl_sz; }
  __host__ bool finish() { return wl_sz == 0; }
};

template <>
class Frontier<BDF_AUTO> {
 public:
  vtx_t numNode = 0;
  Worklist wl1, wl2;
  Worklist *wl_c = nullptr, *wl_n = nullptr;
  char *flag1 = nullptr, *flag2 = nullptr;
  vtx_t src = 0;
  vtx_t wl_sz = 1;
  vtx_t *flag_sz = nullptr;
  float active_perct = 0;
  float switch_th = 1.0;
  float th1 = 0.00000005f, th2 = 0.9f;
  char *finished_d = nullptr;
  bool current_wl = true;
  frontierType current_f = WL;
  FrontierAux *aux = nullptr;

  Frontier() {}
  ~Frontier() {}
  void Init(vtx_t _numNode, vtx_t _src = 0, int gpu_id = 0, float size_threshold = 1.0,
            bool _full = false) {
    (void)size_threshold;
    numNode = _numNode;
    src = _src;
    switch_th = FLAGS_wl_th;
    H_ERR(cudaSetDevice(gpu_id));
    flag1 = alloc_bytemap(numNode, _full ? 1 : 0);
    flag2 = alloc_bytemap(numNode, 0);
    wl1.init(numNode);
    wl2.init(numNode);
    wl_c = &wl1;
    wl_n = &wl2;
    aux = new_aux();
    if (_full) {
      current_f = BITMAP;
      wl_sz = numNode;
    } else {
      current_f = WL;
      wl_c->add_item(src, 0);
      wl_sz = 1;
    }
  }
  // After a level the next frontier is in flag2 (BDF / BITMAP levels) or in
  // wl_n (WL levels).  It becomes the current queue, flag1 mirrors it when the
  // next level runs over the byte map, and the representation is chosen by
  // the size thresholds of include/frontier.cuh:140,206-215.
  void Next() {
    const size_t nvec = bytemap_bytes(numNode) / 16;
    if (current_f == WL) {
      std::swap(wl_c, wl_n);
      wl_n->reset();
    } else {
      H_ERR(cudaMemsetAsync(wl_n->count, 0, sizeof(vtx_t), NULL));
      H_ERR(cudaMemsetAsync(flag1, 0, bytemap_bytes(numNode), NULL));
      std::swap(flag1, flag2);  // flag1 = next frontier as a byte map
      compact_bytemap<<<compact_grid(nvec), 256>>>(flag1, nvec, wl_n->data, wl_n->count,
                                                   wl_n->capacity, 0);
      std::swap(wl_c, wl_n);
      wl_n->reset();
    }
    wl_sz = wl_c->get_sz();
    if (wl_sz < numNode * th1) current_f = WL;
    else if (wl_sz > numNode * th2) current_f = BITMAP;
    else current_f = BDF;
    if (current_f == BITMAP) {
      // flag1 must hold the current frontier: rebuild it from the queue
      H_ERR(cudaMemsetAsync(flag1, 0, bytemap_bytes(numNode), NULL));
      wl_to_flag<<<wl_sz / BLOCK_SIZE + 1, BLOCK_SIZE>>>(*wl_c, flag1, wl_sz);
    }
  }
  __host__ vtx_t get_work_size_h() { return wl_sz; }
  __host__ bool finish() { return wl_sz == 0; }
};

}  // namespace frontier
}  // namespace mgg
#endif
