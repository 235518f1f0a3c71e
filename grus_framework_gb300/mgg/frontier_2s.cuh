// frontier_2s.cuh -- drop-in for the reference's include/frontier_2s.cuh:
// the frontier of the two-stage BFS, split into "local" vertices (expanded
// over the previous active subgraph) and "remote" ones (whose rows are
// gathered into a new subgraph).  Next() follows the reference
// (include/frontier_2s.cuh:67-97): the last remote list becomes the local
// marker map, the next frontier (flag2) is split by that map, and the maps
// are cleared.  Differences: the count of active flags lives in the shared
// aux block (the reference cudaMallocs a counter on every level, :73), and
// wl_to_flag is bounded by the list length (the reference bounds by n).
#ifndef GRUS_MGG_FRONTIER_2S_CUH
#define GRUS_MGG_FRONTIER_2S_CUH

#include <gflags/gflags.h>

#include "common.cuh"
#include "frontier.cuh"
#include "print.cuh"
#include "timer.cuh"
#include "worklist.cuh"

DECLARE_double(wl_th);

namespace mgg {
namespace frontier {

template <frontierType type>
class Frontier_2S {
 public:
  Frontier_2S();
  ~Frontier_2S();
  void Init();
  void Next();
  __host__ vtx_t get_work_size_h();
};

template <>
class Frontier_2S<BDF> {
 public:
  vtx_t numNode = 0;
  Worklist wl1, wl2;
  Worklist *wl_remote = nullptr, *wl_local = nullptr;
  char *flag1 = nullptr, *flag2 = nullptr, *flag_local = nullptr;
  vtx_t src = 0;
  vtx_t wl_sz = 1, wl_sz_remote = 1, wl_sz_local = 0;
  vtx_t *flag_sz = nullptr;
  float active_perct = 0;
  float switch_th = 1.0;
  char *finished_d = nullptr;
  bool current_wl = true;
  FrontierAux *aux = nullptr;

  Frontier_2S() {}
  ~Frontier_2S() {}
  void Init(vtx_t _numNode, vtx_t _src = 0, int gpu_id = 0, float size_threshold = 1.0,
            bool _full = false) {
    (void)size_threshold;
    numNode = _numNode;
    src = _src;
    switch_th = FLAGS_wl_th;
    H_ERR(cudaSetDevice(gpu_id));
    flag_local = alloc_bytemap(numNode, 0);
    flag2 = alloc_bytemap(numNode, 0);
    wl1.init(numNode);
    wl2.init(numNode);
    wl_remote = &wl1;
    wl_local = &wl2;
    H_ERR(cudaMalloc(&flag_sz, sizeof(vtx_t)));
    aux = new_aux();
    if (_full) {
      wl_remote->initFull(numNode);
      wl_sz_remote = numNode;
    } else {
      wl_remote->add_item(src, 0);
    }
  }
  void Next() {
    // previous remote vertices now have their rows in the last subgraph
    wl_to_flag<<<wl_sz_remote / BLOCK_SIZE + 1, BLOCK_SIZE>>>(*wl_remote, flag_local, wl_sz_remote);
    wl_remote->reset();
    wl_local->reset();
    flag_to_wl_remote_local<<<numNode / BLOCK_SIZE + 1, BLOCK_SIZE>>>(*wl_remote, *wl_local, flag_local,
                                                                      flag2, numNode);
    H_ERR(cudaMemsetAsync(flag_local, 0, bytemap_bytes(numNode), NULL));
    H_ERR(cudaMemsetAsync(flag2, 0, bytemap_bytes(numNode), NULL));
    wl_sz_remote = wl_remote->get_sz();
    wl_sz_local = wl_local->get_sz();
    wl_sz = wl_sz_remote + wl_sz_local;
  }
  __device__ vtx_t get_work_size_remote() { return *wl_remote->count; }
  __device__ vtx_t get_work_size_local() { return *wl_local->count; }
  __host__ vtx_t get_work_size_local_h() { return wl_local->get_sz(); }
  __host__ vtx_t get_work_size_remote_h() { return wl_remote->get_sz(); }
  __host__ vtx_t get_work_size_totoal_h() { return wl_sz; }
  __host__ bool finish() { return wl_sz == 0; }
};

}  // namespace frontier
}  // namespace mgg
#endif
