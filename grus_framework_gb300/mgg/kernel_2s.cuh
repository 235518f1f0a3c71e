// kernel_2s.cuh -- drop-in for the reference's include/kernel_2s.cuh: the
// two-stage expansion of bfs_2s (kernel_2s::operator(), :73-91): expand the
// local list over the previous subgraph, build the subgraph of the remote
// list, expand the remote list over it.  The user's functors run in the
// degree-binned expansion (csrc/expand.cuh) over the compact subgraph rows;
// the owner's row is found through the subgraph's lookup (the reference
// reads the degree of the warp index instead of the local index,
// kernel_2s.cuh:51).  edge_id indexes the subgraph's edge array, as in the
// reference.
#ifndef GRUS_MGG_KERNEL_2S_CUH
#define GRUS_MGG_KERNEL_2S_CUH

#include <cuda.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "frontier_2s.cuh"
#include "graph.cuh"
#include "kernel.cuh"
#include "subgraph.cuh"
#include "worklist.cuh"

namespace mgg {
namespace detail {

template <typename U, typename Gen, typename J>
struct SubgraphToFlag {
  const vtx_t *edges;
  char *flag;
  J job;
  using aux_t = uint32_t;
  __device__ __forceinline__ uint32_t aux(uint32_t) const { return 0u; }
  __device__ __forceinline__ void edge(uint32_t src, uint32_t, uint32_t x) {
    U updater;
    Gen generator;
    const vtx_t dst = edges[x];
    generator(updater(src, dst, x, job), flag, dst);
  }
};

// Queue of global ids; rows come from the subgraph through its lookup.
template <class Vis>
__global__ void __launch_bounds__(kBlock)
    expand_subgraph(const vtx_t *queue, const vtx_t *qcount_d, vtx_t qcap, const vtx_t *lookup,
                    const vtx_t *vtx_ptr, Vis vis) {
  const vtx_t qcount = min(*qcount_d, qcap);
  for (uint32_t base = blockIdx.x * kBlock; base < qcount; base += gridDim.x * kBlock) {
    const uint32_t i = base + threadIdx.x;
    vtx_t v = 0, beg = 0, end = 0;
    if (i < qcount) {
      v = queue[i];
      const vtx_t local = lookup[v];
      beg = vtx_ptr[local];
      end = vtx_ptr[local + 1];
    }
    grus::expand_tile<kBlock>(v, beg, end, 0u, vis);
  }
}

}  // namespace detail

template <typename graph_t, typename subgraph_t, typename frontier_t, typename updater_t,
          typename generator_t, typename job_t>
class kernel_2s {
 public:
  void operator()(graph_t G, subgraph_t SG1, subgraph_t SG2, frontier_t F, job_t job) {}
};

template <typename graph_t, typename updater_t, typename generator_t, typename job_t>
class kernel_2s<graph_t, Subgraph<NORMAL>, frontier::Frontier_2S<BDF>, updater_t, generator_t, job_t> {
 public:
  void operator()(graph_t G, Subgraph<NORMAL> SG1, Subgraph<NORMAL> SG2,
                  frontier::Frontier_2S<BDF> F, job_t job) {
    job.prepare();
    if (F.wl_sz_local) {
      detail::SubgraphToFlag<updater_t, generator_t, job_t> vis{SG1.edges, F.flag2, job};
      detail::expand_subgraph<<<detail::grid_for(F.wl_sz_local), detail::kBlock>>>(
          F.wl_local->data, F.wl_local->count, F.wl_local->capacity, SG1.lookup_buffer, SG1.vtx_ptr, vis);
    }
    SG1.clean();
    SG2.build(G, *F.wl_remote);
    if (F.wl_sz_remote) {
      detail::SubgraphToFlag<updater_t, generator_t, job_t> vis{SG2.edges, F.flag2, job};
      detail::expand_subgraph<<<detail::grid_for(F.wl_sz_remote), detail::kBlock>>>(
          F.wl_remote->data, F.wl_remote->count, F.wl_remote->capacity, SG2.lookup_buffer, SG2.vtx_ptr, vis);
    }
  }
};

}  // namespace mgg
#endif
