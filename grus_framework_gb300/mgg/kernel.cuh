// kernel.cuh -- drop-in for the reference's include/kernel.cuh.
//
// kernel<graph_t, frontier_t, updater_t, generator_t, job_t> and
// kernel_pull<updater_t, generator_t, pull_selector_t, job_t> keep the
// reference's functor interface (include/kernel.cuh:124-203): each launch
// calls, for every edge of every active vertex,
//     generator(updater(src, dst, edge_id, job), <next frontier>, dst[, finished])
// with job passed by value and edge_id indexing the CSR (push) or CSC
// (pull).  The reference maps one warp to every active vertex
// (kernel.cuh:18-123); here the user's functors run inside the degree-binned
// expansion of csrc/expand.cuh:
//   * a tile of 256 sources is expanded with CTA (degree >= 256), warp
//     (>= 32) and scan-based gather (< 32) mappings, coalesced column loads;
//   * sources of degree >= 8192 are cut into 1024-edge pieces (grus::kChunk)
//     and expanded by a second launch, one piece per CTA, so hubs spread over
//     every SM.
// kernel<..., Frontier<BDF>> calls job.prepare() before each launch, as the
// reference does; kernel_pull does not (the reference's kernel_pull never
// calls it, kernel.cuh:128-133, and the pull samples are written for that).
// BDF_AUTO dispatches exactly one kernel per level (the reference's switch
// falls through and launches all three, kernel.cuh:186-201).
#ifndef GRUS_MGG_KERNEL_CUH
#define GRUS_MGG_KERNEL_CUH

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "../csrc/expand.cuh"
#include "common.cuh"
#include "frontier.cuh"
#include "graph.cuh"
#include "worklist.cuh"

namespace mgg {
namespace detail {

constexpr int kBlock = 256;
constexpr uint32_t kHuge = 8192;

inline int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
  }
  return sms;
}

inline int grid_for(uint64_t sources) {
  const uint64_t tiles = (sources + kBlock - 1) / kBlock;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(tiles, (uint64_t)sm_count() * 8));
}

// Sources of degree >= kHuge go to the piece list instead of the tile.
__device__ __forceinline__ void divert_huge(vtx_t v, vtx_t &beg, vtx_t end, uint4 *chunks,
                                            vtx_t *ccount, uint32_t ccap) {
  if (end - beg < kHuge) return;
  const uint32_t np = (end - beg + grus::kChunk - 1) / grus::kChunk;
  const uint32_t at = atomicAdd(ccount, np);
  if (at + np <= ccap)
    for (uint32_t k = 0; k < np; ++k)
      chunks[at + k] = make_uint4(v, beg + k * grus::kChunk, min(end, beg + (k + 1) * grus::kChunk), 0u);
  beg = end;
}

// ---- visitors: one per generator overload --------------------------------
template <typename U, typename Gen, typename J>
struct ToFlag {  // generator(bool, char *flag, dst)
  const vtx_t *adjncy;
  char *flag;
  J job;
  using aux_t = uint32_t;
  __device__ __forceinline__ uint32_t aux(uint32_t) const { return 0u; }
  __device__ __forceinline__ void edge(uint32_t src, uint32_t, uint32_t x) {
    U updater;
    Gen generator;
    const vtx_t dst = adjncy[x];
    generator(updater(src, dst, x, job), flag, dst);
  }
};

template <typename U, typename Gen, typename J>
struct ToFlagFinished {  // generator(bool, char *flag, dst, char *finished)
  const vtx_t *adjncy;
  char *flag, *finished;
  J job;
  using aux_t = uint32_t;
  __device__ __forceinline__ uint32_t aux(uint32_t) const { return 0u; }
  __device__ __forceinline__ void edge(uint32_t src, uint32_t, uint32_t x) {
    U updater;
    Gen generator;
    const vtx_t dst = adjncy[x];
    generator(updater(src, dst, x, job), flag, dst, finished);
  }
};

template <typename U, typename Gen, typename J>
struct ToWorklist {  // generator(bool, Worklist, dst)
  const vtx_t *adjncy;
  worklist::Worklist wl;
  J job;
  using aux_t = uint32_t;
  __device__ __forceinline__ uint32_t aux(uint32_t) const { return 0u; }
  __device__ __forceinline__ void edge(uint32_t src, uint32_t, uint32_t x) {
    U updater;
    Gen generator;
    const vtx_t dst = adjncy[x];
    generator(updater(src, dst, x, job), wl, dst);
  }
};

template <typename U, typename Gen, typename J>
struct PullFromFlag {  // the owner is dst; in-edge x brings src
  const vtx_t *adjncy;
  const char *flag1;
  char *flag2, *finished;
  J job;
  using aux_t = uint32_t;
  __device__ __forceinline__ uint32_t aux(uint32_t) const { return 0u; }
  __device__ __forceinline__ void edge(uint32_t dst, uint32_t, uint32_t x) {
    const vtx_t src = adjncy[x];
    if (flag1[src]) {
      U updater;
      Gen generator;
      generator(updater(src, dst, x, job), flag2, dst, finished);
    }
  }
};

// ---- kernels --------------------------------------------------------------
template <class Vis>
__global__ void __launch_bounds__(kBlock)
    expand_queue(const vtx_t *__restrict__ xadj, const vtx_t *queue, const vtx_t *qcount_d,
                 vtx_t qcap, uint4 *chunks, vtx_t *ccount, uint32_t ccap, Vis vis) {
  const vtx_t qcount = min(*qcount_d, qcap);
  for (uint32_t base = blockIdx.x * kBlock; base < qcount; base += gridDim.x * kBlock) {
    const uint32_t i = base + threadIdx.x;
    vtx_t v = 0, beg = 0, end = 0;
    if (i < qcount) {
      v = queue[i];
      beg = xadj[v];
      end = xadj[v + 1];
      divert_huge(v, beg, end, chunks, ccount, ccap);
    }
    grus::expand_tile<kBlock>(v, beg, end, 0u, vis);
  }
}

// Sources are the vertex ids v < n with active(v).
template <class Active, class Vis>
__global__ void __launch_bounds__(kBlock)
    expand_range(const vtx_t *__restrict__ xadj, vtx_t n, Active active, uint4 *chunks,
                 vtx_t *ccount, uint32_t ccap, Vis vis) {
  for (uint32_t base = blockIdx.x * kBlock; base < n; base += gridDim.x * kBlock) {
    const vtx_t v = base + threadIdx.x;
    vtx_t beg = 0, end = 0;
    if (v < n && active(v)) {
      beg = xadj[v];
      end = xadj[v + 1];
      divert_huge(v, beg, end, chunks, ccount, ccap);
    }
    grus::expand_tile<kBlock>(v, beg, end, 0u, vis);
  }
}

template <class Vis>
__global__ void __launch_bounds__(kBlock)
    expand_pieces(const uint4 *chunks, const vtx_t *ccount, uint32_t ccap, Vis vis) {
  grus::expand_chunks<kBlock>(chunks, min(*ccount, ccap), vis);
}

struct ByteActive {
  const char *flag;
  __device__ __forceinline__ bool operator()(vtx_t v) const { return flag[v] != 0; }
};

template <typename Sel, typename J>
struct SelectorActive {
  J job;
  __device__ __forceinline__ bool operator()(vtx_t v) const {
    Sel sel;
    return sel(v, job);
  }
};

template <class Vis>
void run_queue(const vtx_t *xadj, uint64_t m, frontier::FrontierAux *aux,
               const worklist::Worklist &wl, vtx_t qcount_h, const Vis &vis) {
  if (qcount_h == 0) return;
  aux->ensure(m, kHuge, grus::kChunk);
  H_ERR(cudaMemsetAsync(aux->ccount, 0, sizeof(vtx_t), NULL));
  expand_queue<Vis><<<grid_for(qcount_h), kBlock>>>(xadj, wl.data, wl.count, wl.capacity,
                                                    aux->chunks, aux->ccount, aux->chunk_cap, vis);
  expand_pieces<Vis><<<sm_count() * 2, kBlock>>>(aux->chunks, aux->ccount, aux->chunk_cap, vis);
}

template <class Active, class Vis>
void run_range(const vtx_t *xadj, uint64_t m, frontier::FrontierAux *aux, vtx_t n,
               const Active &active, const Vis &vis) {
  if (n == 0) return;
  aux->ensure(m, kHuge, grus::kChunk);
  H_ERR(cudaMemsetAsync(aux->ccount, 0, sizeof(vtx_t), NULL));
  expand_range<Active, Vis><<<grid_for(n), kBlock>>>(xadj, n, active, aux->chunks, aux->ccount,
                                                     aux->chunk_cap, vis);
  expand_pieces<Vis><<<sm_count() * 2, kBlock>>>(aux->chunks, aux->ccount, aux->chunk_cap, vis);
}

}  // namespace detail

// Pull over the CSC: every vertex passing pull_selector scans its in-edges and
// applies the user's functors to those whose source is in flag1.
template <typename updater_t, typename generator_t, typename pull_selector_t, typename job_t>
class kernel_pull {
 public:
  void operator()(graph_t<CSC> G, frontier::Frontier<BITMAP> F, job_t job) {
    detail::PullFromFlag<updater_t, generator_t, job_t> vis{G.adjncy, F.flag1, F.flag2,
                                                            F.finished_d, job};
    detail::SelectorActive<pull_selector_t, job_t> act{job};
    detail::run_range(G.xadj, G.numEdge, F.aux, (vtx_t)F.numNode, act, vis);
  }
};

template <typename graph_t, typename frontier_t, typename updater_t, typename generator_t,
          typename job_t>
class kernel {
 public:
  void operator()(graph_t G, frontier_t F, job_t job) {}
};

template <typename graph_t, typename updater_t, typename generator_t, typename job_t>
class kernel<graph_t, frontier::Frontier<WL>, updater_t, generator_t, job_t> {
 public:
  void operator()(graph_t G, frontier::Frontier<WL> F, job_t job) {
    job.prepare();
    // a generator may append a vertex once per in-edge: room for every edge
    F.wl_n->grow(std::max<uint64_t>(G.numNode, G.numEdge));
    detail::ToWorklist<updater_t, generator_t, job_t> vis{G.adjncy, *F.wl_n, job};
    detail::run_queue(G.xadj, G.numEdge, F.aux, *F.wl_c, F.get_work_size_h(), vis);
  }
};

template <typename graph_t, typename updater_t, typename generator_t, typename job_t>
class kernel<graph_t, frontier::Frontier<BDF>, updater_t, generator_t, job_t> {
 public:
  void operator()(graph_t G, frontier::Frontier<BDF> F, job_t job) {
    job.prepare();
    detail::ToFlag<updater_t, generator_t, job_t> vis{G.adjncy, F.flag2, job};
    detail::run_queue(G.xadj, G.numEdge, F.aux, F.wl1, F.get_work_size_h(), vis);
  }
};

template <typename graph_t, typename updater_t, typename generator_t, typename job_t>
class kernel<graph_t, frontier::Frontier<BITMAP>, updater_t, generator_t, job_t> {
 public:
  void operator()(graph_t G, frontier::Frontier<BITMAP> F, job_t job) {
    job.prepare();
    detail::ToFlagFinished<updater_t, generator_t, job_t> vis{G.adjncy, F.flag2, F.finished_d, job};
    detail::run_range(G.xadj, G.numEdge, F.aux, (vtx_t)F.numNode, detail::ByteActive{F.flag1}, vis);
  }
};

template <typename graph_t, typename updater_t, typename generator_t, typename job_t>
class kernel<graph_t, frontier::Frontier<BDF_AUTO>, updater_t, generator_t, job_t> {
 public:
  void operator()(graph_t G, frontier::Frontier<BDF_AUTO> F, job_t job) {
    job.prepare();
    switch (F.current_f) {
      case WL: {
        F.wl_n->grow(std::max<uint64_t>(G.numNode, G.numEdge));
        detail::ToWorklist<updater_t, generator_t, job_t> vis{G.adjncy, *F.wl_n, job};
        detail::run_queue(G.xadj, G.numEdge, F.aux, *F.wl_c, F.wl_sz, vis);
        break;
      }
      case BITMAP: {
        detail::ToFlag<updater_t, generator_t, job_t> vis{G.adjncy, F.flag2, job};
        detail::run_range(G.xadj, G.numEdge, F.aux, (vtx_t)F.numNode, detail::ByteActive{F.flag1}, vis);
        break;
      }
      default: {
        detail::ToFlag<updater_t, generator_t, job_t> vis{G.adjncy, F.flag2, job};
        detail::run_queue(G.xadj, G.numEdge, F.aux, *F.wl_c, F.wl_sz, vis);
        break;
      }
    }
  }
};

}  // namespace mgg

#endif
