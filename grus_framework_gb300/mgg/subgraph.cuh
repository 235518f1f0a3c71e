// subgraph.cuh -- drop-in for the reference's include/subgraph.cuh: the
// compact "active subgraph" of the two-stage BFS (bfs_2s).
//
// Subgraph<NORMAL>::build(G, wl) copies the adjacency lists of the vertices in
// `wl` into a dense CSR (vtx, vtx_ptr, edges) plus a lookup from global id to
// local index, so the next expansion reads one compact array instead of
// scattered rows of G.  The reference gathers on the HOST, one memcpy per
// vertex over managed memory (include/subgraph.cuh:123-135), never writes
// vtx_ptr[0] (relying on zeroed pages) and re-allocates the scan scratch in
// every by-value copy.  Here the whole build is on the device:
//   lookup + degrees (one thread per vertex), CUB inclusive scan of the
//   degrees into vtx_ptr[1..], and a warp-per-vertex gather of the rows
//   (edges and weights), with the scan scratch shared by every copy.
#ifndef GRUS_MGG_SUBGRAPH_CUH
#define GRUS_MGG_SUBGRAPH_CUH

#include <cub/device/device_scan.cuh>
#include <cuda_runtime.h>
#include <gflags/gflags.h>

#include "common.cuh"
#include "graph.cuh"
#include "intrinsics.cuh"
#include "print.cuh"
#include "timer.cuh"
#include "worklist.cuh"

DECLARE_int32(device);

namespace mgg {
namespace detail {

// Warp per listed vertex: rows of G copied into the compact edge array.
static __global__ void gather_rows(const vtx_t *vtx, vtx_t count, const vtx_t *vtx_ptr,
                                   const vtx_t *xadj, const vtx_t *adjncy, const weight_t *adjwgt,
                                   vtx_t *edges, weight_t *weight) {
  const size_t warp = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  const unsigned lane = threadIdx.x & 31u;
  const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t i = warp; i < count; i += nwarps) {
    const vtx_t v = vtx[i];
    const vtx_t b = xadj[v], d = xadj[v + 1] - b, o = vtx_ptr[i];
    for (vtx_t k = lane; k < d; k += 32) {
      edges[o + k] = adjncy[b + k];
      if (adjwgt && weight) weight[o + k] = adjwgt[b + k];
    }
  }
}

}  // namespace detail

template <subgraphFmt subgraph_t>
class Subgraph {
 public:
  void reserve() {}
};

template <>
class Subgraph<NORMAL> {
 public:
  struct Scratch {
    void *tmp = nullptr;
    size_t bytes = 0;
  };
  vtx_t numNode = 0, numEdge = 0, capacity = 0, edge_capacity = 0;
  vtx_t *lookup_buffer = nullptr;
  vtx_t *vtx = nullptr;
  uint *degreeBuffer = nullptr;
  vtx_t *vtx_ptr = nullptr;
  vtx_t *edges = nullptr;
  weight_t *weight = nullptr;
  uint *degreeBuffer_h = nullptr;
  vtx_t *lookup_buffer_h = nullptr, *vtx_h = nullptr;
  void *d_temp_storage = nullptr;
  size_t temp_storage_bytes = 0, temp_storage_bytes_reserved = 0;
  Scratch *scratch = nullptr;  // shared by all copies

  Subgraph() {}
  ~Subgraph() {}
  // reserve(vertex capacity, edge capacity), as the reference calls it with
  // (G.numNode, G.numEdge) (samples/bfs_2s/bfs_2s.cu:138-139).
  void reserve(vtx_t m, vtx_t n) {
    capacity = m;
    edge_capacity = n;
    H_ERR(cudaMalloc(&vtx, (size_t)(m ? m : 1) * sizeof(vtx_t)));
    H_ERR(cudaMalloc(&degreeBuffer, (size_t)(m ? m : 1) * sizeof(uint)));
    H_ERR(cudaMalloc(&lookup_buffer, (size_t)(m ? m : 1) * sizeof(vtx_t)));
    H_ERR(cudaMalloc(&vtx_ptr, ((size_t)m + 1) * sizeof(vtx_t)));
    H_ERR(cudaMemset(vtx_ptr, 0, sizeof(vtx_t)));
    H_ERR(cudaMalloc(&edges, (size_t)(n ? n : 1) * sizeof(vtx_t)));
    H_ERR(cudaMalloc(&weight, (size_t)(n ? n : 1) * sizeof(weight_t)));
    scratch = new Scratch();
  }
  __forceinline__ __device__ vtx_t get_vtx_from_id(vtx_t id) { return lookup_buffer[id]; }
  __forceinline__ __device__ vtx_t get_vtx(vtx_t id) { return vtx[id]; }
  __forceinline__ __device__ uint get_vtx_degree(vtx_t id) { return vtx_ptr[id + 1] - vtx_ptr[id]; }
  __forceinline__ __device__ vtx_t get_edge_id(vtx_t id, vtx_t offset) { return vtx_ptr[id] + offset; }
  __forceinline__ __device__ vtx_t get_edge_dst(vtx_t id, vtx_t offset) { return edges[vtx_ptr[id] + offset]; }
  __forceinline__ __device__ vtx_t get_edge_weight(vtx_t id, vtx_t offset) {
    return weight[vtx_ptr[id] + offset];
  }

  template <typename graph_t, typename worklist_t>
  void compute_ptr(graph_t G, worklist_t wl) {
    numNode = wl.get_sz();
    if (numNode == 0) return;
    H_ERR(cudaMemcpy(vtx, wl.data, numNode * sizeof(vtx_t), cudaMemcpyDeviceToDevice));
    worklist::compute_lookup_buffer<<<numNode / BLOCK_SIZE + 1, BLOCK_SIZE>>>(
        vtx, vtx_ptr, G.xadj, lookup_buffer, degreeBuffer, numNode);
    size_t need = 0;
    H_ERR(cub::DeviceScan::InclusiveSum(nullptr, need, degreeBuffer, vtx_ptr + 1, (int)numNode));
    if (need > scratch->bytes) {
      if (scratch->tmp) H_ERR(cudaFree(scratch->tmp));
      H_ERR(cudaMalloc(&scratch->tmp, need));
      scratch->bytes = need;
    }
    H_ERR(cub::DeviceScan::InclusiveSum(scratch->tmp, need, degreeBuffer, vtx_ptr + 1, (int)numNode));
  }

  template <typename graph_t, typename worklist_t>
  void construct(graph_t G, worklist_t wl) {
    if (numNode == 0) {
      numEdge = 0;
      return;
    }
    H_ERR(cudaMemcpy(&numEdge, vtx_ptr + numNode, sizeof(vtx_t), cudaMemcpyDeviceToHost));
    int sms = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<uint64_t>((numNode + 7) / 8, (uint64_t)sms * 16);
    detail::gather_rows<<<std::max(grid, 1), 256>>>(vtx, numNode, vtx_ptr, G.xadj, G.adjncy,
                                                     G.adjwgt, edges, weight);
  }

  void move() {}  // already in device memory

  template <typename graph_t, typename worklist_t>
  void build(graph_t G, worklist_t wl) {
    compute_ptr<graph_t, worklist_t>(G, wl);
    construct<graph_t, worklist_t>(G, wl);
    move();
  }
  void clean() {}
};

}  // namespace mgg
#endif
