// graph.cuh -- drop-in for the reference's include/graph.cuh.
//
// graph_t<CSR> / graph_t<CSC> keep the reference's public fields (numNode,
// numEdge, xadj, adjncy, adjwgt, mem_used, needWeight, weighted ...) and stay
// trivially copyable handles of device pointers, because the samples pass
// them by value to kernels and hand G.xadj / G.adjncy to their own kernels
// (samples/pagerank/pr.cu:153-154).  Storage is owned by a libgrus graph
// handle (include/grus.h): CSR in HBM by default, or managed memory under a
// device budget (--mem=managed --budget=...).  Differences from the reference:
//   * CSR2CSC is a device transpose that carries the weights
//     (include/graph.cuh:294 drops them, so the reference's SSSP pull reads a
//     null weight array);
//   * chunks are a host array, not a std::vector member, so the handle stays
//     trivially copyable; make_chunks copies elements, not bytes (the
//     reference copies numNode+1 / edge_in_chunk BYTES, graph.cuh:146-151),
//     and distribute_chunks places chunk i on device i % deviceCount.
#ifndef GRUS_MGG_GRAPH_CUH
#define GRUS_MGG_GRAPH_CUH

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <gflags/gflags.h>

#include <algorithm>

#include "../../include/grus.h"
#include "common.cuh"
#include "intrinsics.cuh"
#include "print.cuh"
#include "timer.cuh"

DECLARE_string(input);
DECLARE_bool(pf);
DECLARE_bool(ab);
DECLARE_bool(rm);
DECLARE_bool(pl);
DECLARE_bool(opt);
DECLARE_int32(device);

namespace mgg {

template <typename T>
void PrintResults(T *results, uint n);

// A 1-D vertex range of a graph (the reference's multi-GPU stub,
// include/graph.cuh:34-112): its own copy of the range's edges, global
// arrays for the rest.
template <graphFmt fmt>
class graph_chunk {
 public:
  uint64_t numNode = 0, numEdge = 0;
  vtx_t *xadj = nullptr, *vwgt = nullptr, *adjncy = nullptr, *adjncy_global = nullptr;
  weight_t *adjwgt = nullptr, *adjwgt_global = nullptr;
  uint64_t node_in_chunk = 0, edge_in_chunk = 0;
  vtx_t start_v = 0, end_v = 0, start_e = 0, end_e = 0;
  uint device_id = 0;
  bool weighted = false;

  __forceinline__ __device__ vtx_t access_edge(vtx_t src, vtx_t offset) {
    if (start_v <= src && src < end_v) return adjncy[xadj[src] + offset - start_e];
    return adjncy_global[xadj[src] + offset];
  }
  __forceinline__ __device__ vtx_t access_weight(vtx_t src, vtx_t offset) {
    if (start_v <= src && src < end_v) return adjwgt[xadj[src] + offset - start_e];
    return adjwgt_global[xadj[src] + offset];
  }
  __forceinline__ __device__ vtx_t get_degree(vtx_t id) { return xadj[id + 1] - xadj[id]; }

  void distribute(int deviceId, cudaStream_t *stream) {
    cudaMemLocation loc{};
    loc.type = cudaMemLocationTypeDevice;
    loc.id = deviceId;
    cudaStream_t s = stream ? *stream : (cudaStream_t)0;
    H_ERR(cudaMemPrefetchAsync(xadj, (numNode + 1) * sizeof(vtx_t), loc, 0, s));
    if (edge_in_chunk) H_ERR(cudaMemPrefetchAsync(adjncy, edge_in_chunk * sizeof(vtx_t), loc, 0, s));
    if (weighted && edge_in_chunk)
      H_ERR(cudaMemPrefetchAsync(adjwgt, edge_in_chunk * sizeof(weight_t), loc, 0, s));
  }
};

template <graphFmt fmt>
std::ostream &operator<<(std::ostream &output, graph_chunk<fmt> &chunk) {
  output << "numNode: \t" << chunk.node_in_chunk << " numEdge: \t" << chunk.edge_in_chunk << endl;
  return output;
}

template <graphFmt fmt>
class graph_base {
 public:
  bool hasZeroID = false;
  uint64_t numNode = 0;
  uint64_t numEdge = 0;
  vtx_t *xadj = nullptr, *vwgt = nullptr, *adjncy = nullptr;
  weight_t *adjwgt = nullptr, *adjwgt_d = nullptr;
  uint *inDegree = nullptr;
  uint *outDegree = nullptr;
  bool weighted = false;
  bool needWeight = false;
  uint64_t mem_used = 0;
  graph_chunk<fmt> *chunks = nullptr;  // host array of numChunk entries
  int numChunk = 0;
  grus_graph *handle = nullptr;        // owns the arrays (never freed, as in the reference)
  int mem_mode = GRUS_MEM_DEVICE;

  void distribute_chunks(cudaStream_t *stream) {
    int ndev = 1;
    cudaGetDeviceCount(&ndev);
    for (int i = 0; i < numChunk; i++) chunks[i].distribute(i % std::max(ndev, 1), stream);
  }

  void make_chunks(int num_gpu) {
    if (num_gpu < 1) num_gpu = 1;
    numChunk = num_gpu;
    chunks = new graph_chunk<fmt>[num_gpu];
    std::vector<vtx_t> h_xadj(numNode + 1);
    H_ERR(cudaMemcpy(h_xadj.data(), xadj, (numNode + 1) * sizeof(vtx_t), cudaMemcpyDefault));
    const uint64_t per = numNode / num_gpu;
    for (int i = 0; i < num_gpu; i++) {
      graph_chunk<fmt> &c = chunks[i];
      const uint64_t v0 = i * per, v1 = (i == num_gpu - 1) ? numNode : v0 + per;
      c.numNode = numNode;
      c.numEdge = numEdge;
      c.start_v = (vtx_t)v0;
      c.end_v = (vtx_t)v1;
      c.node_in_chunk = v1 - v0;
      c.start_e = h_xadj[v0];
      c.end_e = h_xadj[v1];
      c.edge_in_chunk = c.end_e - c.start_e;
      c.device_id = i;
      c.adjncy_global = adjncy;
      c.adjwgt_global = adjwgt;
      c.weighted = adjwgt != nullptr;
      H_ERR(cudaMallocManaged(&c.xadj, (numNode + 1) * sizeof(vtx_t)));
      H_ERR(cudaMemcpy(c.xadj, xadj, (numNode + 1) * sizeof(vtx_t), cudaMemcpyDefault));
      H_ERR(cudaMallocManaged(&c.adjncy, std::max<uint64_t>(c.edge_in_chunk, 1) * sizeof(vtx_t)));
      if (c.edge_in_chunk)
        H_ERR(cudaMemcpy(c.adjncy, adjncy + c.start_e, c.edge_in_chunk * sizeof(vtx_t), cudaMemcpyDefault));
      if (c.weighted) {
        H_ERR(cudaMallocManaged(&c.adjwgt, std::max<uint64_t>(c.edge_in_chunk, 1) * sizeof(weight_t)));
        if (c.edge_in_chunk)
          H_ERR(cudaMemcpy(c.adjwgt, adjwgt + c.start_e, c.edge_in_chunk * sizeof(weight_t), cudaMemcpyDefault));
      }
    }
  }

  // HBM mode: the arrays already live in device memory, nothing to do.
  // Managed mode: libgrus applied the reference's --opt policy (prefetch up
  // to the device budget, AccessedBy for the rest; include/graph.cuh:173-205)
  // when the graph was loaded; with --opt=false the individual --pf/--ab/
  // --rm/--pl hints of include/graph.cuh:206-249 are applied here.
  void Set_Mem_Policy(cudaStream_t *stream = NULL) {
    if (mem_mode != GRUS_MEM_MANAGED || FLAGS_opt) return;
    cudaMemLocation loc{};
    loc.type = cudaMemLocationTypeDevice;
    loc.id = FLAGS_device;
    cudaStream_t s = stream ? *stream : (cudaStream_t)0;
    const size_t xb = (numNode + 1) * sizeof(vtx_t), cb = numEdge * sizeof(vtx_t);
    const size_t wb = adjwgt ? numEdge * sizeof(weight_t) : 0;
    auto hint = [&](cudaMemoryAdvise a) {
      H_ERR(cudaMemAdvise(xadj, xb, a, loc));
      if (cb) H_ERR(cudaMemAdvise(adjncy, cb, a, loc));
      if (needWeight && wb) H_ERR(cudaMemAdvise(adjwgt, wb, a, loc));
    };
    if (FLAGS_pf) {
      H_ERR(cudaMemPrefetchAsync(xadj, xb, loc, 0, s));
      if (cb) H_ERR(cudaMemPrefetchAsync(adjncy, cb, loc, 0, s));
      if (needWeight && wb) H_ERR(cudaMemPrefetchAsync(adjwgt, wb, loc, 0, s));
    }
    if (FLAGS_ab) hint(cudaMemAdviseSetAccessedBy);
    if (FLAGS_rm) hint(cudaMemAdviseSetReadMostly);
    if (FLAGS_pl) hint(cudaMemAdviseSetPreferredLocation);
  }

 protected:
  void adopt(grus_graph *h, bool csc) {
    grus_graph_info info;
    if (grus_graph_get_info(h, &info) != GRUS_OK) {
      fprintf(stderr, "graph: %s\n", grus_last_error());
      exit(EXIT_FAILURE);
    }
    handle = h;
    numNode = info.n;
    numEdge = info.m;
    mem_mode = info.mem_mode;
    xadj = (vtx_t *)(csc ? info.t_offsets : info.offsets);
    adjncy = (vtx_t *)(csc ? info.t_cols : info.cols);
    adjwgt = (weight_t *)(csc ? info.t_weights : info.weights);
    mem_used = (numNode + 1) * sizeof(vtx_t) + numEdge * sizeof(vtx_t);
  }
};

template <graphFmt fmt>
class graph_t : public graph_base<fmt> {};

template <>
class graph_t<CSR> : public graph_base<CSR> {
 public:
  graph_t(bool _needweight = false) {
    this->hasZeroID = false;
    this->needWeight = _needweight;
  }
  // called by graph_loader::Load
  void adopt_handle(grus_graph *h, bool file_weighted) {
    adopt(h, false);
    weighted = file_weighted;
  }
};

template <>
class graph_t<CSC> : public graph_base<CSC> {
 public:
  graph_t() {}
  // Device transpose of G (include/graph.cuh:308-320), weights included.
  void CSR2CSC(graph_t<CSR> G) {
    LOG("transferring CSR to CSC\n");
    const int rc = grus_graph_build_csc(G.handle);
    if (rc != GRUS_OK) {
      fprintf(stderr, "CSR2CSC: %s: %s\n", grus_strerror(rc), grus_last_error());
      exit(EXIT_FAILURE);
    }
    adopt(G.handle, true);
    weighted = G.weighted;
    needWeight = G.needWeight;
  }
};

}  // namespace mgg
#endif
