// graph_loader.cuh -- drop-in for the reference's include/graph_loader.cuh.
//
// graph_loader::Load(G, needWeight) reads FLAGS_input, a Galois v1 .gr file
// (header u64[4] = {1, sizeEdgeTy, n, m}, u64 end offsets, u32 destinations,
// padding, u32 edge data; include/graph_loader.cuh:65-159), through
// grus_graph_load_gr: large reads staged through pinned memory into HBM (or
// managed memory with --mem=managed), offsets converted on the device, and
// every malformed input reported (the reference prints and continues).  As in
// the reference, adjwgt is always present: the file's weights, or 1 for
// every edge of an unweighted file (:92-101).  It prints the same two lines
// (sizes, and the first vertex of maximum out-degree, :132-137).
//
// Extra flags (defined in app.cuh):
//   --mem=device|managed   where the CSR lives (default device = HBM)
//   --budget=X             managed mode device budget: X <= 1 is a fraction
//                          of the CSR bytes, X > 1 a byte count
#ifndef GRUS_MGG_GRAPH_LOADER_CUH
#define GRUS_MGG_GRAPH_LOADER_CUH

#include <cuda_runtime.h>
#include <gflags/gflags.h>

#include <cstdio>

#include "../../include/grus.h"
#include "common.cuh"
#include "graph.cuh"
#include "intrinsics.cuh"
#include "print.cuh"
#include "timer.cuh"

DECLARE_string(input);
DECLARE_string(mem);
DECLARE_double(budget);
DECLARE_int32(device);

namespace mgg {

class graph_loader {
 public:
  string graphFilePath;
  bool hasZeroID = false;
  uint64_t numNode = 0, numEdge = 0, sizeEdgeTy = 0;
  bool weighted = false;
  bool needWeight = false;
  uint64_t mem_used = 0;

  void Load(graph_t<CSR> &G, bool _needweight = true) {
    graphFilePath = FLAGS_input;
    needWeight = _needweight;
    uint64_t h[4] = {0, 0, 0, 0};
    FILE *f = std::fopen(graphFilePath.c_str(), "rb");
    if (!f || std::fread(h, sizeof(uint64_t), 4, f) != 4) {
      if (f) std::fclose(f);
      fprintf(stderr, "graph_loader: cannot read the header of '%s'\n", graphFilePath.c_str());
      exit(EXIT_FAILURE);
    }
    std::fclose(f);
    sizeEdgeTy = h[1];
    numNode = h[2];
    numEdge = h[3];
    cout << graphFilePath + " has " << numNode << " nodes and " << numEdge << "  edges\n";
    const int mode = FLAGS_mem == "managed" ? GRUS_MEM_MANAGED : GRUS_MEM_DEVICE;
    uint64_t budget = 0;
    if (mode == GRUS_MEM_MANAGED && FLAGS_budget > 0) {
      const double csr = (double)(numNode + 1) * 4.0 + (double)numEdge * 8.0;
      budget = FLAGS_budget <= 1.0 ? (uint64_t)(FLAGS_budget * csr) : (uint64_t)FLAGS_budget;
    }
    H_ERR(cudaSetDevice(FLAGS_device));
    grus_graph *g = nullptr;
    const int rc = grus_graph_load_gr(graphFilePath.c_str(), 1, mode, budget, &g);
    if (rc != GRUS_OK) {
      fprintf(stderr, "graph_loader: %s: %s (%s)\n", graphFilePath.c_str(), grus_strerror(rc),
              grus_last_error());
      exit(EXIT_FAILURE);
    }
    weighted = sizeEdgeTy != 0;
    G.adopt_handle(g, weighted);
    mem_used = G.mem_used;
    grus_graph_info info;
    grus_graph_get_info(g, &info);
    printf("%u has max out degree %u\n", info.max_degree_vertex, info.max_degree);
  }
};

}  // namespace mgg
#endif
