// ref_pin.cu -- runs the reference's own host code on the CPU to pin the
// oracle (test infrastructure only; built by oracle/build.py into
// oracle/_ref/ref_pin when the Grus sources are present).
//
//   ref_pin gr  <file.gr> <need_weight 0|1>   graph_loader::Load (include/graph_loader.cuh:160-166)
//   ref_pin csc <file.gr>                     graph_t<CSC>::CSR2CSC -> csr_tocsc (include/graph.cuh:273-320)
//
// Output: "n m", then the offsets, columns and (gr mode) weights, one array
// per line, as decimal text.
#include <cstdio>
#include <cstring>
#include <unistd.h>
#include <gflags/gflags.h>

#include "graph_loader.cuh"

DEFINE_string(input, "", "graph file");
DEFINE_bool(pf, false, "");
DEFINE_bool(ab, false, "");
DEFINE_bool(rm, false, "");
DEFINE_bool(pl, false, "");
DEFINE_bool(opt, true, "");
DEFINE_int32(device, 0, "");

static void dump(const unsigned *a, unsigned long long k) {
  for (unsigned long long i = 0; i < k; ++i) std::printf(i ? " %u" : "%u", a[i]);
  std::printf("\n");
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  FLAGS_input = argv[2];
  // the reference prints progress on stdout; send it to stderr while it runs
  std::fflush(stdout);
  const int saved = dup(1);
  dup2(2, 1);
  mgg::graph_t<mgg::CSR> G(argc > 3 && argv[3][0] == '1');
  mgg::graph_loader loader;
  loader.Load(G, argc > 3 && argv[3][0] == '1');
  if (std::strcmp(argv[1], "csc") == 0) {
    mgg::graph_t<mgg::CSC> T;
    T.CSR2CSC(G);
    std::cout.flush();
    std::fflush(stdout);
    dup2(saved, 1);
    std::printf("%llu %llu\n", (unsigned long long)T.numNode, (unsigned long long)T.numEdge);
    dump(T.xadj, T.numNode + 1);
    dump(T.adjncy, T.numEdge);
    return 0;
  }
  std::cout.flush();
  std::fflush(stdout);
  dup2(saved, 1);
  if (std::strcmp(argv[1], "gr") == 0) {
    std::printf("%llu %llu\n", (unsigned long long)G.numNode, (unsigned long long)G.numEdge);
    dump(G.xadj, G.numNode + 1);
    dump(G.adjncy, G.numEdge);
    dump(G.adjwgt, G.numEdge);
    return 0;
  }
  return 2;
}
