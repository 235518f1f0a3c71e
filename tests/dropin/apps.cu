// apps.cu -- a test program written against the mgg drop-in API exactly the
// way the reference's samples use it (graph_loader, Frontier<...>, kernel<>,
// kernel_pull<>, job/updater/generator/pull_selector functors, SaveResults).
// Each mode runs one operator and writes "<i> <value>" lines to --output.
//
//   apps --algo=bfs|sssp|cc|pr|bfs2s --input=g.gr --src=S --output=out.txt
//        [--pull] [--frontier=bdf|wl|auto|bitmap] [--mem=managed --budget=X]
//
// bfs2s is the two-stage active-subgraph BFS: Frontier_2S<BDF>, two
// Subgraph<NORMAL> swapped every level and kernel_2s, driven the way the
// reference's bfs_2s sample drives them (samples/bfs_2s/bfs_2s.cu:94-138).
#include <gflags/gflags.h>

#include "app.cuh"
#include "common.cuh"
#include "frontier.cuh"
#include "frontier_2s.cuh"
#include "graph.cuh"
#include "graph_loader.cuh"
#include "kernel.cuh"
#include "kernel_2s.cuh"
#include "subgraph.cuh"
#include "worklist.cuh"

using namespace mgg;

DEFINE_string(algo, "bfs", "bfs | sssp | cc | pr | bfs2s");
DEFINE_string(frontier, "bdf", "push frontier: bdf | wl | auto | bitmap");

namespace t {

__global__ void fill(uint *a, vtx_t n, uint v, vtx_t src, uint vsrc) {
  for (vtx_t i = TID_1D; i < n; i += TOTAL_THREADS_1D) a[i] = (i == src) ? vsrc : v;
}
__global__ void iota(uint *a, vtx_t n) {
  for (vtx_t i = TID_1D; i < n; i += TOTAL_THREADS_1D) a[i] = i;
}

// Depth/label job shared by BFS, SSSP and CC.
struct job_t {
  uint *label = nullptr;
  uint itr = 0;
  vtx_t numNode = 0;
  weight_t *adjwgt = nullptr;
  void prepare() {}
};

// next frontier marks, one overload per frontier representation
struct mark {
  __device__ void operator()(bool hit, worklist::Worklist wl, vtx_t dst) {
    if (hit) wl.append(dst);
  }
  __device__ void operator()(bool hit, char *flag, vtx_t dst) {
    if (hit) flag[dst] = 1;
  }
  __device__ void operator()(bool hit, char *flag, vtx_t dst, char *finished) {
    if (hit) {
      flag[dst] = 1;
      *finished = 0;
    }
  }
};

// BFS: first writer of a level wins (all store itr+1).
struct bfs_update {
  __device__ bool operator()(vtx_t, vtx_t dst, vtx_t, job_t job) {
    if (job.label[dst] > job.itr + 1) {
      job.label[dst] = job.itr + 1;
      return true;
    }
    return false;
  }
};
struct bfs_unvisited {
  __device__ bool operator()(vtx_t id, job_t job) { return job.label[id] == INFINIT; }
};

// SSSP: atomic relax (min survives races); frontier marks may repeat a vertex.
struct sssp_update {
  __device__ bool operator()(vtx_t src, vtx_t dst, vtx_t e, job_t job) {
    const uint ds = job.label[src];
    if (ds == INFINIT) return false;
    const uint nd = ds + job.adjwgt[e];
    return nd < atomicMin(&job.label[dst], nd);
  }
};
struct any_vertex {
  __device__ bool operator()(vtx_t, job_t) { return true; }
};

// CC: minimum label along edges.
struct cc_update {
  __device__ bool operator()(vtx_t src, vtx_t dst, vtx_t, job_t job) {
    const uint l = job.label[src];
    return l < atomicMin(&job.label[dst], l);
  }
};

// Delta-push PageRank (the algorithm of the reference's pagerank sample).
__global__ void pr_init(float *rank, float *delta, const vtx_t *xadj, const vtx_t *adjncy, vtx_t n) {
  const size_t tid = blockDim.x * (size_t)blockIdx.x + threadIdx.x;
  const vtx_t lane = threadIdx.x % 32, w = (vtx_t)(tid / 32);
  if (w < n) {
    if (lane == 0) rank[w] = 1.0f - ALPHA;
    const vtx_t d = xadj[w + 1] - xadj[w];
    const float up = ((1.0 - ALPHA) * ALPHA) / d;
    for (vtx_t i = xadj[w] + lane; i < xadj[w + 1]; i += 32) atomicAdd(&delta[adjncy[i]], up);
  }
}
__global__ void pr_fold(float *rank, float *delta, float *delta2, vtx_t n) {
  for (vtx_t i = TID_1D; i < n; i += TOTAL_THREADS_1D) {
    const float r = delta[i];
    delta[i] = 0.f;
    delta2[i] = r;
    rank[i] += r;
  }
}
struct pr_job {
  float *rank, *delta, *delta2;
  uint itr = 0;
  vtx_t numNode;
  vtx_t *xadj;
  weight_t *adjwgt = nullptr;
  void prepare() { pr_fold<<<numNode / 1024 + 1, 1024>>>(rank, delta, delta2, numNode); }
};
struct pr_update {
  __device__ bool operator()(vtx_t src, vtx_t dst, vtx_t, pr_job job) {
    const float up = job.delta2[src] * ALPHA / (job.xadj[src + 1] - job.xadj[src]);
    const float before = atomicAdd(&job.delta[dst], up);
    return (before + up > EPSILON) && (before < EPSILON);
  }
};

template <typename U, typename J, typename F>
uint run_push(graph_t<CSR> &G, J &job, F &frontier) {
  kernel<graph_t<CSR>, F, U, mark, J> K;
  while (!frontier.finish()) {
    K(G, frontier, job);
    H_ERR(cudaDeviceSynchronize());
    frontier.Next();
    job.itr++;
  }
  return job.itr;
}

template <typename U, typename J>
uint push_any(graph_t<CSR> &G, J &job, bool full) {
  const vtx_t n = G.numNode;
  if (FLAGS_frontier == "wl") {
    frontier::Frontier<WL> F;
    F.Init(n, FLAGS_src, FLAGS_device, 1.0, full);
    return run_push<U>(G, job, F);
  } else if (FLAGS_frontier == "auto") {
    frontier::Frontier<BDF_AUTO> F;
    F.Init(n, FLAGS_src, FLAGS_device, 1.0, full);
    return run_push<U>(G, job, F);
  } else if (FLAGS_frontier == "bitmap") {
    frontier::Frontier<BITMAP> F;
    F.Init(n, FLAGS_src, FLAGS_device, 1.0, full);
    return run_push<U>(G, job, F);
  }
  frontier::Frontier<BDF> F;
  F.Init(n, FLAGS_src, FLAGS_device, 1.0, full);
  return run_push<U>(G, job, F);
}

template <typename U, typename S>
uint run_pull(graph_t<CSR> &Gcsr, job_t &job, bool full) {
  graph_t<CSC> G;
  G.CSR2CSC(Gcsr);
  if (job.adjwgt) job.adjwgt = G.adjwgt;  // CSC edge ids index the CSC weights
  frontier::Frontier<BITMAP> F;
  F.Init(G.numNode, FLAGS_src, FLAGS_device, 1.0, full);
  kernel_pull<U, mark, S, job_t> K;
  while (!F.finish()) {
    K(G, F, job);
    H_ERR(cudaDeviceSynchronize());
    F.Next();
    job.itr++;
  }
  return job.itr;
}

// Two-stage BFS: each level expands the frontier's "local" vertices over the
// subgraph built one level earlier and gathers the rows of its "remote"
// vertices into a fresh subgraph before expanding them; the two subgraphs
// trade places every level.
uint run_bfs_2s(graph_t<CSR> &G, job_t &job) {
  frontier::Frontier_2S<BDF> F;
  F.Init(G.numNode, FLAGS_src, FLAGS_device, 1.0, false);
  Subgraph<NORMAL> SG1, SG2;
  SG1.reserve(G.numNode, G.numEdge);
  SG2.reserve(G.numNode, G.numEdge);
  Subgraph<NORMAL> *SG_local = &SG1, *SG_remote = &SG2;
  kernel_2s<graph_t<CSR>, Subgraph<NORMAL>, frontier::Frontier_2S<BDF>, bfs_update, mark, job_t> K;
  while (!F.finish()) {
    K(G, *SG_local, *SG_remote, F, job);
    H_ERR(cudaDeviceSynchronize());
    std::swap(SG_local, SG_remote);
    F.Next();
    job.itr++;
  }
  return job.itr;
}

bool Single() {
  H_ERR(cudaSetDevice(FLAGS_device));
  graph_t<CSR> G(FLAGS_algo == "sssp");
  graph_loader loader;
  loader.Load(G, FLAGS_algo == "sssp");
  G.Set_Mem_Policy(nullptr);
  const vtx_t n = G.numNode;
  Timer t;
  uint itr = 0;
  if (FLAGS_algo == "pr") {
    pr_job job;
    job.numNode = n;
    job.xadj = G.xadj;
    H_ERR(cudaMallocManaged(&job.rank, n * sizeof(float)));
    H_ERR(cudaMallocManaged(&job.delta, n * sizeof(float)));
    H_ERR(cudaMallocManaged(&job.delta2, n * sizeof(float)));
    H_ERR(cudaMemset(job.delta, 0, n * sizeof(float)));
    pr_init<<<n * 32 / BLOCK_SIZE + 1, BLOCK_SIZE>>>(job.rank, job.delta, G.xadj, G.adjncy, n);
    itr = push_any<pr_update>(G, job, true);
    H_ERR(cudaDeviceSynchronize());
    cout << "itr " << itr << " in " << t.Finish() << endl;
    print::SaveResults(FLAGS_output, job.rank, n);
    return true;
  }
  job_t job;
  job.numNode = n;
  H_ERR(cudaMallocManaged(&job.label, n * sizeof(uint)));
  if (FLAGS_algo == "cc") iota<<<n / BLOCK_SIZE + 1, BLOCK_SIZE>>>(job.label, n);
  else fill<<<n / BLOCK_SIZE + 1, BLOCK_SIZE>>>(job.label, n, INFINIT, FLAGS_src, 0);
  if (FLAGS_algo == "sssp") job.adjwgt = G.adjwgt;
  const bool full = FLAGS_algo == "cc";
  if (FLAGS_algo == "bfs2s") {
    itr = run_bfs_2s(G, job);
  } else if (FLAGS_pull) {
    if (FLAGS_algo == "bfs") itr = run_pull<bfs_update, bfs_unvisited>(G, job, full);
    else if (FLAGS_algo == "sssp") itr = run_pull<sssp_update, any_vertex>(G, job, full);
    else itr = run_pull<cc_update, any_vertex>(G, job, full);
  } else {
    if (FLAGS_algo == "bfs") itr = push_any<bfs_update>(G, job, full);
    else if (FLAGS_algo == "sssp") itr = push_any<sssp_update>(G, job, full);
    else itr = push_any<cc_update>(G, job, full);
  }
  H_ERR(cudaDeviceSynchronize());
  cout << "itr " << itr << " in " << t.Finish() << endl;
  print::SaveResults(FLAGS_output, job.label, n);
  return true;
}

struct App {
  static bool Single() { return t::Single(); }
  static bool Multi() { return t::Single(); }
};

}  // namespace t

int main(int argc, char **argv) {
  Skeleton<t::App> app;
  return app(argc, argv);
}
