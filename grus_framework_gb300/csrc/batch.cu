// batch.cu -- many BFS / SSSP queries over many resident graphs in ONE launch.
//
// A worker is one thread-block cluster (kCluster CTAs on one GPC).  Workers
// pull tasks -- (graph, algorithm, source, output slice) -- from a device
// counter and run each query to completion inside the cluster, separating
// levels with the hardware cluster barrier (barrier.cluster), so there is no
// software grid barrier and no wait that can outlive the kernel.  Each
// worker owns device state sized for the largest graph of the batch
// (frontier bitmaps, binned queues, chunk lists, far piles, level counters).
// Algorithms:
//   BFS  : push levels with the degree-binned expansion of expand.cuh (CTA /
//          warp / gather mappings, hub chunks), visited bitmap claims.
//   SSSP : the near/far label-correcting scheme of sssp.cu (atomicMin,
//          Delta buckets), scoped to the cluster.
// Results are bit-exact against single-query runs (BFS depths and SSSP
// distances are schedule-independent).  The same kernel, launched with one
// worker on a stream, is the unit of work of the query server (serve.cu).
// The reference has no batching (one traversal per process run,
// samples/bfs/bfs.cu:135-173, samples/sssp/sssp.cu:123-170).
#include <cooperative_groups.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "batch.cuh"
#include "expand.cuh"
#include "grus_internal.cuh"

namespace cg = cooperative_groups;

namespace grus {
namespace batch {

struct Slot {
  uint32_t qcount, ccount;
  unsigned long long visits;
  uint32_t pad[4];
};

struct FarCtl {
  uint32_t count[2];
  uint32_t minfar[2];
};

// Per-worker control block (global memory), 256 bytes.
struct WorkerCtl {
  Slot slots[4];        // 128 B
  FarCtl far;           // 16 B
  uint32_t err;         // device error bits of this worker
  uint32_t levels;      // levels of the last task
  unsigned long long visits;
  unsigned long long pad[12];
};
static_assert(sizeof(WorkerCtl) == 256, "control block layout");

struct Args {
  const GraphDesc *graphs;
  const Task *tasks;
  uint32_t ntasks;
  uint32_t *out;
  uint32_t *next_task;
  // per-worker state, worker w at base + w * stride (elements)
  uint32_t *bitmaps;          // 4 * Wp words per worker
  uint64_t Wp;
  uint32_t *lists;            // 4 * cap words per worker: queue[2], far[2]
  uint4 *chunks;              // 2 * chunk_cap per worker
  WorkerCtl *ctl;
  uint32_t cap, chunk_cap;
  uint32_t huge, delta;
  uint32_t *err;
};

struct Ctx {
  uint32_t part, parts;       // CTA rank / count within the cluster
  uint32_t ctid, cthreads;    // thread rank / count within the cluster
};

// ---- BFS ------------------------------------------------------------------
struct BfsVisitor {
  const GraphDesc *g;
  uint32_t *visited, *depth, nd;
  uint32_t *qnext, qcap;
  uint4 *cnext;
  uint32_t ccap, huge;
  Slot *nx;
  uint32_t *err;
  using aux_t = uint32_t;
  __device__ __forceinline__ uint32_t aux(uint32_t) const { return 0u; }
  __device__ __forceinline__ void edge(uint32_t, uint32_t, uint32_t x) {
    const uint32_t dst = __ldg(g->cols + x);
    const uint32_t w = dst >> 5, bit = 1u << (dst & 31u);
    if (__ldcg(visited + w) & bit) return;
    if (atomicOr(visited + w, bit) & bit) return;
    depth[dst] = nd;
    const uint32_t b = __ldg(g->offs + dst), e = __ldg(g->offs + dst + 1);
    if (!push_binned(dst, b, e, huge, qnext, &nx->qcount, qcap, cnext, &nx->ccount, ccap))
      atomicOr(err, kErrOverflow);
  }
};

__device__ void run_bfs(const Args &a, const Ctx &c, cg::cluster_group &cl, const GraphDesc *g,
                        uint32_t src, uint32_t *depth, uint32_t *bm, uint32_t *lists, uint4 *chunks,
                        WorkerCtl *ctl) {
  const uint32_t n = g->n, W = (n + 31) / 32;
  uint32_t *visited = bm;
  uint32_t *queue[2] = {lists, lists + a.cap};
  uint4 *ch[2] = {chunks, chunks + a.chunk_cap};
  for (uint32_t i = c.ctid; i < W; i += c.cthreads) visited[i] = 0u;
  if (c.ctid < 4 * sizeof(Slot) / 4) ((uint32_t *)ctl->slots)[c.ctid] = 0u;
  cl.sync();
  if (c.ctid == 0) {
    visited[src >> 5] = 1u << (src & 31u);
    depth[src] = 0u;
    const uint32_t b = __ldg(g->offs + src), e = __ldg(g->offs + src + 1);
    if (!push_binned(src, b, e, a.huge, queue[0], &ctl->slots[0].qcount, a.cap, ch[0],
                     &ctl->slots[0].ccount, a.chunk_cap))
      atomicOr(&ctl->err, kErrOverflow);
  }
  cl.sync();
  uint32_t L = 0;
  while (true) {
    Slot *cur = ctl->slots + (L & 3u), *nx = ctl->slots + ((L + 1) & 3u);
    if (c.ctid < sizeof(Slot) / 4) ((uint32_t *)(ctl->slots + ((L + 2) & 3u)))[c.ctid] = 0u;
    BfsVisitor vis{g, visited, depth, L + 1, queue[(L + 1) & 1u], a.cap, ch[(L + 1) & 1u],
                   a.chunk_cap, a.huge, nx, &ctl->err};
    expand_binned<kBatchBlock>(g->offs, queue[L & 1u], min(__ldcg(&cur->qcount), a.cap), ch[L & 1u],
                               min(__ldcg(&cur->ccount), a.chunk_cap), vis, c.part, c.parts);
    cl.sync();
    ++L;
    if (__ldcg(&nx->qcount) + __ldcg(&nx->ccount) == 0) break;
    if (L > n + 1) {
      if (c.ctid == 0) atomicOr(&ctl->err, kErrLevels);
      break;
    }
  }
  // unreached vertices read INFINIT (each lane one vertex of a visited word)
  for (uint32_t v = c.ctid; v < n; v += c.cthreads)
    if (!((__ldcg(visited + (v >> 5)) >> (v & 31u)) & 1u)) depth[v] = kBatchInfinit;
  if (c.ctid == 0) ctl->levels = L;
  cl.sync();
}

// ---- SSSP -----------------------------------------------------------------
struct RelaxVisitor {
  const GraphDesc *g;
  uint32_t *dist, T;
  uint32_t *inq_next, *farbm, *qnext, *farp, *farcount, qcap;
  uint4 *cnext;
  uint32_t ccap, huge;
  Slot *nx;
  uint32_t *err;
  unsigned long long visits;
  using aux_t = uint32_t;
  __device__ __forceinline__ uint32_t aux(uint32_t v) const { return __ldcg(dist + v); }
  __device__ __forceinline__ void to_near(uint32_t v) {
    const uint32_t w = v >> 5, bit = 1u << (v & 31u);
    if (__ldcg(inq_next + w) & bit) return;
    if (atomicOr(inq_next + w, bit) & bit) return;
    const uint32_t b = __ldg(g->offs + v), e = __ldg(g->offs + v + 1);
    if (!push_binned(v, b, e, huge, qnext, &nx->qcount, qcap, cnext, &nx->ccount, ccap))
      atomicOr(err, kErrOverflow);
  }
  __device__ __forceinline__ void edge(uint32_t, uint32_t du, uint32_t x) {
    ++visits;
    const uint32_t v = __ldg(g->cols + x);
    const uint32_t nd = du + __ldg(g->wts + x);
    if (nd >= __ldcg(dist + v)) return;
    atomicMin(dist + v, nd);  // reduction; the bitmaps deduplicate the marks
    if (nd < T) {
      to_near(v);
    } else {
      const uint32_t w = v >> 5, bit = 1u << (v & 31u);
      if (__ldcg(farbm + w) & bit) return;
      if (atomicOr(farbm + w, bit) & bit) return;
      const uint32_t pos = agg_reserve(farcount);
      if (pos < qcap) farp[pos] = v;
      else atomicOr(err, kErrOverflow);
    }
  }
};

__device__ void run_sssp(const Args &a, const Ctx &c, cg::cluster_group &cl, const GraphDesc *g,
                         uint32_t src, uint32_t *dist, uint32_t *bm, uint32_t *lists, uint4 *chunks,
                         WorkerCtl *ctl) {
  const uint32_t n = g->n, W = (n + 31) / 32;
  const uint64_t Wp = a.Wp;
  uint32_t *inq[3] = {bm, bm + Wp, bm + 2 * Wp};
  uint32_t *farbm = bm + 3 * Wp;
  uint32_t *queue[2] = {lists, lists + a.cap};
  uint32_t *far[2] = {lists + 2 * (uint64_t)a.cap, lists + 3 * (uint64_t)a.cap};
  uint4 *ch[2] = {chunks, chunks + a.chunk_cap};
  for (uint32_t i = c.ctid; i < n; i += c.cthreads) dist[i] = kBatchInfinit;
  for (uint32_t i = c.ctid; i < W; i += c.cthreads) {
    inq[0][i] = 0u;
    inq[1][i] = 0u;
    inq[2][i] = 0u;
    farbm[i] = 0u;
  }
  if (c.ctid < 4 * sizeof(Slot) / 4) ((uint32_t *)ctl->slots)[c.ctid] = 0u;
  if (c.ctid < sizeof(FarCtl) / 4) ((uint32_t *)&ctl->far)[c.ctid] = 0u;
  cl.sync();
  if (c.ctid == 0) {
    dist[src] = 0u;
    const uint32_t b = __ldg(g->offs + src), e = __ldg(g->offs + src + 1);
    if (!push_binned(src, b, e, a.huge, queue[0], &ctl->slots[0].qcount, a.cap, ch[0],
                     &ctl->slots[0].ccount, a.chunk_cap))
      atomicOr(&ctl->err, kErrOverflow);
  }
  cl.sync();
  uint32_t L = 0, T = a.delta, fsel = 0, splits = 0;
  unsigned long long visits = 0;
  while (true) {
    Slot *cur = ctl->slots + (L & 3u), *nx = ctl->slots + ((L + 1) & 3u);
    uint32_t *inq_next = inq[(L + 1) % 3], *inq_clr = inq[(L + 2) % 3];
    for (uint32_t i = c.ctid; i < W; i += c.cthreads) inq_clr[i] = 0u;
    if (c.ctid < sizeof(Slot) / 4) ((uint32_t *)(ctl->slots + ((L + 2) & 3u)))[c.ctid] = 0u;
    RelaxVisitor vis{g, dist, T, inq_next, farbm, queue[(L + 1) & 1u], far[fsel],
                     &ctl->far.count[fsel], a.cap, ch[(L + 1) & 1u], a.chunk_cap, a.huge, nx,
                     &ctl->err, 0ull};
    expand_binned<kBatchBlock>(g->offs, queue[L & 1u], min(__ldcg(&cur->qcount), a.cap), ch[L & 1u],
                               min(__ldcg(&cur->ccount), a.chunk_cap), vis, c.part, c.parts);
    visits += vis.visits;
    cl.sync();
    ++L;
    bool done = false;
    while (__ldcg(&nx->qcount) + __ldcg(&nx->ccount) == 0) {
      const uint32_t fc = min(__ldcg(&ctl->far.count[fsel]), a.cap);
      if (fc == 0) {
        done = true;
        break;
      }
      const uint32_t Told = T;
      uint32_t Tnew = T + a.delta;
      const uint32_t mf = __ldcg(&ctl->far.minfar[splits & 1u]);
      if (splits && mf != 0xFFFFFFFFu && mf >= Tnew) Tnew = (mf / a.delta + 1) * a.delta;
      if (c.ctid == 0) {
        ctl->far.count[fsel ^ 1u] = 0u;
        ctl->far.minfar[(splits + 1) & 1u] = 0xFFFFFFFFu;
      }
      cl.sync();
      const uint32_t *fp = far[fsel];
      uint32_t *kp = far[fsel ^ 1u];
      uint32_t local_min = 0xFFFFFFFFu;
      for (uint32_t i = c.ctid; i < fc; i += c.cthreads) {
        const uint32_t v = __ldcg(fp + i);
        const uint32_t d = __ldcg(dist + v);
        const uint32_t w = v >> 5, bit = 1u << (v & 31u);
        if (d < Told) {
          atomicAnd(farbm + w, ~bit);
        } else if (d < Tnew) {
          atomicAnd(farbm + w, ~bit);
          vis.to_near(v);
        } else {
          const uint32_t pos = agg_reserve(&ctl->far.count[fsel ^ 1u]);
          kp[pos] = v;
          local_min = min(local_min, d);
        }
      }
      for (int o = 16; o > 0; o >>= 1)
        local_min = min(local_min, __shfl_down_sync(0xffffffffu, local_min, o));
      if (lane_id() == 0 && local_min != 0xFFFFFFFFu)
        atomicMin(&ctl->far.minfar[(splits + 1) & 1u], local_min);
      T = Tnew;
      fsel ^= 1u;
      ++splits;
      cl.sync();
    }
    if (done) break;
    if (L > 4u * n + 64u) {
      if (c.ctid == 0) atomicOr(&ctl->err, kErrLevels);
      break;
    }
  }
  if (c.ctid == 0) ctl->levels = L;
  if (visits) atomicAdd(&ctl->visits, visits);
  cl.sync();
}

__global__ void __launch_bounds__(kBatchBlock, 4) batch_kernel(Args a) {
  cg::cluster_group cl = cg::this_cluster();
  __shared__ uint32_t s_task;
  Ctx c;
  c.part = cl.block_rank();
  c.parts = cl.num_blocks();
  c.ctid = c.part * kBatchBlock + threadIdx.x;
  c.cthreads = c.parts * kBatchBlock;
  const uint32_t worker = blockIdx.x / c.parts;
  uint32_t *bm = a.bitmaps + (uint64_t)worker * 4 * a.Wp;
  uint32_t *lists = a.lists + (uint64_t)worker * 4 * a.cap;
  uint4 *chunks = a.chunks + (uint64_t)worker * 2 * a.chunk_cap;
  WorkerCtl *ctl = a.ctl + worker;
  if (c.ctid < sizeof(WorkerCtl) / 4) ((uint32_t *)ctl)[c.ctid] = 0u;
  while (true) {
    if (c.part == 0 && threadIdx.x == 0) s_task = atomicAdd(a.next_task, 1u);
    cl.sync();
    const uint32_t t = *cl.map_shared_rank(&s_task, 0);
    // every CTA has read the leader's word before it is rewritten or the
    // leader exits (a CTA's shared memory must outlive remote reads)
    cl.sync();
    if (t >= a.ntasks) break;
    const Task task = a.tasks[t];
    const GraphDesc *g = a.graphs + task.graph;
    uint32_t *out = a.out + task.out_off;
    if (task.algo == kAlgoSssp && g->wts)
      run_sssp(a, c, cl, g, task.src, out, bm, lists, chunks, ctl);
    else
      run_bfs(a, c, cl, g, task.src, out, bm, lists, chunks, ctl);
  }
  if (c.ctid == 0 && ctl->err) atomicOr(a.err, ctl->err);
}

}  // namespace batch

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
using namespace batch;

// Clusters of up to 16 CTAs: sizes above the portable 8 need an opt-in per
// kernel (set once per process).
static int allow_wide_clusters() {
  static int done = 0;
  if (!done) {
    GRUS_CUDA_TRY(cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    done = 1;
  }
  return GRUS_OK;
}

int batch_occupancy(int cluster, int *workers) {
  if (cluster > 8) {
    const int rc = allow_wide_clusters();
    if (rc) return rc;
  }
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = cluster;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.gridDim = dim3(cluster * 64);
  cfg.blockDim = dim3(kBatchBlock);
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  int nc = 0;
  GRUS_CUDA_TRY(cudaOccupancyMaxActiveClusters(&nc, batch_kernel, &cfg));
  *workers = nc;
  return GRUS_OK;
}

void BatchState::release() {
  cudaFree(bitmaps);
  cudaFree(lists);
  cudaFree(chunks);
  cudaFree(ctl);
  cudaFree(counter);
  cudaFree(err);
  bitmaps = lists = counter = err = nullptr;
  chunks = nullptr;
  ctl = nullptr;
  workers = 0;
}

int BatchState::reserve(int nworkers, uint64_t max_n, uint64_t max_m, uint32_t huge) {
  const uint64_t Wneed = ((max_n + 31) / 32 + 31) / 32 * 32;
  const uint32_t capn = (uint32_t)std::max<uint64_t>(max_n, 1);
  const uint32_t ccapn = (uint32_t)(max_m / kChunk + max_m / std::max(huge, 1u) + 2);
  if (nworkers <= workers && Wneed <= Wp && capn <= cap && ccapn <= chunk_cap) return GRUS_OK;
  release();
  Wp = Wneed;
  cap = capn;
  chunk_cap = ccapn;
  cudaError_t e = cudaMalloc(&bitmaps, (uint64_t)nworkers * 4 * Wp * 4);
  if (e == cudaSuccess) e = cudaMalloc(&lists, (uint64_t)nworkers * 4 * cap * 4);
  if (e == cudaSuccess) e = cudaMalloc(&chunks, (uint64_t)nworkers * 2 * chunk_cap * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&ctl, (uint64_t)nworkers * sizeof(WorkerCtl));
  if (e == cudaSuccess) e = cudaMalloc(&counter, 4);
  if (e == cudaSuccess) e = cudaMalloc(&err, 4);
  if (e == cudaSuccess) e = cudaMemset(err, 0, 4);  // read back after every run
  if (e != cudaSuccess) {
    cudaGetLastError();
    release();
    set_last_error(std::string("batch state: ") + cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  workers = nworkers;
  return GRUS_OK;
}

size_t BatchState::bytes_per_worker(uint64_t max_n, uint64_t max_m, uint32_t huge) {
  const uint64_t Wpp = ((max_n + 31) / 32 + 31) / 32 * 32;
  const uint64_t ccapn = max_m / kChunk + max_m / std::max(huge, 1u) + 2;
  return 4 * Wpp * 4 + 4 * std::max<uint64_t>(max_n, 1) * 4 + 2 * ccapn * sizeof(uint4) +
         sizeof(WorkerCtl);
}

int batch_launch(BatchState &st, int worker0, int nworkers, int cluster, const GraphDesc *graphs,
                 const Task *tasks, uint32_t ntasks, uint32_t *out, uint32_t huge, uint32_t delta,
                 uint32_t *counter, cudaStream_t s) {
  Args a;
  std::memset(&a, 0, sizeof(a));
  a.graphs = graphs;
  a.tasks = tasks;
  a.ntasks = ntasks;
  a.out = out;
  a.next_task = counter;
  a.Wp = st.Wp;
  a.bitmaps = st.bitmaps + (uint64_t)worker0 * 4 * st.Wp;
  a.lists = st.lists + (uint64_t)worker0 * 4 * st.cap;
  a.chunks = st.chunks + (uint64_t)worker0 * 2 * st.chunk_cap;
  a.ctl = (WorkerCtl *)st.ctl + worker0;
  a.cap = st.cap;
  a.chunk_cap = st.chunk_cap;
  a.huge = huge;
  a.delta = std::max(delta, 1u);
  a.err = st.err;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = cluster;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)(cluster * nworkers));
  cfg.blockDim = dim3(kBatchBlock);
  cfg.stream = s;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  GRUS_CUDA_TRY(cudaLaunchKernelEx(&cfg, batch_kernel, a));
  return GRUS_OK;
}

GraphDesc describe(const grus_graph *g) {
  GraphDesc d;
  d.offs = g->csr.offs;
  d.cols = g->csr.cols;
  d.wts = g->csr.wts;
  d.n = (uint32_t)g->n;
  d.flags = g->flags;
  d.m = g->m;
  return d;
}

}  // namespace grus

// ---------------------------------------------------------------------------
// C ABI: plans (resident descriptor tables + worker state), optionally
// replayed as a CUDA graph.
// ---------------------------------------------------------------------------
struct grus_batch {
  std::vector<grus_graph *> graphs;
  grus::GraphDesc *d_graphs = nullptr;
  grus::Task *d_tasks = nullptr, *h_tasks = nullptr;  // pinned staging
  uint32_t task_cap = 0;
  grus::BatchState state;
  int cluster = 16, workers = 0;
  uint32_t huge = 1024, delta = 96;
  uint64_t max_n = 0, max_m = 0, total_out = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint32_t graph_ntasks = 0;
  uint32_t *graph_out = nullptr;
  cudaStream_t graph_stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t done = nullptr;  // last run's work (staging may be rewritten after it)
  bool in_flight = false;
};

using namespace grus;

extern "C" {

int grus_batch_create(grus_graph *const *graphs, int ngraphs, const grus_batch_config *cfg,
                      grus_batch **out) {
  if (!graphs || ngraphs < 1 || !out) return GRUS_EINVAL;
  grus_batch *b = new grus_batch();
  b->graphs.assign(graphs, graphs + ngraphs);
  std::vector<GraphDesc> descs;
  for (int i = 0; i < ngraphs; ++i) {
    if (!graphs[i]) {
      delete b;
      return GRUS_EINVAL;
    }
    descs.push_back(describe(graphs[i]));
    b->max_n = std::max<uint64_t>(b->max_n, graphs[i]->n);
    b->max_m = std::max<uint64_t>(b->max_m, graphs[i]->m);
  }
  if (cfg) {
    if (cfg->cluster_size) b->cluster = (int)cfg->cluster_size;
    if (cfg->huge_degree) b->huge = cfg->huge_degree;
    if (cfg->sssp_delta) b->delta = cfg->sssp_delta;
    if (cfg->workers) b->workers = (int)cfg->workers;
  }
  if (b->cluster < 1 || b->cluster > 16) {
    delete b;
    set_last_error("cluster_size must be 1..16");
    return GRUS_EINVAL;
  }
  int maxw = 0;
  int rc = batch_occupancy(b->cluster, &maxw);
  if (!rc && maxw < 1) {
    set_last_error("batch kernel: no cluster can be resident");
    rc = GRUS_ECUDA;
  }
  if (!rc) {
    b->workers = b->workers ? std::min(b->workers, maxw) : maxw;
    rc = b->state.reserve(b->workers, b->max_n, b->max_m, b->huge);
  }
  cudaError_t e = cudaSuccess;
  if (!rc) e = cudaMalloc(&b->d_graphs, ngraphs * sizeof(GraphDesc));
  if (!rc && e == cudaSuccess)
    e = cudaMemcpy(b->d_graphs, descs.data(), ngraphs * sizeof(GraphDesc), cudaMemcpyHostToDevice);
  if (!rc && e == cudaSuccess) e = cudaEventCreate(&b->ev0);
  if (!rc && e == cudaSuccess) e = cudaEventCreate(&b->ev1);
  if (!rc && e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  if (!rc && e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    rc = status_from_cuda(e);
  }
  if (rc) {
    grus_batch_free(b);
    return rc;
  }
  *out = b;
  return GRUS_OK;
}

static int ensure_tasks(grus_batch *b, uint32_t n) {
  if (n <= b->task_cap) return GRUS_OK;
  if (b->exec) {  // a captured graph points at the old buffers
    cudaGraphExecDestroy(b->exec);
    cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
  }
  cudaFree(b->d_tasks);
  cudaFreeHost(b->h_tasks);
  b->d_tasks = nullptr;
  b->h_tasks = nullptr;
  b->task_cap = 0;
  GRUS_CUDA_TRY(cudaMalloc(&b->d_tasks, n * sizeof(Task)));
  GRUS_CUDA_TRY(cudaMallocHost(&b->h_tasks, n * sizeof(Task)));
  b->task_cap = n;
  return GRUS_OK;
}

// Work items in descending graph size first, so large queries start early.
static void stage_tasks(grus_batch *b, const grus_query *q, int nq) {
  std::vector<int> order(nq);
  for (int i = 0; i < nq; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return b->graphs[q[x].graph]->m > b->graphs[q[y].graph]->m;
  });
  for (int i = 0; i < nq; ++i) {
    const grus_query &s = q[order[i]];
    Task &t = b->h_tasks[i];
    t.graph = s.graph;
    t.algo = s.algo;
    t.src = s.src;
    t.pad = 0;
    t.out_off = s.out_offset;
  }
}

int grus_batch_run(grus_batch *b, const grus_query *queries, int nq, uint32_t *out,
                   int use_graph, grus_stats *stats, void *stream) {
  if (!b || !queries || nq < 0 || !out) return GRUS_EINVAL;
  if (nq == 0) return GRUS_OK;
  for (int i = 0; i < nq; ++i) {
    if (queries[i].graph >= b->graphs.size()) return GRUS_EINVAL;
    const grus_graph *g = b->graphs[queries[i].graph];
    if (queries[i].src >= g->n || queries[i].algo > GRUS_ALGO_SSSP) return GRUS_EINVAL;
    if (queries[i].algo == GRUS_ALGO_SSSP && !g->csr.wts) {
      set_last_error("sssp query on an unweighted graph");
      return GRUS_EINVAL;
    }
  }
  if (!is_device_pointer(out)) {
    set_last_error("grus_batch_run writes device memory (out must be device or managed)");
    return GRUS_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  // the pinned staging buffer is read by the previous run's copy: wait for it
  if (b->in_flight) GRUS_CUDA_TRY(cudaEventSynchronize(b->done));
  int rc = ensure_tasks(b, (uint32_t)nq);
  if (rc) return rc;
  stage_tasks(b, queries, nq);
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(b->ev0, s));
  if (use_graph) {
    // one captured graph per (task count, output buffer): H2D copy of the
    // staged tasks, counter reset, batch kernel
    if (b->exec && (b->graph_ntasks != (uint32_t)nq || b->graph_out != out || b->graph_stream != s)) {
      cudaGraphExecDestroy(b->exec);
      cudaGraphDestroy(b->graph);
      b->exec = nullptr;
      b->graph = nullptr;
    }
    if (!b->exec) {
      cudaStream_t cap_s = nullptr;
      GRUS_CUDA_TRY(cudaStreamCreateWithFlags(&cap_s, cudaStreamNonBlocking));
      cudaError_t e = cudaStreamBeginCapture(cap_s, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaMemcpyAsync(b->d_tasks, b->h_tasks, nq * sizeof(Task), cudaMemcpyHostToDevice, cap_s);
        cudaMemsetAsync(b->state.counter, 0, 4, cap_s);
        rc = batch_launch(b->state, 0, b->workers, b->cluster, b->d_graphs, b->d_tasks, nq, out,
                          b->huge, b->delta, b->state.counter, cap_s);
        e = cudaStreamEndCapture(cap_s, &b->graph);
      }
      cudaStreamDestroy(cap_s);
      if (rc) return rc;
      GRUS_CUDA_TRY(e);
      GRUS_CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
      b->graph_ntasks = (uint32_t)nq;
      b->graph_out = out;
      b->graph_stream = s;
    }
    GRUS_CUDA_TRY(cudaGraphLaunch(b->exec, s));
  } else {
    GRUS_CUDA_TRY(cudaMemcpyAsync(b->d_tasks, b->h_tasks, nq * sizeof(Task), cudaMemcpyHostToDevice, s));
    GRUS_CUDA_TRY(cudaMemsetAsync(b->state.counter, 0, 4, s));
    rc = batch_launch(b->state, 0, b->workers, b->cluster, b->d_graphs, b->d_tasks, nq, out, b->huge,
                      b->delta, b->state.counter, s);
    if (rc) return rc;
  }
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(b->ev1, s));
  GRUS_CUDA_TRY(cudaEventRecord(b->done, s));
  b->in_flight = true;
  if (!stats) return GRUS_OK;
  uint32_t err = 0;
  GRUS_CUDA_TRY(cudaMemcpyAsync(&err, b->state.err, 4, cudaMemcpyDeviceToHost, s));
  GRUS_CUDA_TRY(cudaStreamSynchronize(s));
  if (err) {
    cudaMemset(b->state.err, 0, 4);
    return status_from_device_error(err);
  }
  std::memset(stats, 0, sizeof(*stats));
  stats->kernel_launches = 1;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  stats->device_ms = ms;
  return GRUS_OK;
}

int grus_batch_get_info(const grus_batch *b, grus_batch_config *info) {
  if (!b || !info) return GRUS_EINVAL;
  std::memset(info, 0, sizeof(*info));
  info->cluster_size = (uint32_t)b->cluster;
  info->workers = (uint32_t)b->workers;
  info->huge_degree = b->huge;
  info->sssp_delta = b->delta;
  return GRUS_OK;
}

int grus_batch_free(grus_batch *b) {
  if (!b) return GRUS_EINVAL;
  cudaDeviceSynchronize();
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->state.release();
  cudaFree(b->d_graphs);
  cudaFree(b->d_tasks);
  if (b->h_tasks) cudaFreeHost(b->h_tasks);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->done) cudaEventDestroy(b->done);
  delete b;
  return GRUS_OK;
}

}  // extern "C"
