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
//   SSSP : the near/far label-correcting scheme of sssp.cu (bitmap sets,
//          atomicMin, Delta buckets), scoped to the cluster.
//   SSSP group : up to 32 SSSP queries on one graph as ONE multi-source
//          traversal (msssp_core.cuh) scoped to the cluster, sharing every
//          adjacency read; the host packs queries on the same graph into
//          such groups.
// Queries on graphs of at least big_edges edges do not go to the cluster
// workers: a 16-CTA worker is a small slice of the GPU and such a query would
// set the batch's critical path, so they run first as whole-GPU launches.
// SSSP: up to 32 queries per graph form a pack, and the packs of up to 64
// graphs share ONE multi-graph multi-source launch (msssp.cu), so the graphs'
// levels overlap instead of following one another; BFS: up to 64 sources per
// launch when the graph has enough BFS queries for a pack to beat single
// launches, else one launch each.
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
#include "msssp_core.cuh"
#include "union_plan.h"

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
static_assert(sizeof(Slot) == sizeof(ms::Slot), "multi-source slots reuse the worker slots");

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
  // multi-source groups
  const uint32_t *msrc;
  const unsigned long long *moff;
  uint32_t *ms_d, *ms_masks;
  uint4 *ms_ent;
  uint64_t ms_n;
  uint32_t ms_ks, ms_ent_cap;
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
// The bitmap near/far scheme of sssp.cu scoped to the cluster: near sets
// N[2] and the far set are bitmaps, compacted into the binned lists once per
// level, and a relaxation waits on no atomic.
struct RelaxVisitor {
  const GraphDesc *g;
  uint32_t *dist, T;
  uint32_t *nnext, *farbm;
  unsigned long long visits;
  using aux_t = uint32_t;
  __device__ __forceinline__ uint32_t aux(uint32_t v) const { return __ldcg(dist + v); }
  __device__ __forceinline__ void edge(uint32_t, uint32_t du, uint32_t x) {
    ++visits;
    const uint32_t v = __ldg(g->cols + x);
    const uint32_t nd = du + __ldg(g->wts + x);
    if (nd >= __ldcg(dist + v)) return;
    atomicMin(dist + v, nd);  // reductions; a raced mark costs one redundant expansion
    atomicOr((nd < T ? nnext : farbm) + (v >> 5), 1u << (v & 31u));
  }
};

__device__ void run_sssp(const Args &a, const Ctx &c, cg::cluster_group &cl, const GraphDesc *g,
                         uint32_t src, uint32_t *dist, uint32_t *bm, uint32_t *lists, uint4 *chunks,
                         WorkerCtl *ctl) {
  const uint32_t n = g->n, W = (n + 31) / 32;
  const uint64_t Wp = a.Wp;
  uint32_t *near[2] = {bm, bm + Wp};
  uint32_t *farbm = bm + 3 * Wp;
  uint32_t *queue = lists;
  for (uint32_t i = c.ctid; i < n; i += c.cthreads) dist[i] = kBatchInfinit;
  for (uint32_t i = c.ctid; i < W; i += c.cthreads) {
    near[0][i] = 0u;
    near[1][i] = 0u;
    farbm[i] = 0u;
  }
  if (c.ctid < 4 * sizeof(Slot) / 4) ((uint32_t *)ctl->slots)[c.ctid] = 0u;
  if (c.ctid < sizeof(FarCtl) / 4) ((uint32_t *)&ctl->far)[c.ctid] = 0u;
  if (c.ctid == 0) {
    ctl->far.minfar[0] = 0xFFFFFFFFu;
    ctl->far.minfar[1] = 0xFFFFFFFFu;
  }
  cl.sync();
  if (c.ctid == 0) {
    dist[src] = 0u;
    near[0][src >> 5] = 1u << (src & 31u);
  }
  cl.sync();
  uint32_t L = 0, T = a.delta, splits = 0;
  unsigned long long visits = 0;
  while (true) {
    Slot *sl = ctl->slots + (L & 3u);
    if (c.ctid < sizeof(Slot) / 4) ((uint32_t *)(ctl->slots + ((L + 2) & 3u)))[c.ctid] = 0u;
    uint32_t *ncur = near[L & 1u], *nnext = near[(L + 1) & 1u];
    bitmap_to_binned<kBatchBlock>(ncur, W, g->offs, a.huge, queue, &sl->qcount, a.cap, chunks,
                                  &sl->ccount, a.chunk_cap, &ctl->err, c.part, c.parts);
    cl.sync();
    const uint32_t qc = min(__ldcg(&sl->qcount), a.cap);
    const uint32_t cc = min(__ldcg(&sl->ccount), a.chunk_cap);
    if (qc + cc == 0) {
      // nothing near: advance the threshold and split the far set into ncur
      // (minfar[j & 1]: smallest distance left by split j - 1; FarCtl.count
      // holds the split's moved / remaining counters)
      const uint32_t Told = T;
      uint32_t Tnew = T + a.delta;
      const uint32_t mf = __ldcg(&ctl->far.minfar[splits & 1u]);
      if (mf != 0xFFFFFFFFu && mf >= Tnew) Tnew = (mf / a.delta + 1) * a.delta;
      uint32_t moved = 0, remaining = 0, local_min = 0xFFFFFFFFu;
      for (uint32_t w = c.ctid; w < W; w += c.cthreads) {
        const uint32_t fw = __ldcg(farbm + w);
        if (!fw) continue;
        uint32_t keep = 0, mv = 0;
        for (uint32_t bits = fw; bits; bits &= bits - 1) {
          const uint32_t b = __ffs(bits) - 1;
          const uint32_t d = __ldcg(dist + w * 32 + b);
          if (d < Told) continue;
          if (d < Tnew) {
            mv |= 1u << b;
          } else {
            keep |= 1u << b;
            local_min = min(local_min, d);
          }
        }
        farbm[w] = keep;
        if (mv) ncur[w] = mv;
        moved += __popc(mv);
        remaining += keep != 0;
      }
      for (int o = 16; o > 0; o >>= 1) {
        local_min = min(local_min, __shfl_down_sync(0xffffffffu, local_min, o));
        moved += __shfl_down_sync(0xffffffffu, moved, o);
        remaining += __shfl_down_sync(0xffffffffu, remaining, o);
      }
      if (lane_id() == 0) {
        if (local_min != 0xFFFFFFFFu) atomicMin(&ctl->far.minfar[(splits + 1) & 1u], local_min);
        if (moved) atomicAdd(&ctl->far.count[0], moved);
        if (remaining) atomicAdd(&ctl->far.count[1], remaining);
      }
      cl.sync();
      const uint32_t mv_all = __ldcg(&ctl->far.count[0]), rem_all = __ldcg(&ctl->far.count[1]);
      if (c.ctid == 0) ctl->far.minfar[splits & 1u] = 0xFFFFFFFFu;
      T = Tnew;
      ++splits;
      cl.sync();
      if (c.ctid == 0) {
        ctl->far.count[0] = 0u;
        ctl->far.count[1] = 0u;
      }
      if (mv_all == 0 && rem_all == 0) break;
      continue;
    }
    RelaxVisitor vis{g, dist, T, nnext, farbm, 0ull};
    expand_binned<kBatchBlock>(g->offs, queue, qc, chunks, cc, vis, c.part, c.parts);
    visits += vis.visits;
    cl.sync();
    ++L;
    if (L > 4u * n + 64u) {
      if (c.ctid == 0) atomicOr(&ctl->err, kErrLevels);
      break;
    }
  }
  if (c.ctid == 0) ctl->levels = L;
  if (visits) atomicAdd(&ctl->visits, visits);
  cl.sync();
}

// ---- SSSP group -----------------------------------------------------------
struct ClusterSync {
  cg::cluster_group *cl;
  __device__ __forceinline__ bool operator()() const {
    cl->sync();
    return true;
  }
};

struct GroupOut {
  uint32_t *out;
  const unsigned long long *moff;
  __device__ __forceinline__ uint32_t *operator()(uint32_t s) const { return out + moff[s]; }
};

__device__ void run_msssp(const Args &a, const Ctx &c, cg::cluster_group &cl, const GraphDesc *g,
                          const Task &task, uint32_t worker, WorkerCtl *ctl) {
  ms::View v;
  v.offs = g->offs;
  v.cols = g->cols;
  v.wts = g->wts;
  v.n = g->n;
  v.k = task.pad;
  v.srcs = a.msrc + task.src;
  v.D = a.ms_d + (uint64_t)worker * a.ms_n * a.ms_ks;
  uint32_t *masks = a.ms_masks + (uint64_t)worker * 3 * a.ms_n;
  v.F[0] = masks;
  v.F[1] = masks + a.ms_n;
  v.far = masks + 2 * a.ms_n;
  v.ent = a.ms_ent + (uint64_t)worker * a.ms_ent_cap;
  v.ent_cap = a.ms_ent_cap;
  v.slots = (ms::Slot *)ctl->slots;
  v.minfar = ctl->far.minfar;
  v.err = &ctl->err;
  v.delta = a.delta;
  ClusterSync sync{&cl};
  GroupOut out{a.out, a.moff + task.src};
  ms::Result r;
  if (v.k <= 8) ms::run<8, kBatchBlock>(v, c.ctid, c.cthreads, sync, out, r);
  else if (v.k <= 16) ms::run<16, kBatchBlock>(v, c.ctid, c.cthreads, sync, out, r);
  else ms::run<32, kBatchBlock>(v, c.ctid, c.cthreads, sync, out, r);
  if (c.ctid == 0) ctl->levels = r.levels;
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
    if (task.algo == kAlgoSsspMulti) {
      if (g->wts && a.ms_d && task.pad >= 1 && task.pad <= a.ms_ks)
        run_msssp(a, c, cl, g, task, worker, ctl);
      else if (c.ctid == 0)
        atomicOr(&ctl->err, kErrOverflow);  // no group state: the host sized it wrong
    } else if (task.algo == kAlgoSssp && g->wts)
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
  cudaLaunchConfig_t cfg = {};
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

void BatchState::release_multi() {
  cudaFree(ms_d);
  cudaFree(ms_masks);
  cudaFree(ms_ent);
  ms_d = ms_masks = nullptr;
  ms_ent = nullptr;
  ms_n = 0;
  ms_ks = ms_ent_cap = 0;
  ms_workers = 0;
}

int BatchState::reserve_multi(int nworkers, uint64_t max_n, uint64_t max_m, uint32_t ks) {
  const uint64_t n1 = std::max<uint64_t>(max_n, 1);
  const uint32_t ecap = (uint32_t)std::min<uint64_t>(n1 + max_m / ms::kPiece + 1024, 0xFFFFFFF0ull);
  if (nworkers <= ms_workers && n1 <= ms_n && ks <= ms_ks && ecap <= ms_ent_cap) return GRUS_OK;
  release_multi();
  cudaError_t e = cudaMalloc(&ms_d, (uint64_t)nworkers * n1 * ks * 4);
  if (e == cudaSuccess) e = cudaMalloc(&ms_masks, (uint64_t)nworkers * 3 * n1 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&ms_ent, (uint64_t)nworkers * ecap * sizeof(uint4));
  if (e != cudaSuccess) {
    cudaGetLastError();
    release_multi();
    set_last_error(std::string("batch multi-source state: ") + cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  ms_n = n1;
  ms_ks = ks;
  ms_ent_cap = ecap;
  ms_workers = nworkers;
  return GRUS_OK;
}

void BatchState::release() {
  release_multi();
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
                 uint32_t *counter, cudaStream_t s, const uint32_t *msrc,
                 const unsigned long long *moff) {
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
  a.msrc = msrc;
  a.moff = moff;
  if (msrc && st.ms_d && worker0 + nworkers <= st.ms_workers) {
    a.ms_d = st.ms_d + (uint64_t)worker0 * st.ms_n * st.ms_ks;
    a.ms_masks = st.ms_masks + (uint64_t)worker0 * 3 * st.ms_n;
    a.ms_ent = st.ms_ent + (uint64_t)worker0 * st.ms_ent_cap;
    a.ms_n = st.ms_n;
    a.ms_ks = st.ms_ks;
    a.ms_ent_cap = st.ms_ent_cap;
  }
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = cluster;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
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
  // members of multi-source groups: sources and output offsets (pinned staging)
  uint32_t *d_msrc = nullptr, *h_msrc = nullptr;
  unsigned long long *d_moff = nullptr, *h_moff = nullptr;
  uint32_t member_cap = 0;
  uint32_t group = 1;                  // SSSP queries per multi-source group
  uint32_t ntasks = 0, nmembers = 0;   // of the staged plan
  uint64_t big_edges = 1ull << 21;     // graphs served by whole-GPU launches
  uint64_t launch_entries = 1ull << 23;  // distance entries per multi-graph launch
  std::vector<uint8_t> big;            // per graph
  uint32_t *h_errs = nullptr;          // pinned error words of whole-GPU launches
  uint32_t err_cap = 0;
  void *uws = nullptr;                 // multi-graph SSSP launches' workspace
  grus::BatchState state;
  int cluster = 16, workers = 0;
  uint32_t huge = 1024, delta = 192;
  uint64_t max_n = 0, max_m = 0, total_out = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint32_t graph_ntasks = 0, graph_nmembers = 0;
  uint32_t *graph_out = nullptr;
  cudaStream_t graph_stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t done = nullptr;  // last run's work (staging may be rewritten after it)
  bool in_flight = false;
};

using namespace grus;

// SSSP queries on big graphs (big_q sorted by graph), grouped into launches
// by plan_union (union_plan.h): up to 32 per graph per pack, several graphs'
// packs per multi-graph launch while their distance rows total at most
// launch_entries.  The cap keeps a launch's distance rows in L2: 256 queries
// over 32 RMAT graphs of scales 14-20 in one launch (368 MB of rows) took
// 48.7 ms against 37 ms as one launch per graph.  Each launch's error word is
// copied to h_errs.
static int union_sssp(grus_batch *b, const grus_query *queries, const std::vector<int> &big_q,
                      uint32_t *out, cudaStream_t s, uint32_t *nerr, uint32_t *nlaunch) {
  std::vector<int> sssp;
  for (int qi : big_q)
    if (queries[qi].algo == GRUS_ALGO_SSSP) sssp.push_back(qi);
  if (sssp.empty()) return GRUS_OK;
  std::vector<uint32_t> qgraph(*std::max_element(sssp.begin(), sssp.end()) + 1);
  for (int qi : sssp) qgraph[qi] = queries[qi].graph;
  std::vector<uint64_t> gn(b->graphs.size()), gm(b->graphs.size());
  for (size_t g = 0; g < b->graphs.size(); ++g) {
    gn[g] = b->graphs[g]->n;
    gm[g] = b->graphs[g]->m;
  }
  const UnionPlan plan =
      plan_union(sssp, qgraph, gn, gm, b->launch_entries, (size_t)ms::kMaxUnion, ms::kPiece);
  if (plan.unions) {
    int rc = msssp_union_reserve(&b->uws, plan.unions, plan.max_v, plan.max_m, plan.max_ks);
    if (rc) return rc;
  }
  const auto &launches = plan.launches;
  int region = 0;
  for (const auto &l : launches) {
    CtrlView cv;
    int rc;
    if (l.size() == 1) {
      const UnionPack &p = l[0];
      grus_graph *g = b->graphs[p.graph];
      if (p.q.size() == 1) {
        const grus_query &q = queries[p.q[0]];
        rc = grus_sssp(g, q.src, out + q.out_offset, nullptr, s);
        cv = sssp_ctrl(g);
      } else {
        uint32_t srcs[32];
        uint32_t *outs[32];
        for (size_t k = 0; k < p.q.size(); ++k) {
          srcs[k] = queries[p.q[k]].src;
          outs[k] = out + queries[p.q[k]].out_offset;
        }
        rc = msssp_run(g, srcs, (int)p.q.size(), outs, nullptr, s);
        cv = msssp_ctrl(g);
      }
    } else {
      grus_graph *gs[ms::kMaxUnion];
      uint32_t kq[ms::kMaxUnion];
      std::vector<uint32_t> srcs;
      std::vector<uint32_t *> outs;
      for (size_t i = 0; i < l.size(); ++i) {
        gs[i] = b->graphs[l[i].graph];
        kq[i] = (uint32_t)l[i].q.size();
        for (int qi : l[i].q) {
          srcs.push_back(queries[qi].src);
          outs.push_back(out + queries[qi].out_offset);
        }
      }
      rc = msssp_union_run(b->uws, region++, gs, (int)l.size(), kq, srcs.data(), outs.data(), 0, s,
                           &cv);
    }
    if (rc) return rc;
    ++*nlaunch;
    if (cv.ctrl) {
      GRUS_CUDA_TRY(cudaMemcpyAsync(b->h_errs + *nerr, cv.ctrl + cv.err_off, 4,
                                    cudaMemcpyDeviceToHost, s));
      GRUS_CUDA_TRY(cudaMemsetAsync(cv.ctrl + cv.err_off, 0, 4, s));
      ++*nerr;
    }
  }
  return GRUS_OK;
}

extern "C" {

int grus_batch_create(grus_graph *const *graphs, int ngraphs, const grus_batch_config *cfg,
                      grus_batch **out) {
  if (!graphs || ngraphs < 1 || !out) return GRUS_EINVAL;
  grus_batch *b = new grus_batch();
  b->graphs.assign(graphs, graphs + ngraphs);
  std::vector<GraphDesc> descs;
  if (cfg && cfg->big_edges) b->big_edges = cfg->big_edges == 0xFFFFFFFFu ? ~0ull : cfg->big_edges;
  for (int i = 0; i < ngraphs; ++i) {
    if (!graphs[i]) {
      delete b;
      return GRUS_EINVAL;
    }
    descs.push_back(describe(graphs[i]));
    const bool big = graphs[i]->m >= b->big_edges;
    b->big.push_back(big ? 1 : 0);
    if (big) continue;  // the cluster workers never see this graph
    b->max_n = std::max<uint64_t>(b->max_n, graphs[i]->n);
    b->max_m = std::max<uint64_t>(b->max_m, graphs[i]->m);
  }
  if (cfg) {
    if (cfg->cluster_size) b->cluster = (int)cfg->cluster_size;
    if (cfg->huge_degree) b->huge = cfg->huge_degree;
    if (cfg->sssp_delta) b->delta = cfg->sssp_delta;
    if (cfg->workers) b->workers = (int)cfg->workers;
    if (cfg->group_sources) b->group = cfg->group_sources;
    if (cfg->launch_entries) b->launch_entries = cfg->launch_entries;
  }
  if (b->group < 1 || b->group > (uint32_t)kMaxGroup) {
    delete b;
    set_last_error("group_sources must be 1..32");
    return GRUS_EINVAL;
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

static void drop_graph(grus_batch *b) {
  if (b->exec) {  // a captured graph points at the old buffers
    cudaGraphExecDestroy(b->exec);
    cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
  }
}

static int ensure_tasks(grus_batch *b, uint32_t n) {
  if (n <= b->task_cap) return GRUS_OK;
  drop_graph(b);
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

static int ensure_members(grus_batch *b, uint32_t n) {
  if (n <= b->member_cap) return GRUS_OK;
  drop_graph(b);
  cudaFree(b->d_msrc);
  cudaFree(b->d_moff);
  if (b->h_errs) cudaFreeHost(b->h_errs);
  cudaFreeHost(b->h_msrc);
  cudaFreeHost(b->h_moff);
  b->d_msrc = b->h_msrc = nullptr;
  b->d_moff = b->h_moff = nullptr;
  b->member_cap = 0;
  GRUS_CUDA_TRY(cudaMalloc(&b->d_msrc, n * 4));
  GRUS_CUDA_TRY(cudaMalloc(&b->d_moff, n * 8));
  GRUS_CUDA_TRY(cudaMallocHost(&b->h_msrc, n * 4));
  GRUS_CUDA_TRY(cudaMallocHost(&b->h_moff, n * 8));
  b->member_cap = n;
  return GRUS_OK;
}

// Cost model of one task on one worker, in edge-equivalents: a traversal
// reads the edges and scans the vertex arrays; each extra source of a
// multi-source task adds about a third of a single traversal (measured on
// RMAT graphs: 8 sources cost 3.25 single queries on a 16-CTA worker).
static double task_cost(const grus_graph *g, int k) {
  return ((double)g->m + 16.0 * (double)g->n) * (1.0 + 0.32 * (k - 1));
}

// Plans the run: SSSP queries on the same graph are packed into
// multi-source tasks of up to `group` queries, but a pack never costs more
// than the larger of the most expensive single query and the batch's even
// share per worker, so packing lowers the total work without lengthening the
// critical path (the largest graphs keep one query per worker).  Tasks are
// ordered by descending graph size so large work starts first.
static int stage_tasks(grus_batch *b, const grus_query *q, int nq) {
  std::vector<int> order(nq);
  for (int i = 0; i < nq; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    const uint64_t mx = b->graphs[q[x].graph]->m, my = b->graphs[q[y].graph]->m;
    if (mx != my) return mx > my;
    if (q[x].graph != q[y].graph) return q[x].graph < q[y].graph;
    return q[x].algo < q[y].algo;
  });
  struct Plan {
    Task t;
    int first, k;  // members (multi-source) or -1
  };
  std::vector<Plan> plan;
  std::vector<int> members;
  uint32_t max_k = 0;
  double total = 0.0, top = 0.0;
  for (int i = 0; i < nq; ++i) {
    const double c = task_cost(b->graphs[q[i].graph], 1);
    total += c;
    top = std::max(top, c);
  }
  const double target = std::max(top, total / std::max(b->workers, 1));
  for (int i = 0; i < nq;) {
    const grus_query &s0 = q[order[i]];
    const grus_graph *g0 = b->graphs[s0.graph];
    int j = i + 1;
    if (b->group > 1 && s0.algo == GRUS_ALGO_SSSP)
      while (j < nq && j - i < (int)b->group && q[order[j]].graph == s0.graph &&
             q[order[j]].algo == GRUS_ALGO_SSSP && task_cost(g0, j - i + 1) <= target)
        ++j;
    Plan p;
    p.t.graph = s0.graph;
    p.t.pad = 0;
    p.t.out_off = s0.out_offset;
    if (j - i >= 2) {
      p.t.algo = kAlgoSsspMulti;
      p.first = (int)members.size();
      p.k = j - i;
      p.t.src = (uint32_t)p.first;
      p.t.pad = (uint32_t)p.k;
      for (int x = i; x < j; ++x) members.push_back(order[x]);
      max_k = std::max<uint32_t>(max_k, (uint32_t)p.k);
    } else {
      j = i + 1;
      p.t.algo = s0.algo;
      p.t.src = s0.src;
      p.first = -1;
      p.k = 0;
    }
    plan.push_back(p);
    i = j;
  }
  int rc = ensure_tasks(b, (uint32_t)plan.size());
  if (rc) return rc;
  if (!members.empty()) {
    rc = ensure_members(b, (uint32_t)members.size());
    if (rc) return rc;
    const uint32_t ks = max_k <= 8 ? 8u : (max_k <= 16 ? 16u : 32u);
    const uint32_t *before = b->state.ms_d;
    rc = b->state.reserve_multi(b->workers, b->max_n, b->max_m, ks);
    if (rc) return rc;
    if (b->state.ms_d != before) drop_graph(b);  // a captured launch holds the old state
  }
  for (size_t i = 0; i < plan.size(); ++i) b->h_tasks[i] = plan[i].t;
  for (size_t i = 0; i < members.size(); ++i) {
    b->h_msrc[i] = q[members[i]].src;
    b->h_moff[i] = q[members[i]].out_offset;
  }
  b->ntasks = (uint32_t)plan.size();
  b->nmembers = (uint32_t)members.size();
  return GRUS_OK;
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
  // the pinned staging buffers are read by the previous run's copies: wait
  if (b->in_flight) GRUS_CUDA_TRY(cudaEventSynchronize(b->done));
  std::vector<grus_query> small_q;
  std::vector<int> big_q;
  small_q.reserve(nq);
  for (int i = 0; i < nq; ++i) {
    if (b->big[queries[i].graph]) big_q.push_back(i);
    else small_q.push_back(queries[i]);
  }
  int rc = GRUS_OK;
  if (!small_q.empty()) {
    rc = stage_tasks(b, small_q.data(), (int)small_q.size());
    if (rc) return rc;
  } else {
    b->ntasks = b->nmembers = 0;
  }
  const uint32_t nt = b->ntasks, nm = b->nmembers;
  const uint32_t *msrc = nm ? b->d_msrc : nullptr;
  const unsigned long long *moff = nm ? b->d_moff : nullptr;
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(b->ev0, s));
  // queries on big graphs: whole-GPU launches queued first on the stream
  uint32_t nerr = 0;
  uint32_t nlaunch = 0;  // kernels launched by the big-graph lane
  if (!big_q.empty()) {
    if (b->err_cap < big_q.size()) {
      if (b->h_errs) cudaFreeHost(b->h_errs);
      b->h_errs = nullptr;
      b->err_cap = 0;
      GRUS_CUDA_TRY(cudaMallocHost(&b->h_errs, big_q.size() * 4));
      b->err_cap = (uint32_t)big_q.size();
    }
    std::stable_sort(big_q.begin(), big_q.end(), [&](int x, int y) {
      if (queries[x].graph != queries[y].graph) return queries[x].graph < queries[y].graph;
      return queries[x].algo < queries[y].algo;
    });
    rc = union_sssp(b, queries, big_q, out, s, &nerr, &nlaunch);
    if (rc) return rc;
    for (size_t i = 0; i < big_q.size();) {
      const grus_query &q0 = queries[big_q[i]];
      if (q0.algo == GRUS_ALGO_SSSP) {  // launched by union_sssp
        ++i;
        continue;
      }
      grus_graph *g = b->graphs[q0.graph];
      size_t j = i + 1;
      const size_t cap = q0.algo == GRUS_ALGO_SSSP ? 32 : 64;
      while (j < big_q.size() && j - i < cap && queries[big_q[j]].graph == q0.graph &&
             queries[big_q[j]].algo == q0.algo)
        ++j;
      // BFS queries of a graph run alone unless enough share the graph
      if (q0.algo != GRUS_ALGO_SSSP && j - i < bfs_pack_min(g->m)) j = i + 1;
      CtrlView cv;
      if (j - i == 1) {
        rc = q0.algo == GRUS_ALGO_SSSP ? grus_sssp(g, q0.src, out + q0.out_offset, nullptr, s)
                                       : grus_bfs(g, q0.src, out + q0.out_offset, nullptr, s);
        // a single BFS is the persistent kernel and its narrow-tail kernel
        nlaunch += q0.algo == GRUS_ALGO_SSSP ? 1 : 2;
        cv = q0.algo == GRUS_ALGO_SSSP ? sssp_ctrl(g) : bfs_ctrl(g);
      } else {
        uint32_t srcs[64];
        uint32_t *outs[64];
        for (size_t k = i; k < j; ++k) {
          srcs[k - i] = queries[big_q[k]].src;
          outs[k - i] = out + queries[big_q[k]].out_offset;
        }
        ++nlaunch;
        if (q0.algo == GRUS_ALGO_SSSP) {
          rc = msssp_run(g, srcs, (int)(j - i), outs, nullptr, s);
          cv = msssp_ctrl(g);
        } else {
          rc = msbfs_run(g, srcs, (int)(j - i), outs, nullptr, s);
          cv = msbfs_ctrl(g);
        }
      }
      if (rc) return rc;
      if (cv.ctrl) {
        GRUS_CUDA_TRY(cudaMemcpyAsync(b->h_errs + nerr, cv.ctrl + cv.err_off, 4,
                                      cudaMemcpyDeviceToHost, s));
        GRUS_CUDA_TRY(cudaMemsetAsync(cv.ctrl + cv.err_off, 0, 4, s));
        ++nerr;
      }
      i = j;
    }
  }
  if (nt == 0) {
    // every query was on a big graph
    if (stats) GRUS_CUDA_TRY(cudaEventRecord(b->ev1, s));
    GRUS_CUDA_TRY(cudaEventRecord(b->done, s));
    b->in_flight = true;
    if (!stats) return GRUS_OK;
    GRUS_CUDA_TRY(cudaStreamSynchronize(s));
    uint32_t bits = 0;
    for (uint32_t i = 0; i < nerr; ++i) bits |= b->h_errs[i];
    if (bits) {
      msssp_union_reset(b->uws);
      return status_from_device_error(bits);
    }
    std::memset(stats, 0, sizeof(*stats));
    stats->kernel_launches = nlaunch;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    stats->device_ms = ms;
    return GRUS_OK;
  }
  if (use_graph) {
    // one captured graph per (task count, output buffer): H2D copy of the
    // staged tasks, counter reset, batch kernel
    if (b->exec && (b->graph_ntasks != nt || b->graph_nmembers != nm || b->graph_out != out ||
                    b->graph_stream != s))
      drop_graph(b);
    if (!b->exec) {
      cudaStream_t cap_s = nullptr;
      GRUS_CUDA_TRY(cudaStreamCreateWithFlags(&cap_s, cudaStreamNonBlocking));
      cudaError_t e = cudaStreamBeginCapture(cap_s, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaMemcpyAsync(b->d_tasks, b->h_tasks, nt * sizeof(Task), cudaMemcpyHostToDevice, cap_s);
        if (nm) {
          cudaMemcpyAsync(b->d_msrc, b->h_msrc, nm * 4, cudaMemcpyHostToDevice, cap_s);
          cudaMemcpyAsync(b->d_moff, b->h_moff, nm * 8, cudaMemcpyHostToDevice, cap_s);
        }
        cudaMemsetAsync(b->state.counter, 0, 4, cap_s);
        rc = batch_launch(b->state, 0, b->workers, b->cluster, b->d_graphs, b->d_tasks, nt, out,
                          b->huge, b->delta, b->state.counter, cap_s, msrc, moff);
        e = cudaStreamEndCapture(cap_s, &b->graph);
      }
      cudaStreamDestroy(cap_s);
      if (rc) return rc;
      GRUS_CUDA_TRY(e);
      GRUS_CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
      b->graph_ntasks = nt;
      b->graph_nmembers = nm;
      b->graph_out = out;
      b->graph_stream = s;
    }
    GRUS_CUDA_TRY(cudaGraphLaunch(b->exec, s));
  } else {
    GRUS_CUDA_TRY(cudaMemcpyAsync(b->d_tasks, b->h_tasks, nt * sizeof(Task), cudaMemcpyHostToDevice, s));
    if (nm) {
      GRUS_CUDA_TRY(cudaMemcpyAsync(b->d_msrc, b->h_msrc, nm * 4, cudaMemcpyHostToDevice, s));
      GRUS_CUDA_TRY(cudaMemcpyAsync(b->d_moff, b->h_moff, nm * 8, cudaMemcpyHostToDevice, s));
    }
    GRUS_CUDA_TRY(cudaMemsetAsync(b->state.counter, 0, 4, s));
    rc = batch_launch(b->state, 0, b->workers, b->cluster, b->d_graphs, b->d_tasks, nt, out, b->huge,
                      b->delta, b->state.counter, s, msrc, moff);
    if (rc) return rc;
  }
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(b->ev1, s));
  GRUS_CUDA_TRY(cudaEventRecord(b->done, s));
  b->in_flight = true;
  if (!stats) return GRUS_OK;
  uint32_t err = 0;
  GRUS_CUDA_TRY(cudaMemcpyAsync(&err, b->state.err, 4, cudaMemcpyDeviceToHost, s));
  GRUS_CUDA_TRY(cudaStreamSynchronize(s));
  for (uint32_t i = 0; i < nerr; ++i) err |= b->h_errs[i];
  if (err) {
    cudaMemset(b->state.err, 0, 4);
    msssp_union_reset(b->uws);
    return status_from_device_error(err);
  }
  std::memset(stats, 0, sizeof(*stats));
  stats->kernel_launches = 1 + nlaunch;
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
  info->group_sources = b->group;
  info->big_edges = b->big_edges >= 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)b->big_edges;
  info->launch_entries = (uint32_t)b->launch_entries;
  return GRUS_OK;
}

int grus_batch_free(grus_batch *b) {
  if (!b) return GRUS_EINVAL;
  cudaDeviceSynchronize();
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->state.release();
  grus::msssp_union_free(b->uws);
  cudaFree(b->d_graphs);
  cudaFree(b->d_tasks);
  if (b->h_tasks) cudaFreeHost(b->h_tasks);
  cudaFree(b->d_msrc);
  cudaFree(b->d_moff);
  if (b->h_errs) cudaFreeHost(b->h_errs);
  if (b->h_msrc) cudaFreeHost(b->h_msrc);
  if (b->h_moff) cudaFreeHost(b->h_moff);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->done) cudaEventDestroy(b->done);
  delete b;
  return GRUS_OK;
}

}  // extern "C"
