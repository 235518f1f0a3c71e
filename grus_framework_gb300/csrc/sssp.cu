// sssp.cu -- exact single-source shortest paths over uint32 weights as one
// persistent launch (near/far label correcting, a Delta-stepping variant:
// Meyer & Sanders 2003; GPU near-far piles: Davidson et al. 2014).
//
// Replaces the reference's SSSP_single_gpu loop (samples/sssp/sssp.cu:123-170)
// over kernel<...,Frontier<BDF>> whose updater relaxes with a NON-atomic
// read-modify-write (sssp.cu:51-60) and can keep a larger distance when two
// sources race.  Here every relaxation is atomicMin, so the result is the
// unique fixpoint -- Dijkstra's distances -- whatever the schedule.
//
// The near and far sets are bitmaps (one bit per vertex):
//   N[L & 1]  vertices to expand at level L (improved below the threshold T)
//   N[~L & 1] vertices improved below T during level L
//   F         vertices improved to a distance >= T (far)
// A level
//   1. compacts N[L & 1] into binned work lists (degree < huge: vertex queue;
//      degree >= huge: 1024-edge chunks), clearing the bitmap as it reads it,
//      with one queue reservation per CTA (block scan of the counts);
//   2. expands the lists with the degree-binned mappings of expand.cuh; a
//      relaxation that beats the distance it read lowers it with a
//      non-returning atomicMin and sets v's bit in N[~L & 1] (new distance < T)
//      or F -- also a reduction, so the relaxation path waits on no atomic.
// When a level finds nothing to expand, T advances by Delta (or jumps to the
// bucket of the smallest far distance) and F is scanned: vertices below the
// old T were expanded as near since and are dropped, vertices below the new T
// move to N[L & 1], the rest stay.  Every wait is a bounded grid barrier.
#include <algorithm>
#include <cstring>

#include "expand.cuh"
#include "grus_internal.cuh"

namespace grus {
namespace {

constexpr int kBlock = 256;
constexpr uint32_t kDefHuge = 1024;
constexpr uint32_t kDefDelta = 640;

struct Slot {
  uint32_t qcount, ccount;
  unsigned long long visits;  // edge relaxations attempted in the level
  uint32_t pad[4];
};

// Far-set control.  minfar is double-buffered by split parity so that the
// value every CTA reads at the start of split k (written during split k-1) is
// never the one being reset or reduced during split k.
struct FarCtl {
  uint32_t moved, remaining;  // of the current split
  uint32_t minfar[2];
};

struct Summary {
  uint32_t levels, splits, pad0, pad1;
  unsigned long long visits, nr, mr;
};

// Per-level record: end time, relaxations, frontier size (queue entries +
// hub chunks) and the number of threshold advances so far.
constexpr int kMaxTrace = 256;
struct LevelTrace {
  unsigned long long t_ns, visits;
  uint32_t frontier, splits;
};

struct Args {
  const uint32_t *__restrict__ offs;
  const uint32_t *__restrict__ cols;
  const uint32_t *__restrict__ wts;
  uint32_t n, W;
  uint32_t src;
  uint32_t *dist;
  uint32_t *near[2];      // W words each
  uint32_t *farbm;        // W words
  uint32_t *queue;        // this level's vertex queue
  uint4 *chunks;          // this level's hub chunks
  uint32_t queue_cap, chunk_cap;
  Slot *slots;
  FarCtl *farctl;
  GridBarrier *bar;
  uint32_t *err;
  Summary *summary;
  LevelTrace *trace;
  uint32_t delta, huge;
  uint64_t timeout_ns;
};

struct Workspace {
  uint32_t W = 0;
  uint32_t *dist = nullptr;
  uint32_t *bitmaps = nullptr;  // 3 * Wp words: near[2], farbm
  size_t bitmap_bytes = 0;
  uint32_t *queues = nullptr;   // n
  uint4 *chunks = nullptr;
  uint32_t chunk_cap = 0;
  char *ctrl = nullptr, *ctrl_host = nullptr;
  LevelTrace *trace = nullptr, *trace_host = nullptr;
  int trace_levels = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

constexpr size_t kOffSlots = 0, kOffFar = 256, kOffBar = 384, kOffErr = 640,
                 kOffSummary = 704, kCtrlBytes = 768;
static_assert(kOffBar % 128 == 0 && kOffBar + sizeof(GridBarrier) <= kOffErr, "barrier layout");
static_assert(4 * sizeof(Slot) <= kOffFar && sizeof(FarCtl) <= kOffBar - kOffFar &&
                  sizeof(Summary) <= kCtrlBytes - kOffSummary,
              "control block layout");

void ws_free(void *p) {
  Workspace *w = (Workspace *)p;
  if (!w) return;
  cudaFree(w->dist);
  cudaFree(w->bitmaps);
  cudaFree(w->queues);
  cudaFree(w->chunks);
  cudaFree(w->ctrl);
  cudaFree(w->trace);
  if (w->ctrl_host) cudaFreeHost(w->ctrl_host);
  if (w->trace_host) cudaFreeHost(w->trace_host);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  delete w;
}

int ws_get(grus_graph *g, Workspace **out) {
  if (g->ws[kWsSssp]) {
    *out = (Workspace *)g->ws[kWsSssp];
    return GRUS_OK;
  }
  Workspace *w = new Workspace();
  w->W = (uint32_t)((g->n + 31) / 32);
  const uint64_t Wp = ((uint64_t)w->W + 31) / 32 * 32;
  w->bitmap_bytes = 3 * Wp * 4;
  // chunk lists sized for any chunking degree down to 256 (the autotuner and
  // callers may lower it after the workspace exists)
  const uint32_t huge = std::min(tune_or(g->tuning.huge_degree, kDefHuge), 256u);
  w->chunk_cap = (uint32_t)std::min<uint64_t>(g->m / kChunk + g->m / huge + 2, 0x7FFFFFFFull);
  const uint64_t n1 = std::max<uint64_t>(g->n, 1);
  cudaError_t e = cudaMalloc(&w->bitmaps, w->bitmap_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&w->queues, n1 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&w->chunks, (uint64_t)w->chunk_cap * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&w->ctrl, kCtrlBytes);
  if (e == cudaSuccess) e = cudaMemset(w->ctrl, 0, kCtrlBytes);
  if (e == cudaSuccess) e = cudaMallocHost(&w->ctrl_host, kCtrlBytes);
  if (e == cudaSuccess) e = cudaMalloc(&w->trace, kMaxTrace * sizeof(LevelTrace));
  if (e == cudaSuccess) e = cudaMallocHost(&w->trace_host, kMaxTrace * sizeof(LevelTrace));
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ws_free(w);
    set_last_error(std::string("sssp workspace: ") + cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  g->ws[kWsSssp] = w;
  g->ws_free[kWsSssp] = ws_free;
  *out = w;
  return GRUS_OK;
}

struct RelaxVisitor {
  const Args *a;
  uint32_t T;
  uint32_t *nnext;
  unsigned long long visits;

  using aux_t = uint32_t;

  __device__ __forceinline__ uint32_t aux(uint32_t v) const { return __ldcg(a->dist + v); }
  // A reduction lowers dist(v) and another marks v; neither is waited for.
  // If another thread lowered dist(v) further meanwhile, v is marked all the
  // same (a bit), costing at most one redundant expansion.
  __device__ __forceinline__ void edge(uint32_t, uint32_t du, uint32_t x) {
    ++visits;
    const uint32_t v = __ldg(a->cols + x);
    const uint32_t nd = du + __ldg(a->wts + x);
    if (nd >= __ldcg(a->dist + v)) return;
    atomicMin(a->dist + v, nd);
    atomicOr((nd < T ? nnext : a->farbm) + (v >> 5), 1u << (v & 31u));
  }
};

__global__ void __launch_bounds__(kBlock) sssp_persistent(Args a) {
  const uint32_t gtid = blockIdx.x * kBlock + threadIdx.x;
  const uint32_t nthreads = gridDim.x * kBlock;
  // prologue: distances to INFINIT, bitmaps and control words to zero
  for (uint32_t i = gtid; i < a.n; i += nthreads) a.dist[i] = kInfinit;
  for (uint32_t i = gtid; i < a.W; i += nthreads) {
    a.near[0][i] = 0u;
    a.near[1][i] = 0u;
    a.farbm[i] = 0u;
  }
  if (gtid < 4 * sizeof(Slot) / 4) ((uint32_t *)a.slots)[gtid] = 0u;
  if (gtid < sizeof(FarCtl) / 4) ((uint32_t *)a.farctl)[gtid] = 0u;
  if (gtid == 0) {
    a.farctl->minfar[0] = 0xFFFFFFFFu;
    a.farctl->minfar[1] = 0xFFFFFFFFu;
  }
  if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
  if (gtid == 0) {
    a.dist[a.src] = 0;
    a.near[0][a.src >> 5] = 1u << (a.src & 31u);
  }
  if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;

  uint32_t L = 0, T = a.delta, splits = 0;
  unsigned long long visits = 0;
  if (gtid == 0 && a.trace) a.trace[0] = LevelTrace{global_timer_ns(), 0ull, 1u, 0u};
  while (true) {
    Slot *sl = a.slots + (L & 3u);
    if (gtid < sizeof(Slot) / 4) ((uint32_t *)(a.slots + ((L + 2) & 3u)))[gtid] = 0u;
    uint32_t *ncur = a.near[L & 1u], *nnext = a.near[(L + 1) & 1u];
    bitmap_to_binned<kBlock>(ncur, a.W, a.offs, a.huge, a.queue, &sl->qcount, a.queue_cap,
                             a.chunks, &sl->ccount, a.chunk_cap, a.err, blockIdx.x, gridDim.x);
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    const uint32_t qc = min(__ldcg(&sl->qcount), a.queue_cap);
    const uint32_t cc = min(__ldcg(&sl->ccount), a.chunk_cap);
    if (qc + cc == 0) {
      // nothing near: advance the threshold and split the far set into ncur
      const uint32_t Told = T;
      uint32_t Tnew = T + a.delta;
      const uint32_t mf = __ldcg(&a.farctl->minfar[splits & 1u]);
      if (mf != 0xFFFFFFFFu && mf >= Tnew) Tnew = (mf / a.delta + 1) * a.delta;
      uint32_t moved = 0, remaining = 0, local_min = 0xFFFFFFFFu;
      for (uint32_t w = gtid; w < a.W; w += nthreads) {
        const uint32_t fw = __ldcg(a.farbm + w);
        if (!fw) continue;
        uint32_t keep = 0, mv = 0;
        for (uint32_t bits = fw; bits; bits &= bits - 1) {
          const uint32_t b = __ffs(bits) - 1;
          const uint32_t d = __ldcg(a.dist + w * 32 + b);
          if (d < Told) continue;  // improved below T since: expanded as near
          if (d < Tnew) {
            mv |= 1u << b;
          } else {
            keep |= 1u << b;
            local_min = min(local_min, d);
          }
        }
        a.farbm[w] = keep;
        if (mv) ncur[w] = mv;  // ncur is all zero after its compaction
        moved += __popc(mv);
        remaining += keep != 0;
      }
      for (int o = 16; o > 0; o >>= 1) {
        local_min = min(local_min, __shfl_down_sync(0xffffffffu, local_min, o));
        moved += __shfl_down_sync(0xffffffffu, moved, o);
        remaining += __shfl_down_sync(0xffffffffu, remaining, o);
      }
      if (lane_id() == 0) {
        if (local_min != 0xFFFFFFFFu) atomicMin(&a.farctl->minfar[(splits + 1) & 1u], local_min);
        if (moved) atomicAdd(&a.farctl->moved, moved);
        if (remaining) atomicAdd(&a.farctl->remaining, remaining);
      }
      if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
      const uint32_t mv_all = __ldcg(&a.farctl->moved), rem_all = __ldcg(&a.farctl->remaining);
      if (gtid == 0) a.farctl->minfar[splits & 1u] = 0xFFFFFFFFu;  // read by all before the barrier
      T = Tnew;
      ++splits;
      // every CTA has read the counters before they are cleared; the next
      // split adds to them only after the next compaction's barrier
      if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
      if (gtid == 0) {
        a.farctl->moved = 0u;
        a.farctl->remaining = 0u;
      }
      if (mv_all == 0 && rem_all == 0) break;  // nothing near, nothing far: done
      continue;  // compact the moved vertices (or split again)
    }
    RelaxVisitor vis{&a, T, nnext, 0ull};
    expand_binned<kBlock>(a.offs, a.queue, qc, a.chunks, cc, vis);
    const unsigned long long bv = block_sum_u64<kBlock>(vis.visits);
    if (threadIdx.x == 0 && bv) atomicAdd(&sl->visits, bv);
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    const unsigned long long lv = __ldcg(&sl->visits);
    visits += lv;
    ++L;
    if (gtid == 0 && a.trace && L < (uint32_t)kMaxTrace)
      a.trace[L] = LevelTrace{global_timer_ns(), lv, qc + cc, splits};
    if (L > 4u * a.n + 64u) {
      if (gtid == 0) atomicOr(a.err, kErrLevels);
      break;
    }
  }
  // epilogue: reached vertices and their out-degree sum (m_r)
  unsigned long long nr = 0, mr = 0;
  for (uint32_t v = gtid; v < a.n; v += nthreads)
    if (__ldcg(a.dist + v) != kInfinit) {
      ++nr;
      mr += __ldg(a.offs + v + 1) - __ldg(a.offs + v);
    }
  const unsigned long long bnr = block_sum_u64<kBlock>(nr);
  const unsigned long long bmr = block_sum_u64<kBlock>(mr);
  if (threadIdx.x == 0) {
    atomicAdd(&a.summary->nr, bnr);
    atomicAdd(&a.summary->mr, bmr);
  }
  if (gtid == 0) {
    a.summary->levels = L;
    a.summary->splits = splits;
    a.summary->visits = visits;
  }
}

}  // namespace
}  // namespace grus

using namespace grus;

extern "C" int grus_sssp(grus_graph *g, uint32_t src, uint32_t *dist,
                         grus_stats *stats, void *stream) {
  if (!g || !dist) return GRUS_EINVAL;
  if (g->n == 0 || src >= g->n) {
    set_last_error("source vertex out of range");
    return GRUS_EINVAL;
  }
  if (!g->csr.wts) {
    set_last_error("sssp needs edge weights (load with need_weights or generate weighted)");
    return GRUS_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g->mu);
  Workspace *w = nullptr;
  int rc = ws_get(g, &w);
  if (rc) return rc;
  const bool dev_out = is_device_pointer(dist);
  if (!dev_out && !w->dist) GRUS_CUDA_TRY(cudaMalloc(&w->dist, g->n * 4));
  static int occ = -1;
  if (occ < 0)
    GRUS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sssp_persistent, kBlock, 0));

  Args a;
  std::memset(&a, 0, sizeof(a));
  a.offs = g->csr.offs;
  a.cols = g->csr.cols;
  a.wts = g->csr.wts;
  a.n = (uint32_t)g->n;
  a.W = w->W;
  a.src = src;
  a.dist = dev_out ? dist : w->dist;
  const uint64_t Wp = ((uint64_t)w->W + 31) / 32 * 32;
  a.near[0] = w->bitmaps;
  a.near[1] = w->bitmaps + Wp;
  a.farbm = w->bitmaps + 2 * Wp;
  a.queue = w->queues;
  a.chunks = w->chunks;
  a.queue_cap = (uint32_t)g->n;
  a.chunk_cap = w->chunk_cap;
  a.slots = (Slot *)(w->ctrl + kOffSlots);
  a.farctl = (FarCtl *)(w->ctrl + kOffFar);
  a.bar = (GridBarrier *)(w->ctrl + kOffBar);
  a.err = (uint32_t *)(w->ctrl + kOffErr);
  a.summary = (Summary *)(w->ctrl + kOffSummary);
  a.trace = stats ? w->trace : nullptr;
  a.delta = std::max(1u, tune_or(g->tuning.sssp_delta, kDefDelta));
  a.huge = tune_or(g->tuning.huge_degree, kDefHuge);
  a.timeout_ns = (uint64_t)tune_or(g->tuning.timeout_ms, 30000u) * 1000000ull;

  const bool sync = stats != nullptr || !dev_out;
  // barrier, error word and summary: a timed-out launch leaves stale barrier state
  GRUS_CUDA_TRY(cudaMemsetAsync(w->ctrl + kOffBar, 0, kCtrlBytes - kOffBar, s));
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(w->ev0, s));
  void *args[] = {&a};
  // the L2 window on the distances, which every relaxation reads and lowers
  // with an atomic: RMAT-22 1.99 -> 1.80-1.83 ms against the window on the
  // near/far bitmaps (small and hot enough to stay in L2 without it)
  rc = launch_persistent((const void *)sssp_persistent, args, kBlock,
                         (int)g->tuning.ctas_per_sm, occ, s, a.dist, (size_t)g->n * 4);
  if (rc) return rc;
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(w->ev1, s));
  if (!dev_out) GRUS_CUDA_TRY(cudaMemcpyAsync(dist, w->dist, g->n * 4, cudaMemcpyDeviceToHost, s));
  if (!sync) return GRUS_OK;
  GRUS_CUDA_TRY(cudaMemcpyAsync(w->ctrl_host, w->ctrl, kCtrlBytes, cudaMemcpyDeviceToHost, s));
  GRUS_CUDA_TRY(cudaStreamSynchronize(s));
  const uint32_t errbits = *(uint32_t *)(w->ctrl_host + kOffErr);
  if (errbits) {
    cudaMemsetAsync(w->ctrl, 0, kCtrlBytes, s);
    cudaStreamSynchronize(s);
    return status_from_device_error(errbits);
  }
  if (stats) {
    const Summary *sm = (const Summary *)(w->ctrl_host + kOffSummary);
    GRUS_CUDA_TRY(cudaMemcpy(w->trace_host, w->trace, kMaxTrace * sizeof(LevelTrace),
                             cudaMemcpyDeviceToHost));
    w->trace_levels = std::min<int>((int)sm->levels + 1, kMaxTrace);
    std::memset(stats, 0, sizeof(*stats));
    stats->levels = sm->levels;
    stats->direction_switches = sm->splits;  // threshold advances
    stats->kernel_launches = 1;
    stats->vertices_reached = sm->nr;
    stats->edges_reached = sm->mr;
    stats->edges_relaxed = sm->visits;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, w->ev0, w->ev1);
    stats->device_ms = ms;
  }
  return GRUS_OK;
}

extern "C" int grus_sssp_trace(grus_graph *g, grus_level_trace *out, int max_levels) {
  if (!g || (!out && max_levels > 0) || max_levels < 0) return GRUS_EINVAL;
  std::lock_guard<std::mutex> lk(g->mu);
  const Workspace *w = (const Workspace *)g->ws[kWsSssp];
  if (!w || w->trace_levels < 2) return 0;
  const int levels = std::min(w->trace_levels - 1, max_levels);
  const uint64_t t0 = w->trace_host[0].t_ns;
  for (int i = 0; i < levels; ++i) {
    const LevelTrace &r = w->trace_host[i + 1];
    out[i].end_ns = r.t_ns - t0;
    out[i].edges = r.visits;
    out[i].vertices = r.frontier;
    out[i].pull = r.splits;
  }
  return levels;
}

namespace grus {
CtrlView sssp_ctrl(grus_graph *g) {
  CtrlView v;
  std::lock_guard<std::mutex> lk(g->mu);
  const Workspace *w = (const Workspace *)g->ws[kWsSssp];
  if (w) {
    v.ctrl = w->ctrl;
    v.bytes = kCtrlBytes;
    v.err_off = kOffErr;
    v.bar_off = kOffBar;
  }
  return v;
}
}  // namespace grus
