// msssp.cu -- multi-source SSSP: up to 32 sources in ONE persistent launch
// over the whole GPU (the level loop is msssp_core.cuh; levels are separated
// by the bounded grid barrier).
//
// The reference runs one SSSP per process invocation
// (samples/sssp/sssp.cu:123-170); 32 queries on one graph cost 32 launches of
// its level loop, each re-reading the adjacency lists.  Here the sources
// advance together and share every adjacency read, and the outputs are
// bit-exact against single-source runs.
#include <algorithm>
#include <cstring>

#include "device_util.cuh"
#include "grus_internal.cuh"
#include "msssp_core.cuh"

namespace grus {
namespace {

constexpr int kBlock = 256;
constexpr uint32_t kDefDelta = 1024;
constexpr int kMaxSources = 32;
using ms::kPiece;
using ms::Slot;

struct Summary {
  uint32_t levels, splits, pad0, pad1;
  unsigned long long visits, nr, mr;
};

struct Args {
  ms::View v;
  uint32_t *out[kMaxSources];
  GridBarrier *bar;
  Summary *summary;
  uint64_t timeout_ns;
};

struct GridSync {
  GridBarrier *bar;
  uint32_t *err;
  uint64_t timeout_ns;
  __device__ __forceinline__ bool operator()() const { return grid_sync(bar, err, timeout_ns); }
};

struct OutTable {
  uint32_t *const *out;
  __device__ __forceinline__ uint32_t *operator()(uint32_t s) const { return out[s]; }
};

template <int KS>
__global__ void __launch_bounds__(kBlock, 8) msssp_persistent(Args a) {
  const uint32_t gtid = blockIdx.x * kBlock + threadIdx.x;
  const uint32_t nthreads = gridDim.x * kBlock;
  GridSync sync{a.bar, a.v.err, a.timeout_ns};
  OutTable out{a.out};
  ms::Result r;
  if (!ms::run<KS, kBlock>(a.v, gtid, nthreads, sync, out, r)) return;
  const unsigned long long bnr = block_sum_u64<kBlock>(r.nr);
  const unsigned long long bmr = block_sum_u64<kBlock>(r.mr);
  if (threadIdx.x == 0) {
    atomicAdd(&a.summary->nr, bnr);
    atomicAdd(&a.summary->mr, bmr);
  }
  if (gtid == 0) {
    a.summary->levels = r.levels;
    a.summary->splits = r.splits;
    a.summary->visits = r.visits;
  }
}

// Multi-graph launch: the same level loop over several graphs at once
// (msssp_core.cuh, kUnion); the vertex bases go to shared memory for the
// graph lookups.
struct UnionArgs {
  ms::View v;
  GridBarrier *bar;
  Summary *summary;
  uint64_t timeout_ns;
};

struct NoOut {
  __device__ __forceinline__ uint32_t *operator()(uint32_t) const { return nullptr; }
};

template <int KS>
__global__ void __launch_bounds__(kBlock, 8) msssp_union(UnionArgs a) {
  __shared__ uint32_t s_vb[ms::kMaxUnion + 1];
  for (uint32_t i = threadIdx.x; i <= a.v.ngraphs; i += kBlock)
    s_vb[i] = i < a.v.ngraphs ? a.v.ug[i].vbase : a.v.n;
  __syncthreads();
  const uint32_t gtid = blockIdx.x * kBlock + threadIdx.x;
  const uint32_t nthreads = gridDim.x * kBlock;
  GridSync sync{a.bar, a.v.err, a.timeout_ns};
  ms::Result r;
  if (!ms::run<KS, kBlock, true>(a.v, gtid, nthreads, sync, NoOut{}, r, s_vb)) return;
  const unsigned long long bnr = block_sum_u64<kBlock>(r.nr);
  const unsigned long long bmr = block_sum_u64<kBlock>(r.mr);
  if (threadIdx.x == 0) {
    atomicAdd(&a.summary->nr, bnr);
    atomicAdd(&a.summary->mr, bmr);
  }
  if (gtid == 0) {
    a.summary->levels = r.levels;
    a.summary->splits = r.splits;
    a.summary->visits = r.visits;
  }
}

struct Workspace {
  uint32_t ks = 0;             // row width the distance matrix was sized for
  uint32_t *D = nullptr;       // n * ks
  uint32_t *masks = nullptr;   // 3n: F[0], F[1], far
  uint4 *ent = nullptr;
  uint32_t ent_cap = 0;
  uint32_t *srcs = nullptr;
  char *ctrl = nullptr, *ctrl_host = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

constexpr size_t kOffSlots = 0, kOffFar = 256, kOffBar = 384, kOffErr = 640, kOffSummary = 704,
                 kCtrlBytes = 768;
static_assert(kOffBar % 128 == 0 && kOffBar + sizeof(GridBarrier) <= kOffErr, "barrier layout");
static_assert(4 * sizeof(Slot) <= kOffFar, "slots overlap the far control");
static_assert(sizeof(Summary) <= kCtrlBytes - kOffSummary, "summary overflows the control block");

void ws_free(void *p) {
  Workspace *w = (Workspace *)p;
  if (!w) return;
  cudaFree(w->D);
  cudaFree(w->masks);
  cudaFree(w->ent);
  cudaFree(w->srcs);
  cudaFree(w->ctrl);
  if (w->ctrl_host) cudaFreeHost(w->ctrl_host);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  delete w;
}

int ws_get(grus_graph *g, uint32_t ks, Workspace **out) {
  Workspace *w = (Workspace *)g->ws[kWsMsSssp];
  if (w && w->ks >= ks) {
    *out = w;
    return GRUS_OK;
  }
  if (w) {
    ws_free(w);
    g->ws[kWsMsSssp] = nullptr;
  }
  w = new Workspace();
  w->ks = ks;
  const uint64_t n1 = std::max<uint64_t>(g->n, 1);
  w->ent_cap = (uint32_t)std::min<uint64_t>(n1 + g->m / kPiece + 1024, 0xFFFFFFF0ull);
  cudaError_t e = cudaMalloc(&w->D, n1 * ks * 4);
  if (e == cudaSuccess) e = cudaMalloc(&w->masks, 3 * n1 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&w->ent, (size_t)w->ent_cap * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&w->srcs, kMaxSources * 4);
  if (e == cudaSuccess) e = cudaMalloc(&w->ctrl, kCtrlBytes);
  if (e == cudaSuccess) e = cudaMemset(w->ctrl, 0, kCtrlBytes);
  if (e == cudaSuccess) e = cudaMallocHost(&w->ctrl_host, kCtrlBytes);
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ws_free(w);
    set_last_error(std::string("multi-source sssp workspace: ") + cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  g->ws[kWsMsSssp] = w;
  g->ws_free[kWsMsSssp] = ws_free;
  *out = w;
  return GRUS_OK;
}

template <int KS>
int launch_ks(grus_graph *g, Workspace *w, Args &a, cudaStream_t s) {
  static int occ = -1;
  if (occ < 0)
    GRUS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msssp_persistent<KS>, kBlock, 0));
  void *args[] = {&a};
  return launch_persistent((const void *)msssp_persistent<KS>, args, kBlock,
                           (int)g->tuning.ctas_per_sm, occ, s, w->masks,
                           (size_t)3 * std::max<uint64_t>(g->n, 1) * 4);
}

}  // namespace

int msssp_run(grus_graph *g, const uint32_t *hsrc, int k, uint32_t *const *outs,
              grus_stats *stats, cudaStream_t s) {
  if (!g || !hsrc || !outs || k < 1 || k > kMaxSources || g->n == 0) return GRUS_EINVAL;
  if (!g->csr.wts) {
    set_last_error("sssp needs edge weights (load with need_weights or generate weighted)");
    return GRUS_EINVAL;
  }
  for (int i = 0; i < k; ++i)
    if (hsrc[i] >= g->n || !outs[i]) {
      set_last_error("source vertex out of range");
      return GRUS_EINVAL;
    }
  const uint32_t ks = k <= 8 ? 8u : (k <= 16 ? 16u : 32u);
  std::lock_guard<std::mutex> lk(g->mu);
  Workspace *w = nullptr;
  int rc = ws_get(g, ks, &w);
  if (rc) return rc;
  GRUS_CUDA_TRY(cudaMemcpyAsync(w->srcs, hsrc, k * 4, cudaMemcpyHostToDevice, s));
  Args a;
  std::memset((void *)&a, 0, sizeof(a));
  a.v.offs = g->csr.offs;
  a.v.cols = g->csr.cols;
  a.v.wts = g->csr.wts;
  a.v.n = (uint32_t)g->n;
  a.v.k = (uint32_t)k;
  a.v.srcs = w->srcs;
  a.v.D = w->D;
  const uint64_t n1 = std::max<uint64_t>(g->n, 1);
  a.v.F[0] = w->masks;
  a.v.F[1] = w->masks + n1;
  a.v.far = w->masks + 2 * n1;
  a.v.ent = w->ent;
  a.v.ent_cap = w->ent_cap;
  a.v.slots = (Slot *)(w->ctrl + kOffSlots);
  a.v.minfar = (uint32_t *)(w->ctrl + kOffFar);
  a.v.err = (uint32_t *)(w->ctrl + kOffErr);
  a.v.delta = std::max(1u, tune_or(g->tuning.sssp_delta, kDefDelta));
  for (int i = 0; i < k; ++i) a.out[i] = outs[i];
  a.bar = (GridBarrier *)(w->ctrl + kOffBar);
  a.summary = (Summary *)(w->ctrl + kOffSummary);
  a.timeout_ns = (uint64_t)tune_or(g->tuning.timeout_ms, 30000u) * 1000000ull;
  // barrier, error word and summary: a timed-out launch leaves stale barrier state
  GRUS_CUDA_TRY(cudaMemsetAsync(w->ctrl + kOffBar, 0, kCtrlBytes - kOffBar, s));
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(w->ev0, s));
  // row width must match the kernel: a workspace sized for a wider row is
  // used at its own width
  switch (w->ks) {
    case 8: rc = launch_ks<8>(g, w, a, s); break;
    case 16: rc = launch_ks<16>(g, w, a, s); break;
    default: rc = launch_ks<32>(g, w, a, s); break;
  }
  if (rc) return rc;
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(w->ev1, s));
  if (!stats) return GRUS_OK;
  GRUS_CUDA_TRY(cudaMemcpyAsync(w->ctrl_host, w->ctrl, kCtrlBytes, cudaMemcpyDeviceToHost, s));
  GRUS_CUDA_TRY(cudaStreamSynchronize(s));
  const uint32_t errbits = *(uint32_t *)(w->ctrl_host + kOffErr);
  if (errbits) {
    cudaMemsetAsync(w->ctrl, 0, kCtrlBytes, s);
    cudaStreamSynchronize(s);
    return status_from_device_error(errbits);
  }
  const Summary *sm = (const Summary *)(w->ctrl_host + kOffSummary);
  std::memset(stats, 0, sizeof(*stats));
  stats->levels = sm->levels;
  stats->direction_switches = sm->splits;
  stats->kernel_launches = 1;
  stats->vertices_reached = sm->nr;
  stats->edges_reached = sm->mr;
  stats->edges_relaxed = sm->visits;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, w->ev0, w->ev1);
  stats->device_ms = ms;
  return GRUS_OK;
}

// ---- multi-graph launches --------------------------------------------------
// The caller (a batch) owns the workspace: distance matrix and masks sized for
// the largest launch, and per-launch regions for the graph table and the
// sources, so that several launches queued in one run never share staging.
struct UnionWs {
  uint64_t d_entries = 0;      // capacity of D in u32
  uint64_t vcap = 0;           // vertices the masks cover
  uint32_t *D = nullptr, *masks = nullptr;
  uint4 *ent = nullptr;
  uint64_t ent_cap = 0;
  int regions = 0;             // launches one run may queue
  ms::UnionGraph *ug = nullptr, *ug_host = nullptr;        // regions * kMaxUnion
  uint32_t *seeds = nullptr, *seeds_host = nullptr;        // regions * 2 * kSeedCap
  char *ctrl = nullptr;        // regions * kCtrlBytes
};

constexpr uint32_t kSeedCap = ms::kMaxUnion * kMaxSources;

void msssp_union_free(void *p) {
  UnionWs *w = (UnionWs *)p;
  if (!w) return;
  cudaFree(w->D);
  cudaFree(w->masks);
  cudaFree(w->ent);
  cudaFree(w->ug);
  cudaFree(w->seeds);
  cudaFree(w->ctrl);
  if (w->ug_host) cudaFreeHost(w->ug_host);
  if (w->seeds_host) cudaFreeHost(w->seeds_host);
  delete w;
}

// After a launch reported an error its barrier words may be left mid-count:
// clear every region's control block (the stream has been synchronised).
void msssp_union_reset(void *p) {
  UnionWs *w = (UnionWs *)p;
  if (w && w->ctrl) cudaMemset(w->ctrl, 0, (size_t)w->regions * kCtrlBytes);
}

int msssp_union_reserve(void **wsp, int regions, uint64_t max_v, uint64_t max_m, uint32_t ks) {
  UnionWs *w = (UnionWs *)*wsp;
  const uint64_t v1 = std::max<uint64_t>(max_v, 1);
  const uint64_t ecap = v1 + max_m / kPiece + 1024;
  if (ecap > 0xFFFFFFF0ull || v1 >= 0xFFFFFFFFull) {
    set_last_error("multi-graph sssp launch too large");
    return GRUS_EINVAL;
  }
  if (w && w->regions >= regions && w->vcap >= v1 && w->d_entries >= v1 * ks && w->ent_cap >= ecap)
    return GRUS_OK;
  if (w) cudaDeviceSynchronize();  // launches of an earlier run may still use it
  UnionWs *nw = new UnionWs();
  nw->regions = std::max(regions, w ? w->regions : 0);
  nw->vcap = std::max(v1, w ? w->vcap : 0);
  nw->d_entries = std::max(v1 * ks, w ? w->d_entries : 0);
  nw->ent_cap = std::max(ecap, w ? w->ent_cap : 0);
  msssp_union_free(w);
  *wsp = nullptr;
  cudaError_t e = cudaMalloc(&nw->D, nw->d_entries * 4);
  if (e == cudaSuccess) e = cudaMalloc(&nw->masks, 3 * nw->vcap * 4);
  if (e == cudaSuccess) e = cudaMalloc(&nw->ent, nw->ent_cap * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&nw->ug, (size_t)nw->regions * ms::kMaxUnion * sizeof(ms::UnionGraph));
  if (e == cudaSuccess) e = cudaMalloc(&nw->seeds, (size_t)nw->regions * 2 * kSeedCap * 4);
  if (e == cudaSuccess) e = cudaMalloc(&nw->ctrl, (size_t)nw->regions * kCtrlBytes);
  if (e == cudaSuccess) e = cudaMemset(nw->ctrl, 0, (size_t)nw->regions * kCtrlBytes);
  if (e == cudaSuccess)
    e = cudaMallocHost(&nw->ug_host, (size_t)nw->regions * ms::kMaxUnion * sizeof(ms::UnionGraph));
  if (e == cudaSuccess) e = cudaMallocHost(&nw->seeds_host, (size_t)nw->regions * 2 * kSeedCap * 4);
  if (e != cudaSuccess) {
    cudaGetLastError();
    msssp_union_free(nw);
    set_last_error(std::string("multi-graph sssp workspace: ") + cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  *wsp = nw;
  return GRUS_OK;
}

template <int KS>
int launch_union(UnionWs *w, UnionArgs &a, uint64_t nv, cudaStream_t s) {
  static int occ = -1;
  if (occ < 0)
    GRUS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msssp_union<KS>, kBlock, 0));
  void *args[] = {&a};
  // the L2 window on the launch's distance rows (at most 2^23 entries in a
  // batch, 32 MB) rather than its masks: the C4b batch 34.2-34.3 -> 33.4-33.6
  // ms (two alternating runs)
  return launch_persistent((const void *)msssp_union<KS>, args, kBlock, 0, occ, s, w->D,
                           (size_t)KS * nv * 4);
}

int msssp_union_run(void *wsp, int region, grus_graph *const *gs, int ng, const uint32_t *kq,
                    const uint32_t *srcs, uint32_t *const *outs, uint32_t delta, cudaStream_t s,
                    CtrlView *cv) {
  UnionWs *w = (UnionWs *)wsp;
  if (!w || region < 0 || region >= w->regions || ng < 1 || ng > ms::kMaxUnion) return GRUS_EINVAL;
  ms::UnionGraph *ugh = w->ug_host + (size_t)region * ms::kMaxUnion;
  uint32_t *sv = w->seeds_host + (size_t)region * 2 * kSeedCap, *ss = sv + kSeedCap;
  uint64_t V = 0, M = 0;
  uint32_t kmax = 0, nseeds = 0;
  for (int g = 0; g < ng; ++g) {
    const grus_graph *G = gs[g];
    if (!G || !G->csr.wts || kq[g] < 1 || kq[g] > (uint32_t)kMaxSources) return GRUS_EINVAL;
    std::memset(&ugh[g], 0, sizeof(ugh[g]));
    ugh[g].offs = G->csr.offs;
    ugh[g].cols = G->csr.cols;
    ugh[g].wts = G->csr.wts;
    ugh[g].vbase = (uint32_t)V;
    ugh[g].k = kq[g];
    for (uint32_t i = 0; i < kq[g]; ++i) {
      const uint32_t src = srcs[nseeds];
      if (src >= G->n || !outs[nseeds]) return GRUS_EINVAL;
      ugh[g].out[i] = outs[nseeds];
      sv[nseeds] = (uint32_t)V + src;
      ss[nseeds] = i;
      ++nseeds;
    }
    V += G->n;
    M += G->m;
    kmax = std::max(kmax, kq[g]);
  }
  const uint32_t ks = kmax <= 8 ? 8u : (kmax <= 16 ? 16u : 32u);
  if (V == 0 || V > w->vcap || V * ks > w->d_entries || V + M / kPiece + 1024 > w->ent_cap) {
    set_last_error("multi-graph sssp workspace too small for the launch");
    return GRUS_EINVAL;
  }
  ms::UnionGraph *ugd = w->ug + (size_t)region * ms::kMaxUnion;
  uint32_t *sd = w->seeds + (size_t)region * 2 * kSeedCap;
  char *ctrl = w->ctrl + (size_t)region * kCtrlBytes;
  GRUS_CUDA_TRY(cudaMemcpyAsync(ugd, ugh, ng * sizeof(ms::UnionGraph), cudaMemcpyHostToDevice, s));
  GRUS_CUDA_TRY(cudaMemcpyAsync(sd, sv, nseeds * 4, cudaMemcpyHostToDevice, s));
  GRUS_CUDA_TRY(cudaMemcpyAsync(sd + kSeedCap, ss, nseeds * 4, cudaMemcpyHostToDevice, s));
  GRUS_CUDA_TRY(cudaMemsetAsync(ctrl + kOffBar, 0, kCtrlBytes - kOffBar, s));
  UnionArgs a;
  std::memset((void *)&a, 0, sizeof(a));
  a.v.n = (uint32_t)V;
  a.v.k = kmax;
  a.v.srcs = sd;
  a.v.seed_slot = sd + kSeedCap;
  a.v.nseeds = nseeds;
  a.v.ug = ugd;
  a.v.ngraphs = (uint32_t)ng;
  a.v.D = w->D;
  a.v.F[0] = w->masks;
  a.v.F[1] = w->masks + V;
  a.v.far = w->masks + 2 * V;
  a.v.ent = w->ent;
  a.v.ent_cap = (uint32_t)std::min<uint64_t>(w->ent_cap, 0xFFFFFFF0ull);
  a.v.slots = (Slot *)(ctrl + kOffSlots);
  a.v.minfar = (uint32_t *)(ctrl + kOffFar);
  a.v.err = (uint32_t *)(ctrl + kOffErr);
  a.v.delta = std::max(1u, delta ? delta : kDefDelta);
  a.bar = (GridBarrier *)(ctrl + kOffBar);
  a.summary = (Summary *)(ctrl + kOffSummary);
  a.timeout_ns = 30000ull * 1000000ull;
  int rc;
  switch (ks) {
    case 8: rc = launch_union<8>(w, a, V, s); break;
    case 16: rc = launch_union<16>(w, a, V, s); break;
    default: rc = launch_union<32>(w, a, V, s); break;
  }
  if (rc) return rc;
  if (cv) {
    cv->ctrl = ctrl;
    cv->bytes = kCtrlBytes;
    cv->err_off = kOffErr;
  }
  return GRUS_OK;
}

}  // namespace grus

using namespace grus;

extern "C" int grus_sssp_multi(grus_graph *g, const uint32_t *srcs, int k, uint32_t *dists,
                               grus_stats *stats, void *stream) {
  if (!g || !srcs || !dists || k < 1 || k > kMaxSources) return GRUS_EINVAL;
  if (g->n == 0) return GRUS_EINVAL;
  uint32_t hsrc[kMaxSources];
  GRUS_CUDA_TRY(cudaMemcpy(hsrc, srcs, k * 4, cudaMemcpyDefault));
  cudaStream_t s = (cudaStream_t)stream;
  const bool dev_out = is_device_pointer(dists);
  const size_t out_bytes = (size_t)k * g->n * 4;
  uint32_t *base = dists;
  uint32_t *tmp = nullptr;
  if (!dev_out) {
    GRUS_CUDA_TRY(cudaMalloc(&tmp, out_bytes));
    base = tmp;
  }
  uint32_t *outs[kMaxSources];
  for (int i = 0; i < k; ++i) outs[i] = base + (size_t)i * g->n;
  grus_stats local;
  int rc = msssp_run(g, hsrc, k, outs, stats ? stats : (dev_out ? nullptr : &local), s);
  if (rc == GRUS_OK && !dev_out) {
    cudaError_t e = cudaMemcpyAsync(dists, base, out_bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = status_from_cuda(e);
  }
  if (tmp) cudaFree(tmp);
  return rc;
}

namespace grus {
CtrlView msssp_ctrl(grus_graph *g) {
  CtrlView v;
  std::lock_guard<std::mutex> lk(g->mu);
  const Workspace *w = (const Workspace *)g->ws[kWsMsSssp];
  if (w) {
    v.ctrl = w->ctrl;
    v.bytes = kCtrlBytes;
    v.err_off = kOffErr;
    v.bar_off = kOffBar;
  }
  return v;
}
}  // namespace grus
