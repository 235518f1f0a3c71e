// cc.cu -- connected components with canonical minimum-id labels.
//
// Replaces the reference's CC_single_gpu loop (samples/cc/cc.cu:124-190):
// min-label propagation from a full frontier, label[dst] = atomicMin(label[src])
// along every edge (:69-79), one kernel + compaction + host sync per round,
// about diameter-many rounds.  On a symmetric graph its fixpoint is the minimum
// vertex id of each component; this file computes the same labels with a
// lock-free union-find organised as in Afforest (Sutton, Ben-Nun & Barak,
// IPDPS 2018):
//   1. parent[v] = v
//   2. link every vertex with its first `kSample` neighbours (one pass), compress
//   3. find the most frequent root among 1024 sampled vertices (the giant
//      component) on the device
//   4. every vertex outside the giant component links its remaining
//      neighbours -- degree-binned with the mappings of expand.cuh; vertices
//      inside it are skipped, their edges are seen from the other endpoint
//   5. label[v] = the smallest vertex id among the vertices with v's root
// Linking hooks the root of lower priority under the root of higher
// priority, priority = (degree, id): a hub becomes the root of its
// neighbours' trees, so the many threads that link a low-degree vertex to
// the same hub each swing their own root's parent instead of all racing for
// the hub's (hooking by id made those threads retry one after another).
// The root is then not the smallest id of its set, so step 5 takes the
// minimum explicitly.  Labels are order-independent (the minimum of each
// set), so the result is bit-exact against the oracle's union-find.  Edges
// are taken as undirected: on a non-symmetric graph the result is its weakly
// connected components (step 4 then skips nothing).
#include <algorithm>
#include <cstring>

#include "expand.cuh"
#include "grus_internal.cuh"

namespace grus {
namespace {

constexpr int kBlock = 256;
constexpr uint32_t kSample = 2;
constexpr int kModeSamples = 1024;
constexpr uint32_t kDefHuge = 1024;

__device__ __forceinline__ uint32_t find_root(uint32_t *p, uint32_t x) {
  uint32_t y = __ldcg(p + x);
  while (y != x) {
    const uint32_t z = __ldcg(p + y);
    if (z == y) return y;
    p[x] = z;  // path halving: z is an ancestor of x
    x = z;
    y = __ldcg(p + x);
  }
  return x;
}

// Hooking priority of a vertex: its degree, ties broken by id (a total order,
// so concurrent hooks never form a cycle).
__device__ __forceinline__ uint64_t prio(const uint32_t *__restrict__ offs, uint32_t x) {
  return ((uint64_t)(__ldg(offs + x + 1) - __ldg(offs + x)) << 32) | x;
}

// find_root of two vertices at once: both chains advance in lockstep, so the
// loads of a step are in flight together (path halving on both).
__device__ __forceinline__ void find_root2(uint32_t *p, uint32_t &a, uint32_t &b) {
  uint32_t ya = __ldcg(p + a), yb = __ldcg(p + b);
  bool da = ya == a, db = yb == b;  // at a root
  while (!(da && db)) {
    const uint32_t za = da ? ya : __ldcg(p + ya);
    const uint32_t zb = db ? yb : __ldcg(p + yb);
    if (!da) {
      if (za == ya) {
        a = ya;
        da = true;
      } else {
        p[a] = za;  // path halving: za is an ancestor of a
        a = za;
      }
    }
    if (!db) {
      if (zb == yb) {
        b = yb;
        db = true;
      } else {
        p[b] = zb;
        b = zb;
      }
    }
    if (!da) ya = __ldcg(p + a);
    if (!db) yb = __ldcg(p + b);
    da = da || ya == a;
    db = db || yb == b;
  }
}

__device__ __forceinline__ void link(const uint32_t *__restrict__ offs, uint32_t *p, uint32_t u,
                                     uint32_t v) {
  uint32_t ru = u, rv = v;
  find_root2(p, ru, rv);
  while (ru != rv) {
    if (prio(offs, ru) > prio(offs, rv)) {
      const uint32_t t = ru;
      ru = rv;
      rv = t;
    }
    const uint32_t old = atomicCAS(p + ru, ru, rv);  // hook lower priority under higher
    if (old == ru) return;
    ru = old;
    find_root2(p, ru, rv);
  }
}

__global__ void k_init(uint32_t *p, uint32_t n) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    p[v] = v;
}

// Links every vertex with its first kSample neighbours in one pass: their
// ids are loaded together (usually one line), then linked in turn.
__global__ void k_link_sample(const uint32_t *__restrict__ offs, const uint32_t *__restrict__ cols,
                              uint32_t *p, uint32_t n) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const uint32_t b = __ldg(offs + v), e = __ldg(offs + v + 1);
    uint32_t u[kSample];
#pragma unroll
    for (uint32_t r = 0; r < kSample; ++r) u[r] = b + r < e ? __ldg(cols + b + r) : v;
#pragma unroll
    for (uint32_t r = 0; r < kSample; ++r)
      if (u[r] != v) link(offs, p, v, u[r]);
  }
}

__global__ void k_compress(uint32_t *p, uint32_t n) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    p[v] = find_root(p, v);
}

// After a full compression (p[v] = root): lo[root] = the smallest member id.
// lo starts at all ones.  A warp's lanes hold consecutive ids, so among the
// lanes with the same root the lowest holds the smallest id and alone issues
// the atomic, and only if its id is below the value it reads -- the giant
// component costs a few atomics instead of one per member.
__global__ void k_min_member(const uint32_t *__restrict__ p, uint32_t *lo, uint32_t n) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t v0 = blockIdx.x * blockDim.x; v0 < n; v0 += stride) {
    const uint32_t v = v0 + threadIdx.x;
    const uint32_t r = v < n ? __ldg(p + v) : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(0xffffffffu, r);
    const bool first = (peers & ((1u << (threadIdx.x & 31u)) - 1u)) == 0u;
    if (v < n && first && v < lo[r]) atomicMin(lo + r, v);  // a stale read only costs an atomic
  }
}

__global__ void k_label(const uint32_t *__restrict__ p, const uint32_t *__restrict__ lo,
                        uint32_t *label, uint32_t n) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    label[v] = __ldcg(lo + __ldg(p + v));
}

__global__ void k_fill(uint32_t *x, uint32_t val, uint32_t n) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    x[v] = val;
}

// Most frequent root among kModeSamples vertices picked by a fixed hash.
__global__ void k_giant(uint32_t *p, uint32_t n, uint32_t *giant) {
  __shared__ uint32_t s_root[kModeSamples];
  __shared__ unsigned long long s_best;
  const uint32_t t = threadIdx.x;
  const uint32_t v = (uint32_t)(((uint64_t)t * 2654435761ull + 12345ull) % n);
  s_root[t] = find_root(p, v);
  if (t == 0) s_best = 0;
  __syncthreads();
  uint32_t cnt = 0;
  for (int i = 0; i < kModeSamples; ++i) cnt += s_root[i] == s_root[t];
  // key: count high, then the smaller root wins ties
  atomicMax(&s_best, ((unsigned long long)cnt << 32) | (0xFFFFFFFFu - s_root[t]));
  __syncthreads();
  if (t == 0) *giant = 0xFFFFFFFFu - (uint32_t)(s_best & 0xFFFFFFFFull);
}

struct Ctl {
  uint32_t giant, qcount, ccount, err;
};

// Queues the vertices whose remaining neighbours must still be linked.  On a
// symmetric graph the giant component's vertices are skipped (each of their
// edges is also stored at the other endpoint); otherwise nothing is skipped.
__global__ void k_collect(const uint32_t *__restrict__ offs, uint32_t *p, uint32_t n,
                          Ctl *ctl, uint32_t *queue, uint4 *chunks, uint32_t ccap,
                          uint32_t huge, bool skip_giant) {
  const uint32_t giant = skip_giant ? __ldcg(&ctl->giant) : 0xFFFFFFFFu;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const uint32_t b = __ldg(offs + v), e = __ldg(offs + v + 1);
    if (e - b <= kSample) continue;
    if (find_root(p, v) == giant) continue;
    if (!push_binned(v, b + kSample, e, huge, queue, &ctl->qcount, n, chunks, &ctl->ccount, ccap))
      atomicOr(&ctl->err, kErrOverflow);
  }
}

struct LinkVisitor {
  const uint32_t *offs, *cols;
  uint32_t *p;
  using aux_t = uint32_t;
  __device__ __forceinline__ uint32_t aux(uint32_t v) const { return __ldg(offs + v) + kSample; }
  __device__ __forceinline__ void edge(uint32_t src, uint32_t first, uint32_t x) {
    if (x < first) return;  // neighbours linked in the sampling rounds
    link(offs, p, src, __ldg(cols + x));
  }
};

__global__ void __launch_bounds__(kBlock) k_link_rest(const uint32_t *__restrict__ offs,
                                                      const uint32_t *__restrict__ cols,
                                                      uint32_t *p, const Ctl *ctl,
                                                      const uint32_t *queue, uint32_t qcap,
                                                      const uint4 *chunks, uint32_t ccap) {
  LinkVisitor vis{offs, cols, p};
  expand_binned<kBlock>(offs, queue, min(__ldcg(&ctl->qcount), qcap), chunks,
                        min(__ldcg(&ctl->ccount), ccap), vis);
}

struct Workspace {
  uint32_t *parent = nullptr, *queue = nullptr;
  uint32_t *label = nullptr;  // labels for a host output buffer
  uint4 *chunks = nullptr;
  uint32_t ccap = 0;
  Ctl *ctl = nullptr, *ctl_host = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

void ws_free(void *q) {
  Workspace *w = (Workspace *)q;
  if (!w) return;
  cudaFree(w->parent);
  cudaFree(w->queue);
  cudaFree(w->label);
  cudaFree(w->chunks);
  cudaFree(w->ctl);
  if (w->ctl_host) cudaFreeHost(w->ctl_host);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  delete w;
}

int ws_get(grus_graph *g, Workspace **out) {
  if (g->ws[kWsCc]) {
    *out = (Workspace *)g->ws[kWsCc];
    return GRUS_OK;
  }
  Workspace *w = new Workspace();
  const uint64_t n1 = std::max<uint64_t>(g->n, 1);
  const uint32_t huge = tune_or(g->tuning.huge_degree, kDefHuge);
  w->ccap = (uint32_t)std::min<uint64_t>(g->m / kChunk + g->m / huge + 2, 0x7FFFFFFFull);
  cudaError_t e = cudaMalloc(&w->parent, n1 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&w->queue, n1 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&w->chunks, (uint64_t)w->ccap * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&w->ctl, sizeof(Ctl));
  if (e == cudaSuccess) e = cudaMallocHost(&w->ctl_host, sizeof(Ctl));
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ws_free(w);
    set_last_error(std::string("cc workspace: ") + cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  g->ws[kWsCc] = w;
  g->ws_free[kWsCc] = ws_free;
  *out = w;
  return GRUS_OK;
}

}  // namespace
}  // namespace grus

using namespace grus;

extern "C" int grus_cc(grus_graph *g, uint32_t *label, grus_stats *stats, void *stream) {
  if (!g || !label) return GRUS_EINVAL;
  if (g->n == 0) return GRUS_OK;
  cudaStream_t s = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g->mu);
  Workspace *w = nullptr;
  int rc = ws_get(g, &w);
  if (rc) return rc;
  const bool dev_out = is_device_pointer(label);
  if (!dev_out && !w->label) GRUS_CUDA_TRY(cudaMalloc(&w->label, g->n * 4));
  const uint32_t n = (uint32_t)g->n;
  const int sms = std::max(device_sm_count(), 1);
  const int grid = sms * 8;
  static int occ = -1;
  if (occ < 0) GRUS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_link_rest, kBlock, 0));
  const uint32_t huge = tune_or(g->tuning.huge_degree, kDefHuge);
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(w->ev0, s));
  GRUS_CUDA_TRY(cudaMemsetAsync(w->ctl, 0, sizeof(Ctl), s));
  k_init<<<grid, kBlock, 0, s>>>(w->parent, n);
  k_link_sample<<<grid, kBlock, 0, s>>>(g->csr.offs, g->csr.cols, w->parent, n);
  k_compress<<<grid, kBlock, 0, s>>>(w->parent, n);
  k_giant<<<1, kModeSamples, 0, s>>>(w->parent, n, &w->ctl->giant);
  k_collect<<<grid, kBlock, 0, s>>>(g->csr.offs, w->parent, n, w->ctl, w->queue, w->chunks,
                                    w->ccap, huge, (g->flags & GRUS_GRAPH_SYMMETRIC) != 0);
  k_link_rest<<<sms * std::max(occ, 1), kBlock, 0, s>>>(g->csr.offs, g->csr.cols, w->parent,
                                                          w->ctl, w->queue, n, w->chunks, w->ccap);
  // canonical labels: the smallest member of each set (the queue is free now)
  uint32_t *dst = dev_out ? label : w->label;
  k_compress<<<grid, kBlock, 0, s>>>(w->parent, n);
  k_fill<<<grid, kBlock, 0, s>>>(w->queue, 0xFFFFFFFFu, n);
  k_min_member<<<grid, kBlock, 0, s>>>(w->parent, w->queue, n);
  k_label<<<grid, kBlock, 0, s>>>(w->parent, w->queue, dst, n);
  GRUS_CUDA_TRY(cudaGetLastError());
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(w->ev1, s));
  if (!dev_out) GRUS_CUDA_TRY(cudaMemcpyAsync(label, dst, g->n * 4, cudaMemcpyDeviceToHost, s));
  if (!stats && dev_out) return GRUS_OK;
  GRUS_CUDA_TRY(cudaMemcpyAsync(w->ctl_host, w->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
  GRUS_CUDA_TRY(cudaStreamSynchronize(s));
  if (w->ctl_host->err) return status_from_device_error(w->ctl_host->err);
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->levels = kSample + 1;
    stats->kernel_launches = 10;
    stats->vertices_reached = g->n;
    stats->edges_reached = g->m;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, w->ev0, w->ev1);
    stats->device_ms = ms;
  }
  return GRUS_OK;
}
