// pagerank.cu -- pull PageRank, FP32 ranks, fixed iteration count, one
// persistent launch.
//
//   r_0(v) = 1/n,  r_{t+1}(v) = (1-d)/n + d * sum_{u -> v} r_t(u) / outdeg(u)
//
// Dangling mass is not redistributed, as in the reference, which never pushes
// from out-degree-0 vertices (samples/pagerank/pr.cu:29-31,83).  The reference
// itself runs a delta-push variant (pr.cu:17-90) whose pull mode is broken
// (kernel_pull never calls job.prepare(), include/kernel.cuh:128-133); the
// drop-in headers keep that sample's semantics, this entry point computes the
// definition above.
//
// Layout: in-edges (CSC) from grus_graph_build_csc; a contribution array
// c(u) = r(u)/outdeg(u) double-buffered across iterations, so an iteration is
// one fused pass: gather c over in-edges, form r, write c_next (and r on the
// last iteration).  In-degree is binned:
//   >= kCtaTh (1024) : cut into 2048-edge pieces, one CTA per piece, the
//                      piece sums added in order afterwards
//   >= kWarpTh (64) : one warp, loads four wide, shuffle reduction
//   <  kWarpTh      : the warp's short lists laid end to end, one edge per
//                      lane, segmented warp scan (every lane busy)
// Per-thread partial sums over more than kKahanTh terms use compensated
// (Kahan-Babuska) summation; reductions across lanes are pairwise trees.
// The contribution arrays sit in an L2 persisting window.
#include <algorithm>
#include <cstring>
#include <vector>

#include "grus_internal.cuh"

namespace grus {

namespace {

constexpr int kBlock = 256;
constexpr uint32_t kCtaTh = 1024;   // in-degree from which a vertex is "heavy"
constexpr uint32_t kHChunk = 2048;  // edges per heavy-vertex piece
constexpr uint32_t kKahanTh = 16;
constexpr uint32_t kWarpTh = 64;    // in-degree from which a list gets a warp of its own
constexpr int kShortSteps = 2;      // short-list steps whose gathers are in flight together

struct Args {
  const uint32_t *__restrict__ toffs;  // CSC offsets
  const uint32_t *__restrict__ tcols;  // CSC sources
  const uint32_t *__restrict__ offs;   // CSR offsets (out-degrees)
  uint32_t n;
  float base, damping;
  int iters;
  float *c[2];
  float *rank;
  // heavy vertices (in-degree >= kCtaTh): heavy[i] = (v, first piece, pieces),
  // pieces[j] = (v, begin, end, i), partial[j] = sum over piece j
  uint4 *heavy, *pieces;
  float *partial;
  uint32_t heavy_cap, piece_cap;
  uint32_t *hcount;  // [0] heavy vertices, [1] pieces
  GridBarrier *bar;
  uint32_t *err;
  uint64_t timeout_ns;
};

// Compensated accumulator (Neumaier's variant of Kahan summation).
struct KSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = s + x;
    c += fabsf(s) >= fabsf(x) ? (s - t) + x : (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ float value() const { return s + c; }
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float outdeg_inv(const Args &a, uint32_t v) {
  const uint32_t d = __ldg(a.offs + v + 1) - __ldg(a.offs + v);
  return d ? 1.0f / (float)d : 0.0f;
}

__device__ __forceinline__ void finish(const Args &a, uint32_t v, float sum, float *cn, bool last) {
  const float r = a.base + a.damping * sum;
  cn[v] = r * outdeg_inv(a, v);
  if (last) a.rank[v] = r;
}

// Strided gather of one list: four source ids, then their four
// contributions, are loaded before they are added (four load chains in
// flight per thread).
__device__ __forceinline__ float gather_seq(const Args &a, const float *cs, uint32_t b,
                                            uint32_t e, uint32_t step) {
  if (b >= e) return 0.f;
  const bool comp = (e - b) > kKahanTh * step;
  KSum k;
  float s = 0.f;
  uint32_t x = b;
  for (; x + 3 * step < e; x += 4 * step) {
    const uint32_t u0 = __ldg(a.tcols + x), u1 = __ldg(a.tcols + x + step);
    const uint32_t u2 = __ldg(a.tcols + x + 2 * step), u3 = __ldg(a.tcols + x + 3 * step);
    const float f0 = __ldcg(cs + u0), f1 = __ldcg(cs + u1);
    const float f2 = __ldcg(cs + u2), f3 = __ldcg(cs + u3);
    if (comp) {
      k.add(f0);
      k.add(f1);
      k.add(f2);
      k.add(f3);
    } else {
      s += (f0 + f1) + (f2 + f3);
    }
  }
  for (; x < e; x += step) {
    const float f = __ldcg(cs + __ldg(a.tcols + x));
    if (comp) k.add(f);
    else s += f;
  }
  return comp ? k.value() : s;
}

// The short lists (< kWarpTh in-edges) of a warp's vertices, laid end to end:
// lane k of a step takes edge k of the concatenation (coalesced source-id
// loads, every lane busy), a segmented warp scan sums each vertex's run
// within the step (a fixed pairwise order), and the owning lane adds its
// run's sum.  Steps go in rounds of kShortSteps: all their source ids, then
// all their contributions, are loaded before any is summed (kShortSteps
// gathers in flight per lane).  Returns the full sum for the calling lane's
// vertex.
__device__ __forceinline__ uint32_t short_owner(uint32_t incl, uint32_t k) {
  int j = 0;
#pragma unroll
  for (int step = 16; step >= 1; step >>= 1) {
    const uint32_t pv = __shfl_sync(0xffffffffu, incl, j + step - 1);
    if (pv <= k) j += step;
  }
  return (uint32_t)j;
}

// Adds to acc the calling lane's run within the step starting at k0, whose
// lane value is v (edge k0 + lane's contribution, 0 past the end).
__device__ __forceinline__ void short_step(KSum &acc, uint32_t lane, uint32_t k0, uint32_t oe,
                                           uint32_t excl, uint32_t incl, float v) {
  bool head = lane == 0 || k0 + lane == oe;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float tv = __shfl_up_sync(0xffffffffu, v, o);
    const bool th = __shfl_up_sync(0xffffffffu, head, o);
    if ((int)lane >= o && !head) {
      v += tv;
      head = th;
    }
  }
  // this lane's run within the step ends at min(incl, k0 + 32) - 1
  const uint32_t rs = max(excl, k0), re = min(incl, k0 + 32);
  const float t = __shfl_sync(0xffffffffu, v, rs < re ? re - 1 - k0 : 0);
  if (rs < re) acc.add(t);
}

__device__ __forceinline__ float gather_short(const Args &a, const float *cs, uint32_t beg,
                                              uint32_t deg) {
  const uint32_t lane = lane_id();
  uint32_t incl = deg;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if ((int)lane >= o) incl += t;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  const uint32_t excl = incl - deg;
  KSum acc;
  constexpr int P = kShortSteps;
  for (uint32_t k0 = 0; k0 < total; k0 += 32 * P) {
    uint32_t oe[P], u[P];
    float v[P];
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const uint32_t k = k0 + 32 * i + lane;
      const uint32_t j = short_owner(incl, k);
      const uint32_t ob = __shfl_sync(0xffffffffu, beg, j);
      oe[i] = __shfl_sync(0xffffffffu, excl, j);
      u[i] = k < total ? __ldg(a.tcols + ob + (k - oe[i])) : 0u;
    }
#pragma unroll
    for (int i = 0; i < P; ++i) v[i] = k0 + 32 * i + lane < total ? __ldcg(cs + u[i]) : 0.f;
#pragma unroll
    for (int i = 0; i < P; ++i)
      if (k0 + 32 * i < total) short_step(acc, lane, k0 + 32 * i, oe[i], excl, incl, v[i]);
  }
  return acc.value();
}

// One iteration is
//   A. every warp, independently, takes groups of 32 consecutive vertices:
//      in-lists of 32..kCtaTh-1 edges by the whole warp (four loads in
//      flight), shorter ones laid end to end (gather_short); heavy vertices
//      are skipped;
//   B. every CTA takes pieces of kHChunk edges of the heavy vertices and
//      writes each piece's sum;
//   -- grid barrier --
//   C. each heavy vertex adds its pieces in order (compensated) and finishes;
//   -- grid barrier --
// so no block barrier separates the warps of a light tile, and a heavy
// vertex is spread over many CTAs.  The heavy lists are built once per call.
__global__ void __launch_bounds__(kBlock, 8) pr_persistent(Args a) {
  __shared__ float s_part[kBlock / 32];
  const uint32_t gtid = blockIdx.x * kBlock + threadIdx.x;
  const uint32_t nthreads = gridDim.x * kBlock;
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
  const uint32_t gwarp = gtid >> 5, nwarps = nthreads >> 5;
  const float r0 = 1.0f / (float)a.n;
  for (uint32_t v = gtid; v < a.n; v += nthreads) {
    a.c[0][v] = r0 * outdeg_inv(a, v);
    const uint32_t b = __ldg(a.toffs + v), e = __ldg(a.toffs + v + 1);
    if (e - b >= kCtaTh) {
      const uint32_t np = (e - b + kHChunk - 1) / kHChunk;
      const uint32_t hi = atomicAdd(&a.hcount[0], 1u);
      const uint32_t p0 = atomicAdd(&a.hcount[1], np);
      if (hi >= a.heavy_cap || p0 + np > a.piece_cap) {
        atomicOr(a.err, kErrOverflow);
        continue;
      }
      a.heavy[hi] = make_uint4(v, p0, np, 0u);
      for (uint32_t k = 0; k < np; ++k)
        a.pieces[p0 + k] = make_uint4(v, b + k * kHChunk, min(e, b + (k + 1) * kHChunk), hi);
    }
  }
  if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
  const uint32_t nheavy = min(__ldcg(&a.hcount[0]), a.heavy_cap);
  const uint32_t npieces = min(__ldcg(&a.hcount[1]), a.piece_cap);

  for (int it = 0; it < a.iters; ++it) {
    const float *cs = a.c[it & 1];
    float *cn = a.c[(it + 1) & 1];
    const bool last = it + 1 == a.iters;
    // A: light vertices, warp by warp
    for (uint32_t g0 = gwarp * 32; g0 < a.n; g0 += nwarps * 32) {
      const uint32_t v = g0 + lane;
      uint32_t beg = 0, end = 0;
      if (v < a.n) {
        beg = __ldg(a.toffs + v);
        end = __ldg(a.toffs + v + 1);
      }
      bool done = v >= a.n || end - beg >= kCtaTh;
      while (true) {
        const uint32_t ball = __ballot_sync(0xffffffffu, !done && end - beg >= kWarpTh);
        if (!ball) break;
        const int leader = __ffs(ball) - 1;
        const uint32_t wv = __shfl_sync(0xffffffffu, v, leader);
        const uint32_t wb = __shfl_sync(0xffffffffu, beg, leader);
        const uint32_t we = __shfl_sync(0xffffffffu, end, leader);
        if ((int)lane == leader) done = true;
        const float tot = warp_sum(gather_seq(a, cs, wb + lane, we, 32));
        if ((int)lane == leader) finish(a, wv, tot, cn, last);
      }
      const float sum = gather_short(a, cs, beg, done ? 0u : end - beg);
      if (!done) finish(a, v, sum, cn, last);
    }
    // B: pieces of heavy vertices, CTA by CTA
    for (uint32_t p = blockIdx.x; p < npieces; p += gridDim.x) {
      const uint4 pc = __ldcg(a.pieces + p);
      const float part = warp_sum(gather_seq(a, cs, pc.y + threadIdx.x, pc.z, kBlock));
      if (lane == 0) s_part[warp] = part;
      __syncthreads();
      if (threadIdx.x == 0) {
        float tot = 0.f;
        for (int i = 0; i < kBlock / 32; ++i) tot += s_part[i];
        a.partial[p] = tot;
      }
      __syncthreads();
    }
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    // C: heavy vertices add their pieces in order
    for (uint32_t h = gtid; h < nheavy; h += nthreads) {
      const uint4 hv = __ldcg(a.heavy + h);
      KSum k;
      for (uint32_t j = 0; j < hv.z; ++j) k.add(__ldcg(a.partial + hv.y + j));
      finish(a, hv.x, k.value(), cn, last);
    }
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
  }
}

struct Workspace {
  float *c = nullptr;   // 2 * n contributions
  float *rank = nullptr;
  uint4 *heavy = nullptr, *pieces = nullptr;
  float *partial = nullptr;
  uint32_t heavy_cap = 0, piece_cap = 0;
  char *ctrl = nullptr, *ctrl_host = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

constexpr size_t kOffBar = 0, kOffErr = 256, kOffHeavy = 320, kCtrlBytes = 384;
static_assert(kOffBar + sizeof(GridBarrier) <= kOffErr, "barrier layout");

void ws_free(void *p) {
  Workspace *w = (Workspace *)p;
  if (!w) return;
  cudaFree(w->c);
  cudaFree(w->rank);
  cudaFree(w->heavy);
  cudaFree(w->pieces);
  cudaFree(w->partial);
  cudaFree(w->ctrl);
  if (w->ctrl_host) cudaFreeHost(w->ctrl_host);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  delete w;
}

int ws_get(grus_graph *g, Workspace **out) {
  if (g->ws[kWsPr]) {
    *out = (Workspace *)g->ws[kWsPr];
    return GRUS_OK;
  }
  Workspace *w = new Workspace();
  const uint64_t n1 = std::max<uint64_t>(g->n, 1);
  w->heavy_cap = (uint32_t)std::min<uint64_t>(n1, g->m / kCtaTh + 1);
  w->piece_cap = (uint32_t)(g->m / kHChunk + w->heavy_cap + 1);
  cudaError_t e = cudaMalloc(&w->c, 2 * n1 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&w->heavy, (size_t)w->heavy_cap * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&w->pieces, (size_t)w->piece_cap * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&w->partial, (size_t)w->piece_cap * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&w->ctrl, kCtrlBytes);
  if (e == cudaSuccess) e = cudaMemset(w->ctrl, 0, kCtrlBytes);
  if (e == cudaSuccess) e = cudaMallocHost(&w->ctrl_host, kCtrlBytes);
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ws_free(w);
    set_last_error(std::string("pagerank workspace: ") + cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  g->ws[kWsPr] = w;
  g->ws_free[kWsPr] = ws_free;
  *out = w;
  return GRUS_OK;
}

}  // namespace
}  // namespace grus

using namespace grus;

extern "C" int grus_pagerank(grus_graph *g, float damping, int iters, float *rank,
                             grus_stats *stats, void *stream) {
  if (!g || !rank || iters < 0 || !(damping >= 0.f && damping <= 1.f)) return GRUS_EINVAL;
  if (g->n == 0) return GRUS_OK;
  cudaStream_t s = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g->mu);
  int rc = build_csc_locked(g);
  if (rc) return rc;
  Workspace *w = nullptr;
  rc = ws_get(g, &w);
  if (rc) return rc;
  const bool dev_out = is_device_pointer(rank);
  if (!dev_out && !w->rank) GRUS_CUDA_TRY(cudaMalloc(&w->rank, g->n * 4));
  static int occ = -1;
  if (occ < 0)
    GRUS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pr_persistent, kBlock, 0));
  Args a;
  std::memset(&a, 0, sizeof(a));
  a.toffs = g->csc.offs;
  a.tcols = g->csc.cols;
  a.offs = g->csr.offs;
  a.n = (uint32_t)g->n;
  a.base = (1.0f - damping) / (float)g->n;
  a.damping = damping;
  a.iters = iters;
  a.c[0] = w->c;
  a.c[1] = w->c + g->n;
  a.rank = dev_out ? rank : w->rank;
  a.heavy = w->heavy;
  a.pieces = w->pieces;
  a.partial = w->partial;
  a.heavy_cap = w->heavy_cap;
  a.piece_cap = w->piece_cap;
  a.hcount = (uint32_t *)(w->ctrl + kOffHeavy);
  a.bar = (GridBarrier *)(w->ctrl + kOffBar);
  a.err = (uint32_t *)(w->ctrl + kOffErr);
  a.timeout_ns = (uint64_t)tune_or(g->tuning.timeout_ms, 30000u) * 1000000ull;
  if (iters == 0) {
    // r_0 = 1/n
    std::vector<float> h(g->n, 1.0f / (float)g->n);
    GRUS_CUDA_TRY(cudaMemcpyAsync(rank, h.data(), g->n * 4, cudaMemcpyDefault, s));
    GRUS_CUDA_TRY(cudaStreamSynchronize(s));
    return GRUS_OK;
  }
  // barrier, error word and heavy-list counters: a timed-out launch leaves
  // stale barrier state
  GRUS_CUDA_TRY(cudaMemsetAsync(w->ctrl + kOffBar, 0, kOffHeavy + 8 - kOffBar, s));
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(w->ev0, s));
  void *args[] = {&a};
  rc = launch_persistent((const void *)pr_persistent, args, kBlock, (int)g->tuning.ctas_per_sm,
                         occ, s, w->c, 2 * g->n * 4);
  if (rc) return rc;
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(w->ev1, s));
  if (!dev_out) GRUS_CUDA_TRY(cudaMemcpyAsync(rank, w->rank, g->n * 4, cudaMemcpyDeviceToHost, s));
  if (!stats && dev_out) return GRUS_OK;
  GRUS_CUDA_TRY(cudaMemcpyAsync(w->ctrl_host, w->ctrl, kCtrlBytes, cudaMemcpyDeviceToHost, s));
  GRUS_CUDA_TRY(cudaStreamSynchronize(s));
  const uint32_t errbits = *(uint32_t *)(w->ctrl_host + kOffErr);
  if (errbits) {
    cudaMemsetAsync(w->ctrl, 0, kCtrlBytes, s);
    cudaStreamSynchronize(s);
    return status_from_device_error(errbits);
  }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->levels = (uint32_t)iters;
    stats->kernel_launches = 1;
    stats->vertices_reached = g->n;
    stats->edges_reached = g->m * (uint64_t)iters;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, w->ev0, w->ev1);
    stats->device_ms = ms;
  }
  return GRUS_OK;
}

namespace grus {
CtrlView pr_ctrl(grus_graph *g) {
  CtrlView v;
  std::lock_guard<std::mutex> lk(g->mu);
  const Workspace *w = (const Workspace *)g->ws[kWsPr];
  if (w) {
    v.ctrl = w->ctrl;
    v.bytes = kCtrlBytes;
    v.err_off = kOffErr;
    v.bar_off = kOffBar;
  }
  return v;
}
}  // namespace grus
