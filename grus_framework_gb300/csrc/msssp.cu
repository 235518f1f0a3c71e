// msssp.cu -- multi-source SSSP: up to 32 sources in ONE persistent launch.
//
// The reference runs one SSSP per process invocation
// (samples/sssp/sssp.cu:123-170); 32 queries on one graph cost 32 launches of
// its level loop, each re-reading the adjacency lists.  Here the sources
// advance together and share every adjacency read:
//   D[v][s]   distance of v from source s, vertex-major (KS u32 per vertex, one
//             32/64/128-byte row), so the KS distances of a vertex are one
//             coalesced access;
//   F[v]      bit s set if (v, s) improved below the threshold T and must be
//             expanded (near frontier, two arrays used in turn);
//   Far[v]    bit s set if (v, s) improved to a distance >= T (far pile).
// It is the near/far label-correcting scheme of sssp.cu run per (v, s) pair
// with one shared threshold T.  A level
//   1. compacts the vertices with F[v] != 0 into work entries (v, begin, end,
//      mask) of at most kPiece edges, clearing F[v] as it reads it (one
//      atomic per CTA for the reservation);
//   2. relaxes the entries: a warp takes one entry and deals its lanes the
//      (edge, active source) pairs of it, so work follows the pairs that are
//      live rather than edges x 32; a lane whose candidate beats the distance
//      it read lowers it with a reduction (no round trip) and sets the pair's
//      bit in F'[v] (new distance < T) or Far[v].
// When a level finds no entry, T advances by Delta (or jumps to the bucket of
// the smallest far distance) and Far is scanned: pairs below the old T were
// already expanded and are dropped, pairs below the new T move to F.
// Every wait is a bounded grid barrier.  Each (v, s) pair reaches Dijkstra's
// distance whatever the schedule, so the outputs are bit-exact against
// single-source runs.
#include <algorithm>
#include <cstring>

#include "device_util.cuh"
#include "grus_internal.cuh"

namespace grus {
namespace {

constexpr int kBlock = 256;
constexpr uint32_t kPiece = 128;      // edges per work entry
constexpr uint32_t kDefDelta = 96;
constexpr int kMaxSources = 32;

struct Slot {
  uint32_t nent;          // work entries of the level
  uint32_t moved;         // pairs moved from far to near by a split
  uint32_t remaining;     // vertices still holding far pairs after a split
  uint32_t pad0;
  unsigned long long visits;
  uint32_t pad[10];
};

struct FarCtl {
  uint32_t minfar[2];
};

struct Summary {
  uint32_t levels, splits, pad0, pad1;
  unsigned long long visits, nr, mr;
};

struct Args {
  const uint32_t *__restrict__ offs;
  const uint32_t *__restrict__ cols;
  const uint32_t *__restrict__ wts;
  uint32_t n, k;
  const uint32_t *srcs;
  uint32_t *out[kMaxSources];
  uint32_t *D;
  uint32_t *F[2];
  uint32_t *far;
  uint4 *ent;
  uint32_t ent_cap;
  Slot *slots;
  FarCtl *farctl;
  GridBarrier *bar;
  uint32_t *err;
  Summary *summary;
  uint32_t delta;
  uint64_t timeout_ns;
};

// Step 1: vertices with a non-empty near mask become work entries.
__device__ __forceinline__ void build_entries(const Args &a, uint32_t *F, Slot *sl, uint32_t gtid,
                                              uint32_t nthreads) {
  const uint32_t rounds = (a.n + nthreads - 1) / nthreads;
  for (uint32_t r = 0; r < rounds; ++r) {
    const uint32_t v = r * nthreads + gtid;
    uint32_t m = 0, b = 0, e = 0, nch = 0;
    if (v < a.n) {
      m = __ldcg(F + v);
      if (m) {
        F[v] = 0u;
        b = __ldg(a.offs + v);
        e = __ldg(a.offs + v + 1);
        nch = (e - b + kPiece - 1) / kPiece;
      }
    }
    uint32_t total = 0;
    const uint32_t off = block_exclusive_scan<kBlock>(nch, &total);
    __shared__ uint32_t s_base;
    if (threadIdx.x == 0) s_base = total ? atomicAdd(&sl->nent, total) : 0u;
    __syncthreads();
    const uint32_t base = s_base + off;
    if (nch) {
      if (base + nch > a.ent_cap) {
        atomicOr(a.err, kErrOverflow);
      } else {
        for (uint32_t c = 0; c < nch; ++c)
          a.ent[base + c] = make_uint4(v, b + c * kPiece, min(e, b + (c + 1) * kPiece), m);
      }
    }
    __syncthreads();
  }
}

// Step 2: one entry per warp.  Only the p sources whose bit is set in the
// entry's mask do work: the lanes are dealt (edge, active source) pairs,
// lane = j * p + i takes the i-th active source of edge j, so a warp step
// covers floor(32 / p) edges and every lane of it relaxes a live pair (a
// lane per source would leave 32 - p lanes idle on every edge).
template <int KS>
__device__ __forceinline__ unsigned long long relax_entry(const Args &a, const uint4 ent,
                                                          uint32_t *Fn, uint32_t T) {
  const uint32_t lane = lane_id();
  const uint32_t u = ent.x, b = ent.y, e = ent.z, mask = ent.w;
  const uint32_t p = __popc(mask);
  // distance of u from source `lane`, handed to the lanes by shuffle
  const uint32_t du_all = (lane < (uint32_t)KS && ((mask >> lane) & 1u))
                              ? __ldcg(a.D + (size_t)u * KS + lane) : 0u;
  const uint32_t eps = 32u / p;           // edges per warp step
  const uint32_t j = lane / p, i = lane - j * p;
  const bool live = j < eps;
  const uint32_t s = __fns(mask, 0, (int)i + 1);  // i-th set bit of the mask
  const uint32_t du = __shfl_sync(0xffffffffu, du_all, live ? s : 0u);
  const uint32_t bit = 1u << (s & 31u);
  for (uint32_t x0 = b; x0 < e; x0 += 32) {
    const uint32_t xi = x0 + lane;
    const uint32_t c = xi < e ? __ldg(a.cols + xi) : 0u;
    const uint32_t w = xi < e ? __ldg(a.wts + xi) : 0u;
    const uint32_t ne = min(32u, e - x0);
    for (uint32_t j0 = 0; j0 < ne; j0 += 4 * eps) {
      uint32_t v[4], nd[4], cur[4];
      bool ok[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const uint32_t jj = j0 + r * eps + j;
        ok[r] = live && jj < ne;
        v[r] = __shfl_sync(0xffffffffu, c, jj & 31u);
        nd[r] = du + __shfl_sync(0xffffffffu, w, jj & 31u);
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) cur[r] = ok[r] ? __ldcg(a.D + (size_t)v[r] * KS + s) : 0u;
      // The lowering is a reduction whose old value is not waited for: a pair
      // that another lane lowered further in the meantime is marked again,
      // which costs at most one redundant expansion and never a missed one.
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        if (ok[r] && nd[r] < cur[r]) {
          atomicMin(a.D + (size_t)v[r] * KS + s, nd[r]);
          atomicOr((nd[r] < T ? Fn : a.far) + v[r], bit);
        }
      }
    }
  }
  return lane == 0 ? (unsigned long long)p * (e - b) : 0ull;
}

template <int KS>
__global__ void __launch_bounds__(kBlock) msssp_persistent(Args a) {
  const uint32_t gtid = blockIdx.x * kBlock + threadIdx.x;
  const uint32_t nthreads = gridDim.x * kBlock;
  const uint32_t gwarp = gtid >> 5, nwarps = nthreads >> 5;
  // prologue
  const size_t dn = (size_t)a.n * KS;
  for (size_t i = gtid; i < dn; i += nthreads) a.D[i] = kInfinit;
  for (uint32_t i = gtid; i < a.n; i += nthreads) {
    a.F[0][i] = 0u;
    a.F[1][i] = 0u;
    a.far[i] = 0u;
  }
  if (gtid < 4 * sizeof(Slot) / 4) ((uint32_t *)a.slots)[gtid] = 0u;
  if (gtid < sizeof(FarCtl) / 4) ((uint32_t *)a.farctl)[gtid] = 0xFFFFFFFFu;
  if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
  if (gtid < a.k) {
    const uint32_t src = a.srcs[gtid];
    a.D[(size_t)src * KS + gtid] = 0u;
    atomicOr(a.F[0] + src, 1u << gtid);
  }
  if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;

  uint32_t L = 0, T = a.delta, splits = 0, sel = 0;
  unsigned long long visits = 0;
  while (true) {
    Slot *sl = a.slots + (L & 3u);
    // reset the slot used two levels ahead
    if (gtid < sizeof(Slot) / 4) ((uint32_t *)(a.slots + ((L + 2) & 3u)))[gtid] = 0u;
    build_entries(a, a.F[sel], sl, gtid, nthreads);
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    const uint32_t nent = min(__ldcg(&sl->nent), a.ent_cap);
    if (nent == 0) {
      // near frontier empty: advance T and split the far masks into F[sel]
      const uint32_t Told = T;
      uint32_t Tnew = T + a.delta;
      // minfar[j & 1] holds the smallest distance left in the far masks by
      // split j - 1; split j reduces into the other word and resets this one
      // once every CTA has read it (after the next barrier)
      const uint32_t mf = __ldcg(&a.farctl->minfar[splits & 1u]);
      if (mf != 0xFFFFFFFFu && mf >= Tnew) Tnew = (mf / a.delta + 1) * a.delta;
      uint32_t moved = 0, remaining = 0, local_min = 0xFFFFFFFFu;
      for (uint32_t v = gtid; v < a.n; v += nthreads) {
        const uint32_t fm = __ldcg(a.far + v);
        if (!fm) continue;
        uint32_t keep = 0, mv = 0, bits = fm;
        while (bits) {
          const uint32_t sb = __ffs(bits) - 1;
          bits &= bits - 1;
          const uint32_t d = __ldcg(a.D + (size_t)v * KS + sb);
          if (d < Told) continue;  // improved below T since: expanded as near
          if (d < Tnew) {
            mv |= 1u << sb;
          } else {
            keep |= 1u << sb;
            local_min = min(local_min, d);
          }
        }
        a.far[v] = keep;
        if (mv) a.F[sel][v] = mv;  // F[sel] is all zero after build_entries
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
        if (moved) atomicAdd(&sl->moved, moved);
        if (remaining) atomicAdd(&sl->remaining, remaining);
      }
      if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
      const uint32_t mv_all = __ldcg(&sl->moved), rem_all = __ldcg(&sl->remaining);
      if (gtid == 0) a.farctl->minfar[splits & 1u] = 0xFFFFFFFFu;
      T = Tnew;
      ++splits;
      // the slot's counters are read by every CTA before they are cleared;
      // the next split adds to them only after the next build's barrier
      if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
      if (gtid == 0) {
        sl->moved = 0u;
        sl->remaining = 0u;
      }
      if (mv_all == 0 && rem_all == 0) break;  // nothing near, nothing far: done
      continue;  // build entries from the moved pairs (or split again)
    }
    uint32_t *Fn = a.F[sel ^ 1u];
    unsigned long long lv = 0;
    for (uint32_t i = gwarp; i < nent; i += nwarps) lv += relax_entry<KS>(a, __ldcg(a.ent + i), Fn, T);
    const unsigned long long bv = block_sum_u64<kBlock>(lv);
    if (threadIdx.x == 0 && bv) atomicAdd(&sl->visits, bv);
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    visits += __ldcg(&sl->visits);
    sel ^= 1u;
    ++L;
    if (L > 4u * a.n + 64u) {
      if (gtid == 0) atomicOr(a.err, kErrLevels);
      break;
    }
  }
  // epilogue: outputs (source-major) and reach counts
  unsigned long long nr = 0, mr = 0;
  for (uint32_t v = gtid; v < a.n; v += nthreads) {
    const uint32_t deg = __ldg(a.offs + v + 1) - __ldg(a.offs + v);
    for (uint32_t s = 0; s < a.k; ++s) {
      const uint32_t d = __ldcg(a.D + (size_t)v * KS + s);
      a.out[s][v] = d;
      if (d != kInfinit) {
        ++nr;
        mr += deg;
      }
    }
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

constexpr size_t kOffSlots = 0, kOffFar = 256, kOffBar = 320, kOffErr = 384, kOffSummary = 448,
                 kCtrlBytes = 512;
static_assert(4 * sizeof(Slot) <= kOffFar, "slots overlap the far control");

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
  std::memset(&a, 0, sizeof(a));
  a.offs = g->csr.offs;
  a.cols = g->csr.cols;
  a.wts = g->csr.wts;
  a.n = (uint32_t)g->n;
  a.k = (uint32_t)k;
  a.srcs = w->srcs;
  for (int i = 0; i < k; ++i) a.out[i] = outs[i];
  a.D = w->D;
  const uint64_t n1 = std::max<uint64_t>(g->n, 1);
  a.F[0] = w->masks;
  a.F[1] = w->masks + n1;
  a.far = w->masks + 2 * n1;
  a.ent = w->ent;
  a.ent_cap = w->ent_cap;
  a.slots = (Slot *)(w->ctrl + kOffSlots);
  a.farctl = (FarCtl *)(w->ctrl + kOffFar);
  a.bar = (GridBarrier *)(w->ctrl + kOffBar);
  a.err = (uint32_t *)(w->ctrl + kOffErr);
  a.summary = (Summary *)(w->ctrl + kOffSummary);
  a.delta = std::max(1u, tune_or(g->tuning.sssp_delta, kDefDelta));
  a.timeout_ns = (uint64_t)tune_or(g->tuning.timeout_ms, 30000u) * 1000000ull;
  GRUS_CUDA_TRY(cudaMemsetAsync(w->ctrl + kOffSummary, 0, kCtrlBytes - kOffSummary, s));
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
