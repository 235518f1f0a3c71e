// msbfs.cu -- multi-source BFS: up to 64 sources in ONE persistent launch,
// one bit per source in a 64-bit word per vertex (the bit-parallel
// multi-source BFS of Then et al., "The More the Merrier", VLDB 2014).
//
// The reference runs one traversal per process invocation
// (samples/bfs/bfs.cu:135-173); a batch of 64 sources costs 64 launches of
// its level loop.  Here all 64 advance together:
//   visit[v]  bit k set once source k has reached v
//   front[v]  bit k set if v is in source k's current frontier
// Push levels (sparse frontiers): the frontier list is expanded with the
// degree-binned mappings of expand.cuh; each edge (v,u) ORs
// front[v] & ~visit[u] into an accumulator word of u with one 64-bit atomicOr,
// and the first writer of u records it in the touched list; an apply phase
// then folds the accumulated bits into visit, writes the depths and bins the
// next frontier.  Pull levels (dense frontiers): each vertex ORs the frontier
// words of its in-neighbours until every missing source bit is found, with no
// atomics.  Depths are first kept as one byte per source in a row per
// vertex (16 bytes per 16 sources of the launch), written a 16-byte quarter
// at a time when the vertex gains sources; at the end one pass turns the rows into the per-source outputs,
// 32 consecutive vertices of one source per store.  (Storing each (vertex,
// source) depth as it is found leaves partly written sectors at every
// level.)  Without room for the rows, depths are stored as they are found.
// Output: depths[k * n + v] (source-major), GRUS_INFINIT where unreached.
// Bit-exact against k independent BFS runs whatever the schedule.
#include <algorithm>
#include <cstring>

#include "expand.cuh"
#include "grus_internal.cuh"

namespace grus {
namespace {

constexpr int kBlock = 256;
constexpr uint32_t kPullLane = 32;  // in-edges a lane scans alone in a pull level
constexpr uint32_t kDefHuge = 1024;
// Pull once the frontier's out-edges exceed m / alpha.  A pull level scans
// in-lists until every missing source bit is found, so it costs more the more
// sources a launch carries and the switch comes later for wide launches.
// Measured on RMAT-20/22/23/24: with 64 sources alpha 2-10 is flat and 15
// pulls one level too early (RMAT-23: 12.7 -> 6.0 ms); with 8-16 sources
// alpha 5 is 5 % slower than 10-15 on RMAT-20; 7-10 suits every width.
constexpr float kDefAlpha = 10.f;      // up to 32 sources
constexpr float kDefAlphaWide = 6.f;   // 33-64 sources

struct Slot {
  uint32_t tcount;        // touched / frontier list length of the level
  uint32_t qcount, ccount;
  uint32_t pad;
  unsigned long long mf;  // out-edges of the frontier
  unsigned long long bits;
  unsigned long long live;  // sources present in the level's frontier words
};

struct Summary {
  uint32_t levels, pull_levels, pad0, pad1;
  unsigned long long nr, mr;
};

struct Args {
  const uint32_t *__restrict__ offs;
  const uint32_t *__restrict__ cols;
  const uint32_t *__restrict__ ioffs;
  const uint32_t *__restrict__ icols;
  bool allow_pull;
  uint32_t n;
  uint64_t m;
  int k;
  const uint32_t *srcs;
  uint32_t *out[64];  // depth array of each source (n entries each)
  uint8_t *rows;      // n rows of row_bytes depth bytes, or null (direct stores)
  uint32_t row_bytes; // 16 per 16 sources: 16, 32, 48 or 64
  unsigned long long full;
  unsigned long long *visit, *front[2];
  uint32_t *touched[2];
  uint32_t *queue[2];
  uint4 *chunks[2];
  uint32_t cap, chunk_cap, huge;
  Slot *slots;
  GridBarrier *bar;
  uint32_t *err;
  Summary *summary;
  float alpha;
  uint64_t timeout_ns;
};

__device__ __forceinline__ unsigned long long warp_or64(unsigned long long x) {
  const uint32_t lo = __reduce_or_sync(0xffffffffu, (uint32_t)x);
  const uint32_t hi = __reduce_or_sync(0xffffffffu, (uint32_t)(x >> 32));
  return ((unsigned long long)hi << 32) | lo;
}

// Depth rows: byte s of vertex u's row holds its depth from source s when
// that depth is 1..kRowMaxDepth; 0 means the depth was stored directly (the
// source itself, or a vertex first reached deeper).  Bytes of sources that
// have not reached u are undefined and never read, so rows need no clearing.
constexpr uint32_t kRowMaxDepth = 254;

// w with the bytes selected by the 4-bit nibble set to fill's bytes
__device__ __forceinline__ uint32_t byte_merge(uint32_t w, uint32_t nib, uint32_t fill) {
  const uint32_t m = ((nib * 0x00204081u) & 0x01010101u) * 0xFFu;
  return (w & ~m) | (fill & m);
}

// Sets the row bytes of `bits` to `val`; `had` are the sources that reached
// u before (only quarters holding some of them are read back).
__device__ __forceinline__ void row_set(const Args &a, uint32_t u, unsigned long long bits,
                                        unsigned long long had, uint32_t val) {
  uint4 *row = reinterpret_cast<uint4 *>(a.rows + (size_t)u * a.row_bytes);
  const uint32_t fill = val * 0x01010101u;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint32_t nb = (uint32_t)(bits >> (16 * q)) & 0xFFFFu;
    if (!nb) continue;
    uint4 v = ((had >> (16 * q)) & 0xFFFFull) ? __ldcg(row + q) : make_uint4(0u, 0u, 0u, 0u);
    v.x = byte_merge(v.x, nb & 0xFu, fill);
    v.y = byte_merge(v.y, (nb >> 4) & 0xFu, fill);
    v.z = byte_merge(v.z, (nb >> 8) & 0xFu, fill);
    v.w = byte_merge(v.w, nb >> 12, fill);
    row[q] = v;
  }
}

// Records depth `val` of u from the sources in `bits` (per lane).
__device__ __forceinline__ void record_depths(const Args &a, uint32_t u, unsigned long long bits,
                                              unsigned long long had, uint32_t val) {
  if (a.rows) {
    if (val <= kRowMaxDepth) {
      row_set(a, u, bits, had, val);
      return;
    }
    row_set(a, u, bits, had, 0u);  // stored directly below
  }
  while (bits) {
    const int kb = __ffsll((long long)bits) - 1;
    bits &= bits - 1;
    a.out[kb][u] = val;
  }
}

// Warp-synchronous: lane's vertex u gets `val` for every source bit in
// `bits`; one store instruction per bit present anywhere in the warp.
__device__ __forceinline__ void write_depths(const Args &a, uint32_t u, unsigned long long bits,
                                             uint32_t val) {
  unsigned long long wor = warp_or64(bits);
  while (wor) {
    const int kb = __ffsll((long long)wor) - 1;
    wor &= wor - 1;
    if ((bits >> kb) & 1ull) a.out[kb][u] = val;
  }
}

struct PushVisitor {
  const Args *a;
  const unsigned long long *fcur;
  unsigned long long *acc;
  uint32_t *tnext;
  uint32_t *tcount;
  using aux_t = unsigned long long;
  __device__ __forceinline__ aux_t aux(uint32_t v) const { return __ldcg(fcur + v); }
  __device__ __forceinline__ void edge(uint32_t, aux_t f, uint32_t x) {
    const uint32_t u = __ldg(a->cols + x);
    const unsigned long long bits = f & ~__ldcg(a->visit + u);
    if (!bits) return;
    const unsigned long long seen = __ldcg(acc + u);
    if ((seen | bits) == seen) return;  // every bit already accumulated
    const unsigned long long old = atomicOr(acc + u, bits);
    if (old == 0ull) {
      const uint32_t pos = agg_reserve(tcount);
      if (pos < a->cap) tnext[pos] = u;
      else atomicOr(a->err, kErrOverflow);
    }
  }
};

__global__ void __launch_bounds__(kBlock, 8) msbfs_persistent(Args a) {
  const uint32_t gtid = blockIdx.x * kBlock + threadIdx.x;
  const uint32_t nthreads = gridDim.x * kBlock;
  const uint32_t lane = lane_id();
  // prologue
  for (uint32_t i = gtid; i < a.n; i += nthreads) {
    a.visit[i] = 0ull;
    a.front[0][i] = 0ull;
    a.front[1][i] = 0ull;
  }
  if (gtid < 4 * sizeof(Slot) / 4) ((uint32_t *)a.slots)[gtid] = 0u;
  if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
  if (gtid < (uint32_t)a.k) {
    const uint32_t s = a.srcs[gtid];
    atomicOr(a.visit + s, 1ull << gtid);
    atomicOr(a.front[0] + s, 1ull << gtid);
    a.out[gtid][s] = 0u;
    bool first = true;
    for (uint32_t j = 0; j < gtid; ++j) first &= a.srcs[j] != s;
    if (first) {
      if (a.rows) {
        unsigned long long same = 0;  // every source at s: stored directly above
        for (int j = 0; j < a.k; ++j) same |= (unsigned long long)(a.srcs[j] == s) << j;
        row_set(a, s, same, 0ull, 0u);
      }
      const uint32_t t = atomicAdd(&a.slots[0].tcount, 1u);
      a.touched[0][t] = s;
      atomicOr(&a.slots[0].live, a.full);
      const uint32_t b = __ldg(a.offs + s), e = __ldg(a.offs + s + 1);
      atomicAdd(&a.slots[0].mf, (unsigned long long)(e - b));
      if (!push_binned(s, b, e, a.huge, a.queue[0], &a.slots[0].qcount, a.cap, a.chunks[0],
                       &a.slots[0].ccount, a.chunk_cap))
        atomicOr(a.err, kErrOverflow);
    }
  }
  if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;

  uint32_t L = 0, pull_levels = 0;
  bool pull = false;
  while (true) {
    Slot *cur = a.slots + (L & 3u), *nx = a.slots + ((L + 1) & 3u);
    unsigned long long *fcur = a.front[L & 1u], *acc = a.front[(L + 1) & 1u];
    uint32_t *tcur = a.touched[L & 1u], *tnext = a.touched[(L + 1) & 1u];
    uint32_t *qnext = a.queue[(L + 1) & 1u];
    uint4 *cnext = a.chunks[(L + 1) & 1u];
    if (gtid < sizeof(Slot) / 4) ((uint32_t *)(a.slots + ((L + 2) & 3u)))[gtid] = 0u;
    const uint32_t val = L + 1;
    unsigned long long mf = 0, nbits = 0, live = 0;
    if (!pull) {
      // phase A: push -- accumulate new bits of every touched vertex
      PushVisitor vis{&a, fcur, acc, tnext, &nx->tcount};
      expand_binned<kBlock>(a.offs, a.queue[L & 1u], min(__ldcg(&cur->qcount), a.cap),
                            a.chunks[L & 1u], min(__ldcg(&cur->ccount), a.chunk_cap), vis);
      if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
      // phase B: apply the accumulated bits (they exclude visit: exact)
      const uint32_t tc = min(__ldcg(&nx->tcount), a.cap);
      for (uint32_t base = gtid & ~31u; base < tc; base += nthreads) {
        const uint32_t i = base + lane;
        uint32_t u = 0;
        unsigned long long bits = 0;
        if (i < tc) {
          u = __ldcg(tnext + i);
          bits = __ldcg(acc + u);
          const unsigned long long had = __ldcg(a.visit + u);
          a.visit[u] = had | bits;
          record_depths(a, u, bits, had, val);
          const uint32_t b = __ldg(a.offs + u), e = __ldg(a.offs + u + 1);
          mf += e - b;
          nbits += __popcll(bits);
          live |= bits;
          if (!push_binned(u, b, e, a.huge, qnext, &nx->qcount, a.cap, cnext, &nx->ccount,
                           a.chunk_cap))
            atomicOr(a.err, kErrOverflow);
        }
      }
    } else {
      // phase A: pull -- every vertex missing bits ORs its in-neighbours'
      // frontier words.  Only sources present in those words can add a bit
      // (a source whose frontier died -- one outside the vertex's component
      // -- never will), so a vertex looks for the live sources it misses and
      // is skipped when it misses none.  A lane scans the first kPullLane in-edges of its
      // vertex (four gathers in flight) and stops once no bit is missing;
      // longer lists still missing bits are finished by the whole warp, one
      // vertex at a time, 32 edges per step, so a high-degree vertex costs
      // its warp deg/32 steps instead of deg serial loads on one lane.
      ++pull_levels;
      const unsigned long long lv = __ldcg(&cur->live);
      const uint32_t gw = gtid >> 5, nw = nthreads >> 5;
      for (uint32_t w = gw; w * 32 < a.n; w += nw) {
        const uint32_t u = w * 32 + lane;
        unsigned long long bits = 0, vis = a.full, accb = 0;
        // `want`: vis plus every source that cannot add a bit at this level
        unsigned long long want = a.full;
        uint32_t rest_b = 0, rest_e = 0;
        if (u < a.n) {
          vis = __ldcg(a.visit + u);
          want = vis | (a.full & ~lv);
          if (want != a.full) {
            const uint32_t b = __ldg(a.ioffs + u), e = __ldg(a.ioffs + u + 1);
            const uint32_t lim = min(e, b + kPullLane);
            uint32_t x = b;
            for (; x + 4 <= lim; x += 4) {
              const uint32_t c0 = __ldg(a.icols + x), c1 = __ldg(a.icols + x + 1);
              const uint32_t c2 = __ldg(a.icols + x + 2), c3 = __ldg(a.icols + x + 3);
              accb |= __ldcg(fcur + c0) | __ldcg(fcur + c1) | __ldcg(fcur + c2) | __ldcg(fcur + c3);
              if ((accb | want) == a.full) break;
            }
            if ((accb | want) != a.full) {
              for (; x < lim; ++x) accb |= __ldcg(fcur + __ldg(a.icols + x));
              if ((accb | want) != a.full && e > lim) {
                rest_b = lim;
                rest_e = e;
              }
            }
          }
        }
        unsigned dm = __ballot_sync(0xffffffffu, rest_e > rest_b);
        while (dm) {
          const int sl = __ffs(dm) - 1;
          dm &= dm - 1;
          const uint32_t rb = __shfl_sync(0xffffffffu, rest_b, sl);
          const uint32_t re = __shfl_sync(0xffffffffu, rest_e, sl);
          const unsigned long long have =
              __shfl_sync(0xffffffffu, accb | want, sl);
          unsigned long long wacc = 0;
          for (uint32_t base = rb; base < re; base += 32) {
            const uint32_t x = base + lane;
            if (x < re) wacc |= __ldcg(fcur + __ldg(a.icols + x));
            if ((warp_or64(wacc) | have) == a.full) break;
          }
          wacc = warp_or64(wacc);
          if (lane == sl) accb |= wacc;
        }
        if (u < a.n && want != a.full) {
          bits = accb & ~vis;
          if (bits) {
            acc[u] = bits;
            a.visit[u] = vis | bits;
            const uint32_t ob = __ldg(a.offs + u), oe = __ldg(a.offs + u + 1);
            mf += oe - ob;
            nbits += __popcll(bits);
            live |= bits;
            const uint32_t pos = agg_reserve(&nx->tcount);
            if (pos < a.cap) tnext[pos] = u;
            if (!push_binned(u, ob, oe, a.huge, qnext, &nx->qcount, a.cap, cnext, &nx->ccount,
                             a.chunk_cap))
              atomicOr(a.err, kErrOverflow);
          }
        }
        if (a.rows) {
          if (bits) record_depths(a, u, bits, vis, val);
        } else {
          write_depths(a, u, bits, val);
        }
      }
      if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    }
    // phase B (both): retire the current frontier words so the array can
    // accumulate the level after next
    const uint32_t tcc = min(__ldcg(&cur->tcount), a.cap);
    for (uint32_t i = gtid; i < tcc; i += nthreads) fcur[__ldcg(tcur + i)] = 0ull;
    const unsigned long long bmf = block_sum_u64<kBlock>(mf);
    const unsigned long long bnb = block_sum_u64<kBlock>(nbits);
    // OR of the bits that entered the next frontier: one reduction per warp
    for (int o = 16; o > 0; o >>= 1) live |= __shfl_xor_sync(0xffffffffu, live, o);
    if (lane == 0 && live) atomicOr(&nx->live, live);
    if (threadIdx.x == 0 && (bmf || bnb)) {
      atomicAdd(&nx->mf, bmf);
      atomicAdd(&nx->bits, bnb);
    }
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    ++L;
    const uint32_t T = __ldcg(&nx->tcount);
    if (T == 0) break;
    const unsigned long long MF = __ldcg(&nx->mf);
    pull = a.allow_pull && (double)MF * a.alpha > (double)a.m;
    if (L > a.n + 1) {
      if (gtid == 0) atomicOr(a.err, kErrLevels);
      break;
    }
  }
  // epilogue: INFINIT for every (source, vertex) never reached; reach counts
  unsigned long long nr = 0, mr = 0;
  const uint32_t gw = gtid >> 5, nw = nthreads >> 5;
  for (uint32_t w = gw; w * 32 < a.n; w += nw) {
    const uint32_t u = w * 32 + lane;
    unsigned long long miss = 0;
    if (u < a.n) {
      const unsigned long long vis = __ldcg(a.visit + u);
      miss = a.full & ~vis;
      const uint32_t c = __popcll(vis);
      nr += c;
      mr += (unsigned long long)c * (__ldg(a.offs + u + 1) - __ldg(a.offs + u));
    }
    if (!a.rows) {
      write_depths(a, u, miss, kInfinit);
      continue;
    }
    // the rows become the outputs: per source, 32 consecutive vertices per
    // store (INFINIT where unreached; a 0 byte was stored directly)
    const unsigned long long vis = u < a.n ? a.full & ~miss : 0ull;
    const uint4 *row = reinterpret_cast<const uint4 *>(a.rows + (size_t)u * a.row_bytes);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (16 * q >= a.k) break;
      const uint4 v = (u < a.n && ((vis >> (16 * q)) & 0xFFFFull)) ? __ldcg(row + q)
                                                                    : make_uint4(0u, 0u, 0u, 0u);
      const uint32_t wd[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int sidx = 16 * q + j;
        if (sidx >= a.k) break;
        const bool got = (vis >> sidx) & 1ull;
        const uint32_t byte = (wd[j >> 2] >> (8 * (j & 3))) & 0xFFu;
        if (u < a.n && (!got || byte != 0u)) a.out[sidx][u] = got ? byte : kInfinit;
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
    a.summary->pull_levels = pull_levels;
  }
}

struct Workspace {
  unsigned long long *words = nullptr;  // visit + 2 fronts
  uint32_t *lists = nullptr;            // 2 touched + 2 queues
  uint4 *chunks = nullptr;
  uint32_t chunk_cap = 0;
  uint32_t *srcs = nullptr;
  uint32_t *depth = nullptr;            // when the caller's buffer is on the host
  size_t depth_bytes = 0;
  uint8_t *rows = nullptr;              // n x 64 depth bytes
  bool rows_tried = false;
  char *ctrl = nullptr, *ctrl_host = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

constexpr size_t kOffSlots = 0, kOffBar = 256, kOffErr = 512, kOffSummary = 576, kCtrlBytes = 768;
static_assert(kOffBar % 128 == 0 && kOffBar + sizeof(GridBarrier) <= kOffErr, "barrier layout");
static_assert(4 * sizeof(Slot) <= kOffBar && sizeof(Summary) <= kCtrlBytes - kOffSummary,
              "control block layout");

void ws_free(void *p) {
  Workspace *w = (Workspace *)p;
  if (!w) return;
  cudaFree(w->words);
  cudaFree(w->lists);
  cudaFree(w->chunks);
  cudaFree(w->srcs);
  cudaFree(w->depth);
  cudaFree(w->rows);
  cudaFree(w->ctrl);
  if (w->ctrl_host) cudaFreeHost(w->ctrl_host);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  delete w;
}

int ws_get(grus_graph *g, Workspace **out) {
  if (g->ws[kWsMsBfs]) {
    *out = (Workspace *)g->ws[kWsMsBfs];
    return GRUS_OK;
  }
  Workspace *w = new Workspace();
  const uint64_t n1 = std::max<uint64_t>(g->n, 1);
  const uint32_t huge = tune_or(g->tuning.huge_degree, kDefHuge);
  w->chunk_cap = (uint32_t)std::min<uint64_t>(g->m / kChunk + g->m / huge + 2, 0x7FFFFFFFull);
  cudaError_t e = cudaMalloc(&w->words, 3 * n1 * 8);
  if (e == cudaSuccess) e = cudaMalloc(&w->lists, 4 * n1 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&w->chunks, 2ull * w->chunk_cap * sizeof(uint4));
  if (e == cudaSuccess) e = cudaMalloc(&w->srcs, 64 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&w->ctrl, kCtrlBytes);
  if (e == cudaSuccess) e = cudaMemset(w->ctrl, 0, kCtrlBytes);
  if (e == cudaSuccess) e = cudaMallocHost(&w->ctrl_host, kCtrlBytes);
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&w->ev1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ws_free(w);
    set_last_error(std::string("msbfs workspace: ") + cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  g->ws[kWsMsBfs] = w;
  g->ws_free[kWsMsBfs] = ws_free;
  *out = w;
  return GRUS_OK;
}

}  // namespace

int msbfs_run(grus_graph *g, const uint32_t *hsrc, int k, uint32_t *const *outs,
              grus_stats *stats, cudaStream_t s) {
  if (!g || !hsrc || !outs || k < 1 || k > 64 || g->n == 0) return GRUS_EINVAL;
  for (int i = 0; i < k; ++i)
    if (hsrc[i] >= g->n || !outs[i]) {
      set_last_error("source vertex out of range");
      return GRUS_EINVAL;
    }
  std::lock_guard<std::mutex> lk(g->mu);
  Workspace *w = nullptr;
  int rc = ws_get(g, &w);
  if (rc) return rc;
  if (!w->rows_tried) {
    // the depth rows; without room for them depths are stored directly
    w->rows_tried = true;
    if (cudaMalloc(&w->rows, std::max<uint64_t>(g->n, 1) * 64) != cudaSuccess) {
      cudaGetLastError();
      w->rows = nullptr;
    }
  }
  static int occ = -1;
  if (occ < 0)
    GRUS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msbfs_persistent, kBlock, 0));
  GRUS_CUDA_TRY(cudaMemcpyAsync(w->srcs, hsrc, k * 4, cudaMemcpyHostToDevice, s));
  Args a;
  std::memset(&a, 0, sizeof(a));
  a.offs = g->csr.offs;
  a.cols = g->csr.cols;
  a.ioffs = (g->flags & GRUS_GRAPH_SYMMETRIC) ? g->csr.offs : g->csc.offs;
  a.icols = (g->flags & GRUS_GRAPH_SYMMETRIC) ? g->csr.cols : g->csc.cols;
  a.allow_pull = a.ioffs != nullptr;
  a.n = (uint32_t)g->n;
  a.m = g->m;
  a.k = k;
  a.srcs = w->srcs;
  for (int i = 0; i < k; ++i) a.out[i] = outs[i];
  a.rows = w->rows;
  // rows as wide as the sources need, so narrow launches share sectors
  a.row_bytes = 16u * (((uint32_t)k + 15u) / 16u);
  a.full = k == 64 ? ~0ull : ((1ull << k) - 1);
  a.visit = w->words;
  a.front[0] = w->words + g->n;
  a.front[1] = w->words + 2 * g->n;
  a.touched[0] = w->lists;
  a.touched[1] = w->lists + g->n;
  a.queue[0] = w->lists + 2 * g->n;
  a.queue[1] = w->lists + 3 * g->n;
  a.chunks[0] = w->chunks;
  a.chunks[1] = w->chunks + w->chunk_cap;
  a.cap = (uint32_t)g->n;
  a.chunk_cap = w->chunk_cap;
  a.huge = tune_or(g->tuning.huge_degree, kDefHuge);
  a.slots = (Slot *)(w->ctrl + kOffSlots);
  a.bar = (GridBarrier *)(w->ctrl + kOffBar);
  a.err = (uint32_t *)(w->ctrl + kOffErr);
  a.summary = (Summary *)(w->ctrl + kOffSummary);
  a.alpha = tune_or(g->tuning.multi_alpha, k > 32 ? kDefAlphaWide : kDefAlpha);
  a.timeout_ns = (uint64_t)tune_or(g->tuning.timeout_ms, 30000u) * 1000000ull;
  // barrier, error word and summary: a timed-out launch leaves stale barrier state
  GRUS_CUDA_TRY(cudaMemsetAsync(w->ctrl + kOffBar, 0, kCtrlBytes - kOffBar, s));
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(w->ev0, s));
  void *args[] = {&a};
  rc = launch_persistent((const void *)msbfs_persistent, args, kBlock, (int)g->tuning.ctas_per_sm,
                         occ, s, nullptr, 0);
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
  if (stats) {
    const Summary *sm = (const Summary *)(w->ctrl_host + kOffSummary);
    std::memset(stats, 0, sizeof(*stats));
    stats->levels = sm->levels;
    stats->bottom_up_levels = sm->pull_levels;
    stats->kernel_launches = 1;
    stats->vertices_reached = sm->nr;
    stats->edges_reached = sm->mr;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, w->ev0, w->ev1);
    stats->device_ms = ms;
  }
  return GRUS_OK;
}

}  // namespace grus

using namespace grus;

extern "C" int grus_bfs_multi(grus_graph *g, const uint32_t *srcs, int k, uint32_t *depths,
                              grus_stats *stats, void *stream) {
  if (!g || !srcs || !depths || k < 1 || k > 64) return GRUS_EINVAL;
  if (g->n == 0) return GRUS_EINVAL;
  uint32_t hsrc[64];
  GRUS_CUDA_TRY(cudaMemcpy(hsrc, srcs, k * 4, cudaMemcpyDefault));
  cudaStream_t s = (cudaStream_t)stream;
  const bool dev_out = is_device_pointer(depths);
  const size_t out_bytes = (size_t)k * g->n * 4;
  uint32_t *base = depths;
  if (!dev_out) {
    Workspace *w = nullptr;
    {
      std::lock_guard<std::mutex> lk(g->mu);
      int rc = ws_get(g, &w);
      if (rc) return rc;
      if (w->depth_bytes < out_bytes) {
        cudaFree(w->depth);
        w->depth = nullptr;
        w->depth_bytes = 0;
        GRUS_CUDA_TRY(cudaMalloc(&w->depth, out_bytes));
        w->depth_bytes = out_bytes;
      }
    }
    base = w->depth;
  }
  uint32_t *outs[64];
  for (int i = 0; i < k; ++i) outs[i] = base + (size_t)i * g->n;
  grus_stats local;
  // a host output is copied back after the launch: wait for it and check errors
  int rc = msbfs_run(g, hsrc, k, outs, stats ? stats : (dev_out ? nullptr : &local), s);
  if (rc) return rc;
  if (!dev_out) {
    GRUS_CUDA_TRY(cudaMemcpyAsync(depths, base, out_bytes, cudaMemcpyDeviceToHost, s));
    GRUS_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return GRUS_OK;
}

namespace grus {
CtrlView msbfs_ctrl(grus_graph *g) {
  CtrlView v;
  std::lock_guard<std::mutex> lk(g->mu);
  const Workspace *w = (const Workspace *)g->ws[kWsMsBfs];
  if (w) {
    v.ctrl = w->ctrl;
    v.bytes = kCtrlBytes;
    v.err_off = kOffErr;
    v.bar_off = kOffBar;
  }
  return v;
}
}  // namespace grus
