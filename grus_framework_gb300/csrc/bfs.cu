// bfs.cu -- single-source BFS as ONE persistent, direction-optimising launch.
//
// Replaces the reference's host-driven level loop (samples/bfs/bfs.cu:135-173:
// per level kernel<...,Frontier<BDF>> push_kernel + flag_to_wl compaction +
// three blocking 4-byte D2H copies, include/kernel.cuh:62-80,154-165,
// src/worklist.cu:87-93) and its static --pull variant (kernel_pull over a
// byte-map Frontier<BITMAP>, include/kernel.cuh:18-40,124-133).
//
// Design (sm_103a, 152 SMs):
//   * cooperative launch of SMs x k CTAs; levels are separated by a grid
//     barrier whose waits are time-bounded (grus_internal.cuh); no host sync
//     inside a traversal.
//   * frontier state: 1-bit bitmaps (visited + three rotating frontier maps,
//     4 * n/8 bytes, one contiguous block covered by an L2 persistence window)
//     and a vertex queue for push levels.
//   * push (top-down) levels, degree-binned:
//       - degree >= huge (8192): split into 1024-edge chunks when enqueued,
//         each chunk expanded by a whole CTA (spreads hubs over all SMs);
//       - degree >= 256: CTA-cooperative expansion within a queue tile;
//       - degree >= 32: warp-cooperative expansion;
//       - degree < 32: warp scan-based gather (lanes take consecutive edges of
//         the warp's 32 vertices, owner found by a shuffle binary search).
//     A discovered vertex is claimed with one atomicOr on the L2-resident
//     visited bitmap and appended with a warp-aggregated reservation.
//   * pull (bottom-up) levels: a warp owns 32 consecutive vertices (one bitmap
//     word); each unvisited vertex scans its first `bu_scan` neighbours four at
//     a time and stops at the first frontier parent; longer unresolved lists
//     are finished by the whole warp (32 neighbours per ballot).  The word's
//     next-frontier and visited bits are written with one store per warp.
//   * pull levels read in-edges: the CSR itself on a symmetric graph, the CSC
//     (grus_graph_build_csc) on a directed one; without a CSC a directed graph
//     runs push-only.
//   * direction: Beamer's heuristic -- push->pull when the frontier grows and
//     m_f > m_u/alpha, pull->push when n_f < n/beta and the frontier shrinks;
//     the first push level after a pull level turns the frontier bitmap into
//     the queue with one atomic per CTA per 256 words.
//   * narrow tail: a long traversal (16+ levels) whose push frontier and
//     remaining edges have become small is handed to bfs_narrow, a cluster of
//     up to 16 CTAs of 1024 threads launched after the persistent kernel,
//     which runs the remaining levels with one hardware cluster barrier each,
//     frontiers in distributed shared memory and prefetches of the next
//     level's adjacency (about 3.3 µs per level against 9-10 µs for a grid
//     barrier level).
// Depths are order-independent (every writer stores level+1), so results are
// bit-exact against the serial oracle whatever the schedule.
#include <algorithm>
#include <cstring>

#include "expand.cuh"
#include "grus_internal.cuh"

namespace grus {
namespace {

namespace cg = cooperative_groups;

constexpr int kBlock = 256;
constexpr uint32_t kDefHuge = 8192;   // chunking threshold
constexpr uint32_t kDefBuScan = 4;    // pull: neighbours a lane checks alone (one round)
// ... for a managed graph, whose adjacency may be read over the host link:
// deferring fewer lists to the warp's 32-neighbour rounds reads fewer lines
constexpr uint32_t kDefBuScanManaged = 8;
constexpr uint32_t kDefBuWords = 4;   // pull: bitmap words per warp step
constexpr float kDefAlpha = 15.f, kDefBeta = 18.f;
// Narrow tail: a traversal still running after kNarrowAfter levels, with a
// push frontier of at most kNarrowNf vertices per tail CTA and at most
// kNarrowMu edges left whose source is undiscovered, is finished by one
// thread-block cluster of up to 16 CTAs of 1024 threads.  The edge bound caps
// the work the cluster may be left with.
constexpr uint32_t kNarrowAfter = 16;
constexpr uint32_t kNarrowNf = 4096;
constexpr uint64_t kNarrowMu = 1ull << 26;
constexpr int kNarrowBlock = 1024;
constexpr int kNarrowMaxCluster = 16;
constexpr uint32_t kNarrowCap = 4096;   // shared-memory frontier entries per buffer per CTA

struct LevelSlot {
  uint32_t qcount;         // queue entries of this level
  uint32_t ccount;         // chunk entries of this level
  uint32_t nf;             // vertices discovered into this level
  uint32_t scount;         // pull: vertices left unresolved, with in-edges
  unsigned long long mf;   // sum of their out-degrees
  uint32_t dcount;         // pull with the index: vertices it left to probe
  uint32_t fcount;         // pull over a queue: vertices found, queued from the top
};

struct Summary {
  uint32_t levels, bu_levels, switches, pad;
  unsigned long long nr, mr;
};

// Hand-over from the persistent kernel to bfs_narrow (control block).
struct Handover {
  uint32_t flag;              // 1: bfs_narrow continues the traversal
  uint32_t level;             // depth of the handed-over frontier
  uint32_t nf;                // its queue entries (queue[qsel])
  uint32_t qsel;
  unsigned long long nr, mr;  // reach counts so far
  uint32_t bu_levels, switches;
  uint32_t spill[3];          // spilled frontier entries, by depth mod 3
};

// Per-level record written by one thread after each level's barrier:
// entry 0 holds the kernel start time, entry L+1 the end of level L.
constexpr int kMaxTrace = 128;
struct LevelTrace {
  unsigned long long t_ns;
  unsigned long long mf;
  uint32_t nf, pull;
};

struct Args {
  const uint32_t *__restrict__ offs;   // out-edges (push levels)
  const uint32_t *__restrict__ cols;
  const uint32_t *__restrict__ ioffs;  // in-edges (pull levels): the CSR itself
  const uint32_t *__restrict__ icols;  // on a symmetric graph, else the CSC
  const uint2 *__restrict__ rep;       // pull index {rep, out-degree} (null: none), grus_graph::bfs_rep
  bool allow_pull;                     // false when no in-edge arrays exist
  uint32_t n, W;
  uint64_t m;
  uint32_t src;
  uint32_t *depth;
  // Depths as bit planes (null: depths are stored as vertices are found):
  // bit p of vertex v's depth is bit v of plane p (planes[p * Wp + v / 32]).
  // Setting bits in L2-resident words replaces scattered 4-byte stores into
  // the depth array, each a partial write of a sector in HBM; the depth
  // array is then written once, whole lines, when the traversal ends.
  uint32_t *planes;
  uint32_t Wp, nplanes;
  uint32_t *visited;      // W words; fronts follow contiguously
  uint32_t *aux;          // W words, with the pull index: the index pass's
                          // unresolved vertices of in-degree one
  uint32_t *front[3];
  uint32_t *queue[2];
  uint4 *chunks[2];
  uint32_t queue_cap, chunk_cap;
  LevelSlot *slots;       // 4 rotating slots
  GridBarrier *bar;
  uint32_t *err;
  Summary *summary;
  LevelTrace *trace;      // optional (null: no trace)
  float alpha, beta;
  uint32_t huge, bu_scan;
  uint32_t narrow_nf;     // hand over at most this many frontier vertices (0: never)
  Handover *ho;
  uint64_t timeout_ns;
};

// Depth bit planes from this many vertices on.  Below it the depth array
// stays in L2 (16 MB at 2^22 vertices), its partial-sector stores cost
// little, and the planes' extra pass and atomics do not repay: best of 12
// with the L2 flushed, stores against planes, RMAT scale 18 0.087 against
// 0.099 ms, 21 0.130 against 0.136, 22 0.160 against 0.158, 23 0.267
// against 0.211, 24 0.433 against 0.347.
constexpr uint64_t kPlanesMinN = 1ull << 22;

struct Workspace {
  uint64_t n = 0, m = 0;
  uint32_t W = 0;
  uint32_t *depth = nullptr;     // used when the caller's buffer is on the host
  uint32_t *bitmaps = nullptr;   // visited + 3 fronts + aux (+ depth planes), (5[+P])*Wp words
  size_t bitmap_bytes = 0;       // the part kept in the L2 persisting window
  uint32_t nplanes = 0;          // P: bits of the largest possible depth
  uint32_t *planes = nullptr;    // P*Wp words: after the fronts from kPlanesMinN
  uint32_t *planes_own = nullptr;  // vertices on, else allocated when first asked for
  uint32_t *queues = nullptr;    // 2 * n
  uint4 *chunks = nullptr;       // 2 * chunk_cap
  uint32_t chunk_cap = 0;
  char *ctrl = nullptr;          // slots, barrier, err, summary
  char *ctrl_host = nullptr;     // pinned mirror for readback
  LevelTrace *trace = nullptr;   // device per-level records
  LevelTrace *trace_host = nullptr;
  int trace_levels = 0;          // records valid in trace_host
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

constexpr size_t kOffSlots = 0, kOffBar = 256, kOffErr = 512, kOffSummary = 576,
                 kOffHandover = 640, kCtrlBytes = 768;
static_assert(kOffBar % 128 == 0 && kOffBar + sizeof(GridBarrier) <= kOffErr, "barrier layout");
static_assert(4 * sizeof(LevelSlot) <= kOffBar && sizeof(Summary) <= kOffHandover - kOffSummary,
              "control block layout");
static_assert(kOffHandover + sizeof(Handover) <= kCtrlBytes, "hand-over overflows the control block");

void ws_free(void *p) {
  Workspace *w = (Workspace *)p;
  if (!w) return;
  cudaFree(w->depth);
  cudaFree(w->bitmaps);
  cudaFree(w->planes_own);
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
  if (g->ws[kWsBfs]) {
    *out = (Workspace *)g->ws[kWsBfs];
    return GRUS_OK;
  }
  Workspace *w = new Workspace();
  w->n = g->n;
  w->m = g->m;
  w->W = (uint32_t)((g->n + 31) / 32);
  const uint64_t Wp = ((uint64_t)w->W + 31) / 32 * 32;  // 128-byte aligned maps
  // depths reach at most n - 1; the window covers the maps and the planes of
  // depths below 16
  uint32_t P = 1;
  while (P < 32 && (g->n >> P) != 0) ++P;
  w->nplanes = P;
  const bool with_planes = g->n >= kPlanesMinN;
  w->bitmap_bytes = (5 + (with_planes ? std::min<uint64_t>(P, 4) : 0)) * Wp * 4;
  // chunk lists sized for any chunking degree down to 256 (the autotuner and
  // callers may lower it after the workspace exists)
  const uint32_t huge = std::min(tune_or(g->tuning.huge_degree, kDefHuge), 256u);
  const uint64_t cap = g->m / kChunk + g->m / std::max(huge, 1u) + 2;
  w->chunk_cap = (uint32_t)std::min<uint64_t>(cap, 0x7FFFFFFFull);
  cudaError_t e = cudaMalloc(&w->bitmaps, (5 + (with_planes ? (uint64_t)P : 0)) * Wp * 4);
  if (e == cudaSuccess && with_planes) w->planes = w->bitmaps + 5 * Wp;
  if (e == cudaSuccess) e = cudaMalloc(&w->queues, 2 * std::max<uint64_t>(g->n, 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&w->chunks, 2ull * w->chunk_cap * sizeof(uint4));
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
    set_last_error(std::string("bfs workspace: ") + cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  g->ws[kWsBfs] = w;
  g->ws_free[kWsBfs] = ws_free;
  *out = w;
  return GRUS_OK;
}

// The representatives alone: word 2v of the index.
__device__ __forceinline__ const uint32_t *rep_ids(const Args &a) {
  return reinterpret_cast<const uint32_t *>(a.rep);
}

// Records depth nd for the vertices of `mask` in word w: one non-returning
// atomicOr per set bit of nd into the bit planes, else plain stores of nd.
__device__ __forceinline__ void mark_depth(const Args &a, uint32_t w, uint32_t mask, uint32_t nd) {
  uint32_t d = nd;
  for (uint32_t p = 0; d; ++p, d >>= 1)
    if (d & 1u) atomicOr(a.planes + (size_t)p * a.Wp + w, mask);
}

// Writes every vertex's depth from the bit planes of depths below 2^np and
// the visited bitmap (unreached: INFINIT).  A warp takes 32 consecutive
// words (1,024 vertices): lane j loads word j of the visited map and of each
// plane, one coalesced request per map, so a step waits for one L2 round
// trip.  Then, eight times, each lane takes four consecutive vertices (bits
// 4(j mod 8) .. +3 of word 4i + j/8, read from its owner lane by a shuffle)
// and stores their depths as one 16-byte word: 512 contiguous bytes per
// warp store.  Two slower forms measured at RMAT-24 (np = 3): lane = vertex
// with the planes read one after another, 1 + np round trips per 8 words
// (62 us); the same with all loads of a step issued together (71 us, the
// loads queued behind the stores).
template <int NP>
__device__ __forceinline__ void write_depths_np(const Args &a, uint32_t np) {
  const uint32_t lane = lane_id();
  const uint32_t gw = (blockIdx.x * kBlock + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * kBlock) >> 5;
  const bool vec = ((uintptr_t)a.depth & 15u) == 0;
  const uint32_t sh = 4 * (lane & 7u);
  for (uint32_t w0 = gw * 32; w0 < a.W; w0 += nw * 32) {
    const uint32_t w = w0 + lane;
    const bool ok = w < a.W;
    const uint32_t vis = ok ? __ldcg(a.visited + w) : 0u;
    uint32_t pw[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p)
      pw[p] = ok && (uint32_t)p < np ? __ldcg(a.planes + (size_t)p * a.Wp + w) : 0u;
#pragma unroll 2
    for (int i = 0; i < 8; ++i) {
      const int t = i * 4 + (int)(lane >> 3);
      const uint32_t vt = __shfl_sync(0xffffffffu, vis, t) >> sh;
      uint32_t nib[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) nib[p] = __shfl_sync(0xffffffffu, pw[p], t) >> sh;
      uint32_t o[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        uint32_t d = 0u;
#pragma unroll
        for (int p = 0; p < NP; ++p) d |= ((nib[p] >> e) & 1u) << p;
        o[e] = ((vt >> e) & 1u) ? d : kInfinit;
      }
      if (w0 + t >= a.W) continue;
      const uint64_t v0 = (uint64_t)(w0 + t) * 32 + sh;
      if (vec && v0 + 4 <= a.n) {
        *reinterpret_cast<uint4 *>(a.depth + v0) = make_uint4(o[0], o[1], o[2], o[3]);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (v0 + e < a.n) a.depth[v0 + e] = o[e];
      }
    }
  }
}

__device__ __noinline__ void write_depths(const Args &a, uint32_t np) {
  if (np <= 4) write_depths_np<4>(a, np);
  else if (np <= 8) write_depths_np<8>(a, np);
  else if (np <= 16) write_depths_np<16>(a, np);
  else {
    // depths of 65,536 and more: a word per warp step
    const uint32_t lane = lane_id();
    const uint32_t gw = (blockIdx.x * kBlock + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * kBlock) >> 5;
    for (uint32_t w = gw; w < a.W; w += nw) {
      const uint32_t vis = __ldcg(a.visited + w);
      uint32_t d = 0u;
      for (uint32_t p = 0; p < np; ++p)
        d |= ((__ldcg(a.planes + (size_t)p * a.Wp + w) >> lane) & 1u) << p;
      const uint32_t v = w * 32 + lane;
      if (v < a.n) a.depth[v] = ((vis >> lane) & 1u) ? d : kInfinit;
    }
  }
}

// ---------------------------------------------------------------------------
// push level: visitor for expand_binned (expand.cuh)
// ---------------------------------------------------------------------------
template <bool P>
struct PushVisitor {
  const Args *a;
  uint32_t nd;
  uint32_t *fnext, *qnext;
  uint4 *cnext;
  LevelSlot *nx;
  uint32_t nf;
  unsigned long long mf;

  using aux_t = uint32_t;

  __device__ __forceinline__ uint32_t aux(uint32_t) const { return 0u; }
  // Claim dst with one atomicOr on the visited bitmap; the winner writes the
  // depth, marks the next frontier and appends dst to the binned lists.
  __device__ __forceinline__ void edge(uint32_t, uint32_t, uint32_t x) {
    const uint32_t dst = __ldg(a->cols + x);
    const uint32_t w = dst >> 5, bit = 1u << (dst & 31u);
    // level 0 reaches only unvisited vertices (but the source), so there the
    // test before the claim is a wasted round trip (RMAT scales 16-24: 2-3 %)
    if (nd > 1 && (__ldcg(a->visited + w) & bit)) return;
    if (atomicOr(a->visited + w, bit) & bit) return;
    if (P) mark_depth(*a, w, bit, nd);
    else a->depth[dst] = nd;
    atomicOr(fnext + w, bit);
    const uint32_t b = __ldg(a->offs + dst), e = __ldg(a->offs + dst + 1);
    nf += 1;
    mf += e - b;
    if (!push_binned(dst, b, e, a->huge, qnext, &nx->qcount, a->queue_cap, cnext,
                     &nx->ccount, a->chunk_cap))
      atomicOr(a->err, kErrOverflow);
  }
};

__device__ __forceinline__ void enqueue_binned(const Args &a, uint32_t v,
                                               uint32_t *qnext, uint4 *cnext,
                                               LevelSlot *nx) {
  const uint32_t b = __ldg(a.offs + v), e = __ldg(a.offs + v + 1);
  if (!push_binned(v, b, e, a.huge, qnext, &nx->qcount, a.queue_cap, cnext, &nx->ccount,
                   a.chunk_cap))
    atomicOr(a.err, kErrOverflow);
}

// ---------------------------------------------------------------------------
// pull level
// ---------------------------------------------------------------------------
// A warp owns K consecutive bitmap words (32 vertices each) per
// step and interleaves their load chains (visited words, offsets, the first
// neighbours, their frontier bits) so several memory round trips are in
// flight per warp.  Each unvisited lane checks its first `bu_scan`
// in-neighbours, four at a time; lanes whose list is longer and still
// unresolved are then finished by the whole warp, 32 neighbours per ballot.
// Everything is warp-synchronous: no block barrier inside a pull level.
// Every unvisited vertex with in-edges that a pull level leaves unresolved
// is a survivor; together they are every vertex a later level can still
// reach, so the next pull level probes the survivors instead of every bitmap
// word (after the first pull level of RMAT-24, 0.85 M survivors against
// 16.7 M vertices, half of them isolated).  A pull level over bitmap words
// records its survivors as a bitmap (`sbm`, one plain store per word by the
// warp that owns it: a queue append per word would put one atomic per word
// on a single counter) and counts them in *scount.
template <int K, bool P>
__device__ __forceinline__ void bu_level(const Args &a, uint32_t L, const uint32_t *fcur,
                                         uint32_t *fnext, uint32_t &nf, unsigned long long &mf,
                                         uint32_t *sbm, uint32_t &ns) {
  const uint32_t nd = L + 1;
  const uint32_t lane = lane_id();
  const uint32_t scan = a.bu_scan;
  const uint32_t gw = (blockIdx.x * kBlock + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * kBlock) >> 5;
  for (uint32_t w0 = gw * K; w0 < a.W; w0 += nw * K) {
    uint32_t vis[K], b[K], e[K], lim[K];
    bool act[K], found[K];
#pragma unroll
    for (int k = 0; k < K; ++k) vis[k] = w0 + k < a.W ? __ldcg(a.visited + w0 + k) : 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const uint32_t v = (w0 + k) * 32 + lane;
      act[k] = !((vis[k] >> lane) & 1u) && v < a.n;
      found[k] = false;
      b[k] = e[k] = lim[k] = 0;
      if (act[k]) {
        b[k] = __ldg(a.ioffs + v);
        e[k] = __ldg(a.ioffs + v + 1);
        lim[k] = min(e[k], b[k] + scan);
      }
    }
    // with the pull index: the representative in-neighbour first (coalesced)
    if (a.rep) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const uint32_t v = (w0 + k) * 32 + lane;
        const uint32_t r = act[k] ? __ldg(rep_ids(a) + 2 * (size_t)v) : kNoRep;
        found[k] = r != kNoRep && test_bit(fcur, r);
      }
    }
    // probe rounds: four neighbours per word, K words at once
    for (uint32_t r = 0; r < scan; r += 4) {
      uint32_t u[K][4];
      bool any = false;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const uint32_t x = b[k] + r;
        const bool go = act[k] && !found[k] && x < lim[k];
        any |= go;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          u[k][j] = go && x + j < lim[k] ? __ldg(a.icols + x + j) : 0xFFFFFFFFu;
      }
      if (!__any_sync(0xffffffffu, any)) break;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        bool h = false;
#pragma unroll
        for (int j = 0; j < 4; ++j) h |= u[k][j] != 0xFFFFFFFFu && test_bit(fcur, u[k][j]);
        found[k] |= h;
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      uint32_t pending = __ballot_sync(0xffffffffu, act[k] && !found[k] && lim[k] < e[k]);
      while (pending) {
        const int j = __ffs(pending) - 1;
        pending &= pending - 1;
        const uint32_t jb = __shfl_sync(0xffffffffu, lim[k], j);
        const uint32_t je = __shfl_sync(0xffffffffu, e[k], j);
        for (uint32_t base = jb; base < je; base += 32) {
          const uint32_t x = base + lane;
          const bool h = x < je && test_bit(fcur, __ldg(a.icols + x));
          if (__ballot_sync(0xffffffffu, h)) {
            if ((int)lane == j) found[k] = true;
            break;
          }
        }
      }
      const uint32_t mask = __ballot_sync(0xffffffffu, found[k]);
      const uint32_t w = w0 + k, v = w * 32 + lane;
      if (mask) {
        if (lane == 0) {
          a.visited[w] = vis[k] | mask;
          fnext[w] = mask;
          if (P) mark_depth(a, w, mask, nd);
        }
        if (found[k]) {
          if (!P) a.depth[v] = nd;
          nf += 1;
          mf += __ldg(a.offs + v + 1) - __ldg(a.offs + v);
        }
      }
      const uint32_t smask = __ballot_sync(0xffffffffu, act[k] && !found[k] && b[k] < e[k]);
      if (lane == 0 && w < a.W) {
        sbm[w] = smask;
        ns += __popc(smask);
      }
    }
  }
}

// First pull level with the pull index (graphs in the planes form): each
// unvisited vertex tests only its representative in-neighbour (one
// coalesced 8-byte index entry and one frontier bit), so a warp step never
// waits on adjacency reads.  Of the vertices it leaves unresolved, those of
// in-degree one on a symmetric graph are next level's survivors already
// (their one in-neighbour is the representative) and are marked in
// `a.aux`; the others are marked in `dbm` (one plain store per word by the
// warp that owns it) and probed afterwards from a dense queue by
// bu_level_survivors: with the probes of the few unresolved lanes removed
// from the word pass, its steps no longer wait on the adjacency reads of one
// or two lanes each.
template <int K, bool P>
__device__ __forceinline__ void bu_level_rep(const Args &a, uint32_t L, const uint32_t *fcur,
                                             uint32_t *fnext, uint32_t &nf, unsigned long long &mf,
                                             uint32_t *dbm) {
  const uint32_t nd = L + 1;
  // in-degree = out-degree on a symmetric graph (in-edges are the CSR)
  const bool sym = a.ioffs == a.offs;
  const uint32_t lane = lane_id();
  const uint32_t gw = (blockIdx.x * kBlock + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * kBlock) >> 5;
  for (uint32_t w0 = gw * K; w0 < a.W; w0 += nw * K) {
    uint32_t vis[K], r[K], dg[K];
#pragma unroll
    for (int k = 0; k < K; ++k) vis[k] = w0 + k < a.W ? __ldcg(a.visited + w0 + k) : 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const uint32_t v = (w0 + k) * 32 + lane;
      const bool act = !((vis[k] >> lane) & 1u) && v < a.n;
      if constexpr (P) {
        const uint2 rd = act ? __ldg(a.rep + v) : make_uint2(kNoRep, 0u);
        r[k] = rd.x;
        dg[k] = rd.y;
      } else {
        // graphs below the planes threshold: this form keeps the stores
        // kernel free of spills (the index entry's degree is not used)
        r[k] = act ? __ldg(rep_ids(a) + 2 * (size_t)v) : kNoRep;
        dg[k] = act ? __ldg(a.offs + v + 1) - __ldg(a.offs + v) : 0u;
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const bool found = r[k] != kNoRep && test_bit(fcur, r[k]);
      const uint32_t mask = __ballot_sync(0xffffffffu, found);
      // a vertex whose one in-neighbour is its representative is resolved:
      // it survives to the next level without a probe
      const bool unres = r[k] != kNoRep && !found;
      const bool one = sym && dg[k] == 1u;
      const uint32_t dmask = __ballot_sync(0xffffffffu, unres && !one);
      const uint32_t smask = __ballot_sync(0xffffffffu, unres && one);
      const uint32_t w = w0 + k, v = w * 32 + lane;
      if (found) {
        if (!P) a.depth[v] = nd;
        nf += 1;
        mf += dg[k];
      }
      if (lane == 0 && w < a.W) {
        if (mask) {
          a.visited[w] = vis[k] | mask;
          fnext[w] = mask;
          if (P) mark_depth(a, w, mask, nd);
        }
        dbm[w] = dmask;
        a.aux[w] = smask;
      }
    }
  }
}

// A pull level over the survivors of the previous one (a queue): lane i of a
// warp step takes K survivors (entries i, i + 32, ...) with their load chains
// interleaved, as bu_level does for K words; the vertices of one bitmap word
// are spread over warps, so found ones set their bits with atomics.  Those
// still unresolved are appended to the next survivor queue, one reservation
// per warp step.
template <int K, bool P>
__device__ __forceinline__ void bu_level_survivors(const Args &a, uint32_t L, const uint32_t *fcur,
                                                   uint32_t *fnext, const uint32_t *sin,
                                                   uint32_t S, uint32_t &nf, unsigned long long &mf,
                                                   uint32_t *sq, uint32_t *scount,
                                                   uint32_t *fcount, bool use_rep = true) {
  const uint32_t nd = L + 1;
  const uint32_t lane = lane_id();
  const uint32_t scan = a.bu_scan;
  const uint32_t gw = (blockIdx.x * kBlock + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * kBlock) >> 5;
  for (uint32_t i0 = gw * 32 * K; i0 < S; i0 += nw * 32 * K) {
    uint32_t v[K], b[K], e[K], lim[K];
    bool act[K], found[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const uint32_t i = i0 + k * 32 + lane;
      act[k] = i < S;
      v[k] = act[k] ? __ldcg(sin + i) : 0u;
    }
    const bool idx = use_rep && a.rep;
    // P (big graphs): a vertex the index settles adds its out-degree from its
    // entry here, and only the others read their offsets (a random vertex's
    // offsets are one more sector from HBM); one found by a probe reads its
    // out-degree below.  Otherwise offsets and representative load together.
    const bool early_mf = P && idx;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      found[k] = false;
      b[k] = e[k] = lim[k] = 0;
      if constexpr (P) {
        if (idx && act[k]) {
          const uint2 rd = __ldg(a.rep + v[k]);
          found[k] = rd.x != kNoRep && test_bit(fcur, rd.x);
          if (found[k]) mf += rd.y;
        }
      } else {
        uint32_t r = kNoRep;
        if (act[k]) {
          b[k] = __ldg(a.ioffs + v[k]);
          e[k] = __ldg(a.ioffs + v[k] + 1);
          lim[k] = min(e[k], b[k] + scan);
          if (idx) r = __ldg(rep_ids(a) + 2 * (size_t)v[k]);
        }
        found[k] = r != kNoRep && test_bit(fcur, r);
      }
    }
    if constexpr (P) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (act[k] && !found[k]) {
          b[k] = __ldg(a.ioffs + v[k]);
          e[k] = __ldg(a.ioffs + v[k] + 1);
          lim[k] = min(e[k], b[k] + scan);
        }
      }
    }
    for (uint32_t r = 0; r < scan; r += 4) {
      uint32_t u[K][4];
      bool any = false;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const uint32_t x = b[k] + r;
        const bool go = act[k] && !found[k] && x < lim[k];
        any |= go;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          u[k][j] = go && x + j < lim[k] ? __ldg(a.icols + x + j) : 0xFFFFFFFFu;
      }
      if (!__any_sync(0xffffffffu, any)) break;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        bool h = false;
#pragma unroll
        for (int j = 0; j < 4; ++j) h |= u[k][j] != 0xFFFFFFFFu && test_bit(fcur, u[k][j]);
        found[k] |= h;
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      uint32_t pending = __ballot_sync(0xffffffffu, act[k] && !found[k] && lim[k] < e[k]);
      while (pending) {
        const int j = __ffs(pending) - 1;
        pending &= pending - 1;
        const uint32_t jb = __shfl_sync(0xffffffffu, lim[k], j);
        const uint32_t je = __shfl_sync(0xffffffffu, e[k], j);
        for (uint32_t base = jb; base < je; base += 32) {
          const uint32_t x = base + lane;
          const bool h = x < je && test_bit(fcur, __ldg(a.icols + x));
          if (__ballot_sync(0xffffffffu, h)) {
            if ((int)lane == j) found[k] = true;
            break;
          }
        }
      }
      if (found[k]) {
        const uint32_t w = v[k] >> 5, bit = 1u << (v[k] & 31u);
        // probed (b < e): the index did not settle it
        atomicOr(a.visited + w, bit);
        atomicOr(fnext + w, bit);
        if (P) mark_depth(a, w, bit, nd);
        else a.depth[v[k]] = nd;
        nf += 1;
        if (!early_mf || b[k] < e[k]) mf += __ldg(a.offs + v[k] + 1) - __ldg(a.offs + v[k]);
      }
    }
    uint32_t m[K], tot = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      m[k] = __ballot_sync(0xffffffffu, act[k] && !found[k]);
      tot += __popc(m[k]);
    }
    if (tot) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(scount, tot);
      base = __shfl_sync(0xffffffffu, base, 0);
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if ((m[k] >> lane) & 1u) {
          const uint32_t at = base + __popc(m[k] & ((1u << lane) - 1u));
          if (at < a.queue_cap) sq[at] = v[k];
          else atomicOr(a.err, kErrOverflow);
        }
        base += __popc(m[k]);
      }
    }
    // the vertices found, from the top of the same queue downwards: every
    // vertex this level finds comes through here, so a push level next reads
    // them from there instead of converting the frontier bitmap
    if (fcount) {
      tot = 0;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        m[k] = __ballot_sync(0xffffffffu, act[k] && found[k]);
        tot += __popc(m[k]);
      }
      if (tot) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(fcount, tot);
        base = __shfl_sync(0xffffffffu, base, 0);
#pragma unroll
        for (int k = 0; k < K; ++k) {
          if ((m[k] >> lane) & 1u) {
            const uint32_t at = base + __popc(m[k] & ((1u << lane) - 1u));
            if (at < a.queue_cap) sq[a.queue_cap - 1 - at] = v[k];
          }
          base += __popc(m[k]);
        }
      }
    }
  }
}

// First push level after a pull level: its frontier exists only as the
// bitmap `fmap`.  Each CTA owns a contiguous range of words, loads them
// coalesced and reserves queue space with ONE atomicAdd per 256 words (a
// block scan of the popcounts places every thread's vertices), so the
// conversion is a bandwidth pass over n/8 bytes, not a per-vertex atomic
// storm.  Degrees are not read here: the expansion's CTA mapping takes any
// degree.
__device__ __forceinline__ void bitmap_to_queue(const Args &a, uint32_t *fmap, uint32_t *q,
                                                uint32_t *qcount, bool clear = false) {
  __shared__ uint32_t s_base;
  const uint32_t per = (a.W + gridDim.x - 1) / gridDim.x;
  const uint32_t w0 = blockIdx.x * per, w1 = min(a.W, w0 + per);
  for (uint32_t base = w0; base < w1; base += kBlock) {
    const uint32_t w = base + threadIdx.x;
    uint32_t word = w < w1 ? __ldcg(fmap + w) : 0u;
    if (clear && word) fmap[w] = 0u;
    uint32_t total = 0;
    uint32_t at = block_exclusive_scan<kBlock>(__popc(word), &total);
    if (threadIdx.x == 0 && total) s_base = atomicAdd(qcount, total);
    __syncthreads();
    if (!total) continue;
    at += s_base;
    while (word) {
      const int bit = __ffs(word) - 1;
      word &= word - 1;
      if (at < a.queue_cap) q[at] = w * 32 + bit;
      ++at;
    }
  }
}

// bitmap_to_queue over two maps at once, one block scan of both counts
// (packed in 16-bit halves: at most 256 x 32 per block): m1 is cleared as it
// is read, m2 is left as it is.
__device__ __forceinline__ void bitmaps_to_queues(const Args &a, uint32_t *m1, uint32_t *q1,
                                                  uint32_t *c1, const uint32_t *m2, uint32_t *q2,
                                                  uint32_t *c2) {
  __shared__ uint32_t s_base[2];
  const uint32_t per = (a.W + gridDim.x - 1) / gridDim.x;
  const uint32_t w0 = blockIdx.x * per, w1 = min(a.W, w0 + per);
  for (uint32_t base = w0; base < w1; base += kBlock) {
    const uint32_t w = base + threadIdx.x;
    uint32_t x1 = w < w1 ? __ldcg(m1 + w) : 0u;
    uint32_t x2 = w < w1 ? __ldcg(m2 + w) : 0u;
    if (x1) m1[w] = 0u;
    uint32_t total = 0;
    const uint32_t at = block_exclusive_scan<kBlock>(__popc(x1) | (__popc(x2) << 16), &total);
    if (threadIdx.x == 0) {
      if (total & 0xFFFFu) s_base[0] = atomicAdd(c1, total & 0xFFFFu);
      if (total >> 16) s_base[1] = atomicAdd(c2, total >> 16);
    }
    __syncthreads();
    if (!total) continue;
    uint32_t at1 = s_base[0] + (at & 0xFFFFu), at2 = s_base[1] + (at >> 16);
    while (x1) {
      const int bit = __ffs(x1) - 1;
      x1 &= x1 - 1;
      if (at1 < a.queue_cap) q1[at1] = w * 32 + bit;
      ++at1;
    }
    while (x2) {
      const int bit = __ffs(x2) - 1;
      x2 &= x2 - 1;
      if (at2 < a.queue_cap) q2[at2] = w * 32 + bit;
      ++at2;
    }
  }
}

// P: depths as bit planes (Args::planes set) or stored as vertices are found
template <int K, bool P>
__global__ void __launch_bounds__(kBlock) bfs_persistent(Args a) {
  const uint32_t gtid = blockIdx.x * kBlock + threadIdx.x;
  const uint32_t nthreads = gridDim.x * kBlock;
  if (gtid == 0 && a.trace) a.trace[0] = LevelTrace{global_timer_ns(), 0ull, 1u, 0u};
  // prologue: clear the bitmaps and the level slots, and seed the source as
  // the clearing goes (its visited and frontier bits, and level 0's work in
  // slot 0: one queue entry, or its chunks written by as many threads, as
  // push_binned bins it), so one grid barrier ends the prologue
  const uint32_t sb = __ldg(a.offs + a.src), se = __ldg(a.offs + a.src + 1);
  {
    const uint32_t sw = a.src >> 5, sbit = 1u << (a.src & 31u);
    const uint32_t fw = (uint32_t)(a.front[0] - a.visited) + sw;
    const uint32_t d = se - sb;
    const bool chunked = d >= a.huge;
    const uint32_t nch = chunked ? (d + kChunk - 1) / kChunk : 0u;
    uint32_t *bm = a.visited;
    const uint32_t words = (uint32_t)(a.front[2] - a.visited) + a.W;
    for (uint32_t i = gtid; i < words; i += nthreads) bm[i] = (i == sw || i == fw) ? sbit : 0u;
    if (P)
      for (uint32_t i = gtid; i < a.W; i += nthreads) a.planes[i] = 0u;
    if (gtid < 4 * sizeof(LevelSlot) / 4) {
      uint32_t val = 0u;
      if (gtid == offsetof(LevelSlot, qcount) / 4 && d > 0 && !chunked) val = 1u;
      if (gtid == offsetof(LevelSlot, ccount) / 4 && chunked && nch <= a.chunk_cap) val = nch;
      ((uint32_t *)a.slots)[gtid] = val;
    }
    if (chunked) {
      if (nch > a.chunk_cap) {
        if (gtid == 0) atomicOr(a.err, kErrOverflow);
      } else {
        for (uint32_t c = gtid; c < nch; c += nthreads)
          a.chunks[0][c] = make_uint4(a.src, sb + c * kChunk, min(se, sb + (c + 1) * kChunk), 0u);
      }
    }
    if (gtid == 0) {
      if (a.ho) a.ho->flag = 0u;
      if (!P) a.depth[a.src] = 0;
      if (d > 0 && !chunked) a.queue[0][0] = a.src;
    }
  }
  if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;

  uint32_t L = 0;
  bool bu = false, from_pull = false;
  bool fq = false;  // the previous level queued every vertex it found (pull over a queue)
  // Survivors of the previous pull level: 0 none, 1 a bitmap in the words
  // this level writes as its next frontier (cleared before use), 2 a queue in
  // queue[L & 1] of S entries.
  int surv = 0;
  uint32_t S = 0;
  uint64_t mu = a.m - (uint64_t)(se - sb);
  uint32_t prev_nf = 1, bu_levels = 0, switches = 0;
  unsigned long long nr = 1, mr = se - sb;
  while (true) {
    LevelSlot *cur = a.slots + (L & 3u);
    LevelSlot *nx = a.slots + ((L + 1) & 3u);
    uint32_t *fcur = a.front[L % 3];
    uint32_t *fnext = a.front[(L + 1) % 3];
    uint32_t *fclr = a.front[(L + 2) % 3];
    // a pull level over bitmap words writes every word of fclr (its survivors)
    if (!(bu && surv == 0))
      for (uint32_t i = gtid; i < a.W; i += nthreads) fclr[i] = 0u;
    // plane p is first written at level 2^p - 1 (depth 2^p): clear it now
    if (P && ((L + 2) & (L + 1)) == 0) {
      const uint32_t p = 31 - __clz(L + 2);
      if (p < a.nplanes) {
        uint32_t *pl = a.planes + (size_t)p * a.Wp;
        for (uint32_t i = gtid; i < a.W; i += nthreads) pl[i] = 0u;
      }
    }
    if (gtid < sizeof(LevelSlot) / 4) ((uint32_t *)(a.slots + ((L + 2) & 3u)))[gtid] = 0u;
    uint32_t nf = 0;
    unsigned long long mf = 0;
    bool qpass = false;  // this pull level ran over a queue only
    if (!bu) {
      PushVisitor<P> vis{&a, L + 1, fnext, a.queue[(L + 1) & 1u], a.chunks[(L + 1) & 1u], nx, 0u, 0ull};
      const uint32_t *q = a.queue[L & 1u];
      uint32_t qc;
      if (from_pull && fq) {
        // the pull level queued what it found at the top of this queue
        qc = min(__ldcg(&cur->fcount), a.queue_cap);
        q += a.queue_cap - qc;
      } else {
        if (from_pull) {
          bitmap_to_queue(a, fcur, a.queue[L & 1u], &cur->qcount);
          // survivors recorded as a bitmap sit in this level's next frontier
          if (surv == 1)
            for (uint32_t i = gtid; i < a.W; i += nthreads) fnext[i] = 0u;
          if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
        }
        qc = min(__ldcg(&cur->qcount), a.queue_cap);
      }
      const uint32_t cc = min(__ldcg(&cur->ccount), a.chunk_cap);
      expand_binned<kBlock>(a.offs, q, qc, a.chunks[L & 1u], cc, vis);
      nf = vis.nf;
      mf = vis.mf;
    } else {
      // the two-pass form with the index on big graphs (the planes form);
      // below that the word pass tests the representative itself: at RMAT
      // scales 16-20 its barrier and conversion cost more than they save
      if (surv == 0 && a.rep && P) {
        // the index pass over the words, then the vertices it left as a
        // queue (their bitmap in fclr, cleared as it is read)
        // twice the words per warp step of the probing passes: this pass
        // holds four registers per word (RMAT-24: 8 words 85 us, 4 words
        // 110 us, 12 or 16 words 142 us)
        bu_level_rep<2 * K, P>(a, L, fcur, fnext, nf, mf, fclr);
        if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
        // the vertices to probe as this level's queue; those of in-degree
        // one start the next level's survivor queue, which the probe pass
        // appends to
        bitmaps_to_queues(a, fclr, a.queue[L & 1u], &nx->dcount, a.aux, a.queue[(L + 1) & 1u],
                          &nx->scount);
        if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
        const uint32_t D = min(__ldcg(&nx->dcount), a.queue_cap);
        bu_level_survivors<K, P>(a, L, fcur, fnext, a.queue[L & 1u], D, nf, mf,
                              a.queue[(L + 1) & 1u], &nx->scount, nullptr, false);
      } else if (surv == 0) {
        uint32_t ns = 0;
        bu_level<K, P>(a, L, fcur, fnext, nf, mf, fclr, ns);
        const unsigned long long bns = block_sum_u64<kBlock>(ns);
        if (threadIdx.x == 0 && bns) atomicAdd(&nx->scount, (uint32_t)bns);
      } else {
        if (surv == 1) {
          // the survivor bitmap (this level's next frontier) becomes a queue
          // and is cleared as it is read
          bitmap_to_queue(a, fnext, a.queue[L & 1u], &cur->qcount, true);
          if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
          S = min(__ldcg(&cur->qcount), a.queue_cap);
        }
        // half the entries per lane of the other passes: twice the warp
        // steps over a queue of about 1.4 steps per warp, so fewer warps idle
        // for a whole step (RMAT scale 20 0.103 -> 0.097 ms, 22 0.144 ->
        // 0.138, 24 unchanged)
        bu_level_survivors<(K > 1 ? K / 2 : 1), P>(a, L, fcur, fnext, a.queue[L & 1u], S, nf, mf,
                                                  a.queue[(L + 1) & 1u], &nx->scount, &nx->fcount);
        qpass = true;
      }
    }
    const unsigned long long bnf = block_sum_u64<kBlock>(nf);
    const unsigned long long bmf = block_sum_u64<kBlock>(mf);
    if (threadIdx.x == 0 && bnf) {
      atomicAdd(&nx->nf, (uint32_t)bnf);
      atomicAdd(&nx->mf, bmf);
    }
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    const uint32_t NF = __ldcg(&nx->nf);
    const unsigned long long MF = __ldcg(&nx->mf);
    if (gtid == 0 && a.trace && L + 1 < (uint32_t)kMaxTrace)
      a.trace[L + 1] = LevelTrace{global_timer_ns(), MF, NF, bu ? 1u : 0u};
    if (bu) ++bu_levels;
    if (NF == 0) break;
    nr += NF;
    mr += MF;
    mu = mu > MF ? mu - MF : 0;
    bool nbu = bu;
    const uint32_t SN = bu ? min(__ldcg(&nx->scount), a.queue_cap) : 0u;
    if (!bu) {
      // push -> pull while the frontier grows and its edges outweigh m_u/alpha
      if (a.allow_pull && NF > prev_nf && (double)MF * a.alpha > (double)mu) nbu = true;
    } else if (SN > MF) {
      // more unresolved vertices than frontier out-edges: pushing is cheaper
      // once the frontier has shrunk enough
      if ((double)NF * a.beta < (double)a.n && NF < prev_nf) nbu = false;
    }
    if (a.narrow_nf && !bu && !nbu && L + 1 >= kNarrowAfter && NF <= a.narrow_nf &&
        MF <= 16ull * a.narrow_nf && mu <= kNarrowMu && __ldcg(&nx->ccount) == 0) {
      // A long traversal down to a small push frontier: every further level
      // would be a grid barrier for a few thousand vertices.  Hand over to
      // bfs_narrow (launched after this kernel).  Vertices unreached so far
      // read INFINIT now; the narrow kernel writes the depth of each vertex it
      // reaches later.
      if (P) {
        write_depths(a, 32 - __clz(L + 1));
      } else {
        const uint32_t lane = lane_id();
        const uint32_t gw = gtid >> 5, nw = nthreads >> 5;
        for (uint32_t w = gw; w < a.W; w += nw) {
          const uint32_t vis = __ldcg(a.visited + w);
          const uint32_t v = w * 32 + lane;
          if (!((vis >> lane) & 1u) && v < a.n) a.depth[v] = kInfinit;
        }
      }
      if (gtid == 0) {
        Handover *h = a.ho;
        h->level = L + 1;
        h->nf = min(__ldcg(&nx->qcount), a.queue_cap);
        h->qsel = (L + 1) & 1u;
        h->nr = nr;
        h->mr = mr;
        h->bu_levels = bu_levels;
        h->switches = switches;
        __threadfence();
        h->flag = 1u;
      }
      return;
    }
    from_pull = bu && !nbu;
    fq = bu && qpass;
    // a push level after a word-based pull level still clears the bitmap
    surv = !bu ? 0 : (surv == 0 && !(a.rep && P) ? 1 : 2);
    if (!nbu && surv == 2) surv = 0;
    S = SN;
    if (nbu != bu) ++switches;
    bu = nbu;
    prev_nf = NF;
    ++L;
    if (L >= a.n + 1) {
      if (gtid == 0) atomicOr(a.err, kErrLevels);
      break;
    }
  }
  // epilogue: every depth from the planes, or INFINIT for unreached vertices
  if (P) {
    write_depths(a, 32 - __clz(L));
  } else {
    const uint32_t lane = lane_id();
    const uint32_t gw = gtid >> 5, nw = nthreads >> 5;
    for (uint32_t w = gw; w < a.W; w += nw) {
      const uint32_t vis = __ldcg(a.visited + w);
      const uint32_t v = w * 32 + lane;
      if (!((vis >> lane) & 1u) && v < a.n) a.depth[v] = kInfinit;
    }
  }
  if (gtid == 0) {
    a.summary->levels = L + 1;
    a.summary->bu_levels = bu_levels;
    a.summary->switches = switches;
    a.summary->nr = nr;
    a.summary->mr = mr;
  }
}

// Starts filling this SM's L1 (or only L2) with the line holding p (no wait).
__device__ __forceinline__ void prefetch_l1(const void *p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}
__device__ __forceinline__ void prefetch_l2(const void *p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Per-level state of the tail cluster.  Every frontier vertex has an owner
// CTA (a hash of its id); the owner keeps it as the (begin, end) range of its
// out-edges in shared memory, or -- beyond kNarrowCap entries -- the vertex id
// goes to a global spill list shared by the cluster.
struct Tail {
  cg::cluster_group cl;
  uint32_t rank, C;
  uint2 *q;            // this CTA's 2 * kNarrowCap entries
  uint32_t *cnt;       // this CTA's 2 entry counters
  uint32_t *found;     // this CTA's flag: it found a vertex at this level
};

__device__ __forceinline__ uint32_t tail_owner(uint32_t v, uint32_t C) {
  return __umulhi(v * 2654435761u, C);
}

// Claims up to kNarrowBatch targets at once.  The chain per batch is short:
// the column ids come from L1 (their lines were prefetched), the claiming
// atomicOr goes to L2 while the targets' offsets are prefetched, and a new
// vertex's offsets then come from L1.  A new vertex gets depth d and, if it
// has out-edges, a place in its owner's next frontier and a prefetch of its
// first out-edges.
constexpr int kNarrowBatch = 4;

__device__ __forceinline__ void narrow_batch(const Args &a, Tail &t,
                                             const uint32_t (&xs)[kNarrowBatch], int cnt,
                                             uint32_t d, uint32_t nxt, unsigned long long &nr,
                                             unsigned long long &mr) {
  uint32_t c[kNarrowBatch], old[kNarrowBatch];
#pragma unroll
  for (int r = 0; r < kNarrowBatch; ++r) c[r] = r < cnt ? __ldg(a.cols + xs[r]) : 0u;
#pragma unroll
  for (int r = 0; r < kNarrowBatch; ++r)
    if (r < cnt) prefetch_l1(a.offs + c[r]);
#pragma unroll
  for (int r = 0; r < kNarrowBatch; ++r) {
    const uint32_t bit = 1u << (c[r] & 31u);
    old[r] = r < cnt ? atomicOr(a.visited + (c[r] >> 5), bit) : bit;
  }
#pragma unroll
  for (int r = 0; r < kNarrowBatch; ++r) {
    if (old[r] & (1u << (c[r] & 31u))) continue;
    const uint32_t v = c[r];
    a.depth[v] = d;
    const uint32_t cb = __ldg(a.offs + v), ce = __ldg(a.offs + v + 1);
    ++nr;
    mr += ce - cb;
    *t.found = 1u;
    if (ce == cb) continue;
    const uint32_t o = tail_owner(v, t.C);
    if (o == t.rank) {
      prefetch_l1(a.cols + cb);
      prefetch_l1(a.cols + ce - 1);
    } else {
      prefetch_l2(a.cols + cb);
      prefetch_l2(a.cols + ce - 1);
    }
    // one reservation per owner among the lanes pushing together
    cg::coalesced_group pg = cg::coalesced_threads();
    cg::coalesced_group peers = cg::labeled_partition(pg, o);
    uint32_t base = 0;
    if (peers.thread_rank() == 0) base = atomicAdd(t.cl.map_shared_rank(t.cnt + nxt, o), peers.size());
    const uint32_t pos = peers.shfl(base, 0) + peers.thread_rank();
    if (pos < kNarrowCap) {
      t.cl.map_shared_rank(t.q, o)[nxt * kNarrowCap + pos] = make_uint2(cb, ce);
    } else {
      const uint32_t g = atomicAdd(&a.ho->spill[d % 3], 1u);
      if (g < a.queue_cap) a.queue[d & 1u][g] = v;
      else atomicOr(a.err, kErrOverflow);  // cannot happen: spilled vertices are distinct
    }
  }
}

// The narrow tail of a long traversal: one cluster of C CTAs (1 <= C <= 16)
// of 1024 threads takes the small frontier the persistent kernel handed over
// and runs the remaining levels with one hardware cluster barrier per level.
// Each CTA deals the edges of the frontier vertices it owns evenly to its
// threads (a block scan of the degrees and a binary search for each thread's
// first entry), so a wide vertex is shared by many threads, and each thread
// claims its edges in batches; spilled entries are dealt over the whole
// cluster one vertex per thread.  A CTA that found a vertex writes the new
// depth into every CTA's stamp before the level's barrier, so after it each
// CTA reads its own stamp; stamps only grow, so no CTA has to clear them.
// Returns at once when the persistent kernel finished the traversal itself.
__global__ void __launch_bounds__(kNarrowBlock) bfs_narrow(Args a) {
  extern __shared__ uint2 s_q[];  // 2 * kNarrowCap entries
  __shared__ uint32_t s_pref[kNarrowCap + 1];
  __shared__ uint32_t s_cnt[2], s_found, s_stamp;
  __shared__ unsigned long long s_red[kNarrowBlock / 32];
  Handover *ho = a.ho;
  if (__ldcg(&ho->flag) != 1u) return;  // the same answer in every CTA
  Tail t{cg::this_cluster(), 0, 1, s_q, s_cnt, &s_found};
  t.rank = t.cl.block_rank();
  t.C = t.cl.num_blocks();
  const uint32_t tid = threadIdx.x;
  uint32_t d = __ldcg(&ho->level);  // depth of the current frontier
  const uint32_t d0 = d;
  const uint32_t nf0 = __ldcg(&ho->nf);
  const uint32_t *q0 = a.queue[__ldcg(&ho->qsel)];
  if (tid == 0) {
    s_cnt[0] = 0;
    s_cnt[1] = 0;
    s_found = 0;
    s_stamp = d;
    if (t.rank == 0) {
      ho->spill[d % 3] = 0u;  // the counters of depths d0 and d0 + 1
      ho->spill[(d + 1) % 3] = 0u;
      a.summary->nr = __ldcg(&ho->nr);
      a.summary->mr = __ldcg(&ho->mr);
      if (a.trace && d + 1 < (uint32_t)kMaxTrace) a.trace[d + 1] = LevelTrace{0ull, 0ull, 0u, 0u};
    }
  }
  __syncthreads();
  // this CTA's share of the handed-over queue (vertex ids) becomes ranges in
  // buffer 0; vertices without out-edges are left out, so every entry has at
  // least one edge, which the edge dealing relies on
  for (uint32_t i = t.rank + t.C * tid; i < nf0; i += t.C * kNarrowBlock) {
    const uint32_t v = __ldcg(q0 + i);
    const uint2 r = make_uint2(__ldg(a.offs + v), __ldg(a.offs + v + 1));
    if (r.x == r.y) continue;
    const uint32_t pos = atomicAdd(&s_cnt[0], 1u);
    if (pos < kNarrowCap) s_q[pos] = r;
    else atomicOr(a.err, kErrOverflow);  // cannot happen: nf0 <= C * kNarrowCap
  }
  t.cl.sync();  // every CTA's counters are set before any remote push
  unsigned long long nr = 0, mr = 0;
  uint32_t cur = 0, levels = 0;
  constexpr uint32_t kPer = (kNarrowCap + kNarrowBlock - 1) / kNarrowBlock;
  while (true) {
    const uint32_t nxt = cur ^ 1u;
    const uint32_t in_smem = min(s_cnt[cur], kNarrowCap);
    // entries spilled into the frontier at depth d
    const uint32_t spilled = min(__ldcg(&ho->spill[d % 3]), a.queue_cap);
    const uint2 *qc = s_q + cur * kNarrowCap;
    // exclusive prefix of the entries' degrees; the first line of each
    // entry's adjacency is pulled into L1 meanwhile
    const uint32_t e0 = tid * kPer;
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < kPer; ++k)
      if (e0 + k < in_smem) {
        const uint2 r = qc[e0 + k];
        prefetch_l1(a.cols + r.x);
        sum += r.y - r.x;
      }
    uint32_t E = 0;
    uint32_t run = block_exclusive_scan<kNarrowBlock>(sum, &E);
#pragma unroll
    for (uint32_t k = 0; k < kPer; ++k)
      if (e0 + k < in_smem) {
        s_pref[e0 + k] = run;
        run += qc[e0 + k].y - qc[e0 + k].x;
      }
    if (tid == 0) {
      s_pref[in_smem] = E;
      // the spill counter for depth d + 2 is reused: its last readers
      // finished before the previous cluster barrier
      if (t.rank == 0) {
        ho->spill[(d + 2) % 3] = 0u;
        if (a.trace && d + 2 < (uint32_t)kMaxTrace) a.trace[d + 2] = LevelTrace{0ull, 0ull, 0u, 0u};
      }
      if (a.trace && d + 1 < (uint32_t)kMaxTrace) {
        atomicAdd(&a.trace[d + 1].mf, (unsigned long long)E);
        atomicAdd(&a.trace[d + 1].nf, in_smem);
      }
    }
    __syncthreads();
    if (tid == 0) s_cnt[cur] = 0;  // read by every thread above; refilled next level
    // this thread's edges [lo, hi) of the E in shared-memory entries
    const uint32_t lo = (uint32_t)((unsigned long long)tid * E / kNarrowBlock);
    const uint32_t hi = (uint32_t)((unsigned long long)(tid + 1) * E / kNarrowBlock);
    if (lo < hi) {
      uint32_t j = 0, span = in_smem;  // largest j with s_pref[j] <= lo
      while (span > 1) {
        const uint32_t half = span / 2;
        if (s_pref[j + half] <= lo) j += half;
        span -= half;
      }
      uint32_t x = qc[j].x + (lo - s_pref[j]);
      uint32_t xe = qc[j].y;
      for (uint32_t k = lo; k < hi; k += kNarrowBatch) {
        const int cnt = (int)min(hi - k, (uint32_t)kNarrowBatch);
        uint32_t xs[kNarrowBatch];
#pragma unroll
        for (int r = 0; r < kNarrowBatch; ++r) {
          xs[r] = x;
          if (r < cnt && ++x == xe && k + r + 1 < hi) {
            ++j;
            x = qc[j].x;
            xe = qc[j].y;
          }
        }
        narrow_batch(a, t, xs, cnt, d + 1, nxt, nr, mr);
      }
    }
    // spilled entries (rare: a frontier beyond C * kNarrowCap), one vertex
    // per thread over the whole cluster
    if (spilled) {
      const uint32_t *sp = a.queue[d & 1u];
      for (uint32_t i = t.rank * kNarrowBlock + tid; i < spilled; i += t.C * kNarrowBlock) {
        const uint32_t v = __ldcg(sp + i);
        const uint32_t b = __ldg(a.offs + v), e = __ldg(a.offs + v + 1);
        for (uint32_t x = b; x < e; x += kNarrowBatch) {
          const int cnt = (int)min(e - x, (uint32_t)kNarrowBatch);
          uint32_t xs[kNarrowBatch];
#pragma unroll
          for (int r = 0; r < kNarrowBatch; ++r) xs[r] = x + r;
          narrow_batch(a, t, xs, cnt, d + 1, nxt, nr, mr);
        }
      }
    }
    __syncthreads();
    if (tid < t.C && s_found) *t.cl.map_shared_rank(&s_stamp, tid) = d + 1;
    // every push and stamp of this level is visible after the barrier
    t.cl.sync();
    if (tid == 0) s_found = 0;  // set again at the next level, after its scan barriers
    const bool found = s_stamp > d;  // stamps only grow: a faster CTA may already write d + 2
    if (t.rank == 0 && tid == 0 && a.trace && d + 1 < (uint32_t)kMaxTrace)
      a.trace[d + 1].t_ns = global_timer_ns();
    if (!found) {
      levels = d + 1;  // nothing at depth d + 1
      break;
    }
    ++d;
    cur = nxt;
    if (d > a.n + 1) {
      if (t.rank == 0 && tid == 0) atomicOr(a.err, kErrLevels);
      levels = d;
      break;
    }
  }
  // reach counts: the persistent kernel's share (set above) plus each CTA's
  for (int o = 16; o > 0; o >>= 1) {
    nr += __shfl_down_sync(0xffffffffu, nr, o);
    mr += __shfl_down_sync(0xffffffffu, mr, o);
  }
  if ((tid & 31u) == 0) s_red[tid >> 5] = nr;
  __syncthreads();
  if (tid == 0) {
    unsigned long long v = 0;
    for (int i = 0; i < kNarrowBlock / 32; ++i) v += s_red[i];
    atomicAdd(&a.summary->nr, v);
  }
  __syncthreads();
  if ((tid & 31u) == 0) s_red[tid >> 5] = mr;
  __syncthreads();
  if (tid == 0) {
    unsigned long long v = 0;
    for (int i = 0; i < kNarrowBlock / 32; ++i) v += s_red[i];
    atomicAdd(&a.summary->mr, v);
    if (t.rank == 0) {
      a.summary->levels = levels;
      a.summary->bu_levels = __ldcg(&ho->bu_levels);
      a.summary->switches = __ldcg(&ho->switches);
      a.summary->pad = d0;  // level of the hand-over
    }
  }
  // no CTA leaves while another may still write its shared memory
  t.cl.sync();
  if (t.rank == 0 && tid == 0) ho->flag = 0u;
}

constexpr size_t kNarrowSmem = 2 * kNarrowCap * sizeof(uint2);

// The largest cluster of bfs_narrow CTAs (16, 8, 4, 2 or 1) the device can
// co-schedule, decided once per process; 1 needs no cluster launch.
int narrow_cluster() {
  static const int c = [] {
    cudaFuncSetAttribute(bfs_narrow, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kNarrowSmem);
    cudaFuncSetAttribute(bfs_narrow, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    for (int k = kNarrowMaxCluster; k > 1; k /= 2) {
      cudaLaunchAttribute attr;
      attr.id = cudaLaunchAttributeClusterDimension;
      attr.val.clusterDim.x = (unsigned)k;
      attr.val.clusterDim.y = 1;
      attr.val.clusterDim.z = 1;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)k);
      cfg.blockDim = dim3(kNarrowBlock);
      cfg.dynamicSmemBytes = kNarrowSmem;
      cfg.attrs = &attr;
      cfg.numAttrs = 1;
      int nc = 0;
      if (cudaOccupancyMaxActiveClusters(&nc, bfs_narrow, &cfg) == cudaSuccess && nc >= 1) return k;
      cudaGetLastError();
    }
    return 1;
  }();
  return c;
}

}  // namespace
}  // namespace grus

using namespace grus;

extern "C" int grus_bfs(grus_graph *g, uint32_t src, uint32_t *depth,
                        grus_stats *stats, void *stream) {
  if (!g || !depth) return GRUS_EINVAL;
  if (g->n == 0 || src >= g->n) {
    set_last_error("source vertex out of range");
    return GRUS_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g->mu);
  Workspace *w = nullptr;
  int rc = ws_get(g, &w);
  if (rc) return rc;
  const bool dev_out = is_device_pointer(depth);
  if (!dev_out && !w->depth) GRUS_CUDA_TRY(cudaMalloc(&w->depth, g->n * 4));

  // pull-level words per warp step: 2 (more resident warps) or 4 (more
  // loads in flight per warp)
  const bool wide = tune_or(g->tuning.bu_words, kDefBuWords) >= 4;
  const uint32_t pmode = g->tuning.depth_planes;
  const bool planes = pmode == 1 || (pmode == 0 && g->n >= kPlanesMinN);
  auto kern = wide ? (planes ? bfs_persistent<4, true> : bfs_persistent<4, false>)
                   : (planes ? bfs_persistent<2, true> : bfs_persistent<2, false>);
  static int occ_tab[4] = {-1, -1, -1, -1};
  int &occ = occ_tab[(wide ? 2 : 0) + (planes ? 1 : 0)];
  if (occ < 0) {
    GRUS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kBlock, 0));
  }
  const int sms = device_sm_count();
  int per_sm = occ;
  if (g->tuning.ctas_per_sm) per_sm = std::min<int>(per_sm, (int)g->tuning.ctas_per_sm);
  if (per_sm < 1) {
    set_last_error("bfs kernel cannot be resident");
    return GRUS_ECUDA;
  }

  Args a;
  std::memset(&a, 0, sizeof(a));
  a.offs = g->csr.offs;
  a.cols = g->csr.cols;
  // pull levels need in-edges: the CSR of a symmetric graph, else a built CSC
  a.ioffs = g->csc.offs;
  a.icols = g->csc.cols;
  if (g->flags & GRUS_GRAPH_SYMMETRIC) {
    a.ioffs = g->csr.offs;
    a.icols = g->csr.cols;
  }
  a.allow_pull = a.ioffs != nullptr;
  if (a.allow_pull) {
    rc = build_rep_locked(g);
    if (rc) return rc;
    a.rep = g->bfs_rep;
  }
  a.n = (uint32_t)g->n;
  a.W = w->W;
  a.m = g->m;
  a.src = src;
  a.depth = dev_out ? depth : w->depth;
  const uint64_t Wp = ((uint64_t)w->W + 31) / 32 * 32;
  a.visited = w->bitmaps;
  a.front[0] = w->bitmaps + Wp;
  a.front[1] = w->bitmaps + 2 * Wp;
  a.front[2] = w->bitmaps + 3 * Wp;
  a.aux = w->bitmaps + 4 * Wp;
  if (planes) {
    if (!w->planes) {
      GRUS_CUDA_TRY(cudaMalloc(&w->planes_own, (uint64_t)w->nplanes * Wp * 4));
      w->planes = w->planes_own;
    }
    a.planes = w->planes;
  }
  a.Wp = (uint32_t)Wp;
  a.nplanes = w->nplanes;
  a.queue[0] = w->queues;
  a.queue[1] = w->queues + g->n;
  a.chunks[0] = w->chunks;
  a.chunks[1] = w->chunks + w->chunk_cap;
  a.queue_cap = (uint32_t)g->n;
  a.chunk_cap = w->chunk_cap;
  a.slots = (LevelSlot *)(w->ctrl + kOffSlots);
  a.bar = (GridBarrier *)(w->ctrl + kOffBar);
  a.err = (uint32_t *)(w->ctrl + kOffErr);
  a.summary = (Summary *)(w->ctrl + kOffSummary);
  a.trace = w->trace;
  a.alpha = tune_or(g->tuning.alpha, kDefAlpha);
  a.beta = tune_or(g->tuning.beta, kDefBeta);
  a.huge = tune_or(g->tuning.huge_degree, kDefHuge);
  a.bu_scan = tune_or(g->tuning.bu_scan,
                      g->mem_mode == GRUS_MEM_MANAGED ? kDefBuScanManaged : kDefBuScan);
  const int ncl = narrow_cluster();
  a.narrow_nf = g->tuning.tail_cluster == 2 ? 0u : kNarrowNf * (uint32_t)ncl;
  a.ho = (Handover *)(w->ctrl + kOffHandover);
  a.timeout_ns = (uint64_t)tune_or(g->tuning.timeout_ms, 30000u) * 1000000ull;

  cudaLaunchAttribute attrs[2];
  int nattr = 0;
  attrs[nattr].id = cudaLaunchAttributeCooperative;
  attrs[nattr].val.cooperative = 1;
  ++nattr;
  const int win = l2_window(s, w->bitmaps, w->bitmap_bytes);
  if (win > 0) {
    attrs[nattr].id = cudaLaunchAttributeAccessPolicyWindow;
    attrs[nattr].val.accessPolicyWindow.base_ptr = w->bitmaps;
    attrs[nattr].val.accessPolicyWindow.num_bytes = (size_t)win;
    attrs[nattr].val.accessPolicyWindow.hitRatio = l2_hit_ratio((size_t)win);
    attrs[nattr].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attrs[nattr].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    ++nattr;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(sms * per_sm));
  cfg.blockDim = dim3(kBlock);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cfg.attrs = attrs;
  cfg.numAttrs = nattr;

  const bool sync = stats != nullptr || !dev_out;
  // barrier and error word: a timed-out launch leaves stale barrier state
  GRUS_CUDA_TRY(cudaMemsetAsync(w->ctrl + kOffBar, 0, kOffSummary - kOffBar, s));
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(w->ev0, s));
  GRUS_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, a));
  // continues a long traversal the persistent kernel handed over; returns at
  // once otherwise
  {
    cudaLaunchAttribute cattr;
    cattr.id = cudaLaunchAttributeClusterDimension;
    cattr.val.clusterDim.x = (unsigned)ncl;
    cattr.val.clusterDim.y = 1;
    cattr.val.clusterDim.z = 1;
    cudaLaunchConfig_t ncfg = {};
    ncfg.gridDim = dim3((unsigned)ncl);
    ncfg.blockDim = dim3(kNarrowBlock);
    ncfg.dynamicSmemBytes = kNarrowSmem;
    ncfg.stream = s;
    ncfg.attrs = &cattr;
    ncfg.numAttrs = ncl > 1 ? 1 : 0;
    GRUS_CUDA_TRY(cudaLaunchKernelEx(&ncfg, bfs_narrow, a));
  }
  if (stats) GRUS_CUDA_TRY(cudaEventRecord(w->ev1, s));
  if (!dev_out) GRUS_CUDA_TRY(cudaMemcpyAsync(depth, w->depth, g->n * 4, cudaMemcpyDeviceToHost, s));
  if (!sync) return GRUS_OK;
  GRUS_CUDA_TRY(cudaMemcpyAsync(w->ctrl_host, w->ctrl, kCtrlBytes, cudaMemcpyDeviceToHost, s));
  GRUS_CUDA_TRY(cudaMemcpyAsync(w->trace_host, w->trace, kMaxTrace * sizeof(LevelTrace),
                                cudaMemcpyDeviceToHost, s));
  GRUS_CUDA_TRY(cudaStreamSynchronize(s));
  w->trace_levels = std::min<int>(((const Summary *)(w->ctrl_host + kOffSummary))->levels + 1, kMaxTrace);
  const uint32_t errbits = *(uint32_t *)(w->ctrl_host + kOffErr);
  if (errbits) {
    // reset the control block so the next call starts clean
    cudaMemsetAsync(w->ctrl, 0, kCtrlBytes, s);
    cudaStreamSynchronize(s);
    return status_from_device_error(errbits);
  }
  if (stats) {
    const Summary *sm = (const Summary *)(w->ctrl_host + kOffSummary);
    std::memset(stats, 0, sizeof(*stats));
    stats->levels = sm->levels;
    stats->bottom_up_levels = sm->bu_levels;
    stats->direction_switches = sm->switches;
    stats->kernel_launches = 2;
    stats->vertices_reached = sm->nr;
    stats->edges_reached = sm->mr;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, w->ev0, w->ev1);
    stats->device_ms = ms;
  }
  return GRUS_OK;
}

extern "C" int grus_bfs_trace(grus_graph *g, grus_level_trace *out, int max_levels) {
  if (!g || !out || max_levels < 0) return GRUS_EINVAL;
  std::lock_guard<std::mutex> lk(g->mu);
  const Workspace *w = (const Workspace *)g->ws[kWsBfs];
  if (!w || w->trace_levels < 2) return 0;
  const int levels = std::min(w->trace_levels - 1, max_levels);
  const uint64_t t0 = w->trace_host[0].t_ns;
  for (int i = 0; i < levels; ++i) {
    const LevelTrace &r = w->trace_host[i + 1];
    out[i].end_ns = r.t_ns - t0;
    out[i].edges = r.mf;
    out[i].vertices = r.nf;
    out[i].pull = r.pull;
  }
  return levels;
}

// ---------------------------------------------------------------------------
// grus_bfs_static: the same persistent BFS with no allocation at call time.
//
// Some callers cannot call cudaMalloc: code embedded in a host process that
// owns the whole device-memory budget through its own pool (or holds the free
// HBM in a balloon, as this library's managed mode does, so any new
// allocation would fail), and latency-critical loops where cudaMalloc/cudaFree
// would synchronise the device and stall work on other streams.  For them
// the scratch (frontier bitmaps, queues, chunk lists, control block) lives in
// one file-scope __device__ array of fixed size, sized for graphs of up to
// GRUS_STATIC_MAX_VERTICES vertices and GRUS_STATIC_MAX_EDGES edges.  Every
// GPU that loads this library holds that array until the process exits.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side stand-in), so the first call on each device looks the
// address up with cudaGetSymbolAddress while that device is current and
// caches it; make that first call before any stream capture.  All calls on a
// device share the array and it keeps the last call's contents: each call
// clears its control block, and the kernel's prologue clears the bitmaps and
// level slots.  Calls that overlap on the GPU (different streams or threads,
// same device) race on the array and must be serialised by the caller.
// ---------------------------------------------------------------------------
namespace grus {
namespace {

constexpr uint64_t kStaticMaxN = GRUS_STATIC_MAX_VERTICES;
constexpr uint64_t kStaticMaxM = GRUS_STATIC_MAX_EDGES;
constexpr uint64_t kStaticWp = ((kStaticMaxN + 31) / 32 + 31) / 32 * 32;
constexpr uint64_t kStaticChunkCap = kStaticMaxM / kChunk + kStaticMaxM / kDefHuge + 2;
constexpr size_t kStaticBitmapOff = kCtrlBytes;
constexpr size_t kStaticQueueOff = kStaticBitmapOff + 4 * kStaticWp * 4;
constexpr size_t kStaticChunkOff = kStaticQueueOff + 2 * kStaticMaxN * 4;
constexpr size_t kStaticBytes = kStaticChunkOff + 2 * kStaticChunkCap * sizeof(uint4);
static_assert(kStaticBitmapOff % 256 == 0 && kStaticQueueOff % 256 == 0 &&
                  kStaticChunkOff % 256 == 0,
              "scratch sections must stay 256-byte aligned");

// [control block | visited + 3 frontier bitmaps | 2 queues | 2 chunk lists]
static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

std::mutex g_static_mu;
// Per device: the context the entry was looked up in, the array's device
// address in it and the persistent kernel's occupancy on that device.
struct StaticEntry {
  void *ctx = nullptr;
  void *base = nullptr;
  int occ = 0;
};
StaticEntry g_static[64];

// The current CUDA context (cuCtxGetCurrent, reached through the runtime so
// the library needs no link against the driver library), or null.
void *current_context() {
  using Fn = int (*)(void **);
  static Fn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (Fn) nullptr;
    return (Fn)p;
  }();
  void *ctx = nullptr;
  if (fn && fn(&ctx) != 0) ctx = nullptr;
  return ctx;
}

// Device address of g_static_scratch on the current device and the grid's
// CTAs per SM.  Looked up once per device, and again if the device's context
// changed since (a cudaDeviceReset makes the old address meaningless).
int static_scratch(void **base, int *occ) {
  int dev = 0;
  GRUS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return GRUS_ENODEV;
  // the caller's pointer checks (cudaPointerGetAttributes) have made the
  // device's context current by now
  void *ctx = current_context();
  std::lock_guard<std::mutex> lk(g_static_mu);
  StaticEntry &e = g_static[dev];
  if (!e.base || e.ctx != ctx) {
    void *p = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(&p, g_static_scratch);
    if (rc != cudaSuccess || !p) {
      set_last_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(rc));
      return status_from_cuda(rc == cudaSuccess ? cudaErrorInvalidSymbol : rc);
    }
    int o = 0;
    GRUS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, bfs_persistent<4, false>, kBlock, 0));
    e.ctx = ctx;
    e.base = p;
    e.occ = std::max(o, 1);
  }
  *base = e.base;
  *occ = e.occ;
  return GRUS_OK;
}

}  // namespace
}  // namespace grus

extern "C" int grus_bfs_static(uint64_t n, uint64_t m, const uint32_t *offsets,
                               const uint32_t *cols, int symmetric, uint32_t src,
                               uint32_t *depth, grus_stats *stats, void *stream) {
  if (!offsets || (m && !cols) || !depth) return GRUS_EINVAL;
  if (n > kStaticMaxN || m > kStaticMaxM) {
    set_last_error("grus_bfs_static handles at most GRUS_STATIC_MAX_VERTICES (2^20) vertices "
                   "and GRUS_STATIC_MAX_EDGES (2^25) edges; use grus_bfs for larger graphs");
    return GRUS_EOVERFLOW;
  }
  if (n == 0 || src >= n) {
    set_last_error("source vertex out of range");
    return GRUS_EINVAL;
  }
  if (!is_device_pointer(offsets) || (m && !is_device_pointer(cols)) || !is_device_pointer(depth)) {
    set_last_error("grus_bfs_static needs device (or managed) offsets, cols and depth");
    return GRUS_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  void *base = nullptr;
  int occ = 1;
  int rc = static_scratch(&base, &occ);
  if (rc) return rc;
  char *ctrl = (char *)base;
  uint32_t *bitmaps = (uint32_t *)((char *)base + kStaticBitmapOff);
  uint32_t *queues = (uint32_t *)((char *)base + kStaticQueueOff);
  uint4 *chunks = (uint4 *)((char *)base + kStaticChunkOff);
  const uint32_t W = (uint32_t)((n + 31) / 32);
  const uint64_t Wp = ((uint64_t)W + 31) / 32 * 32;

  Args a;
  std::memset(&a, 0, sizeof(a));
  a.offs = offsets;
  a.cols = cols;
  a.ioffs = symmetric ? offsets : nullptr;
  a.icols = symmetric ? cols : nullptr;
  a.allow_pull = symmetric != 0;
  a.n = (uint32_t)n;
  a.W = W;
  a.m = m;
  a.src = src;
  a.depth = depth;
  a.visited = bitmaps;
  a.front[0] = bitmaps + Wp;
  a.front[1] = bitmaps + 2 * Wp;
  a.front[2] = bitmaps + 3 * Wp;
  a.queue[0] = queues;
  a.queue[1] = queues + n;
  a.chunk_cap = (uint32_t)(m / kChunk + m / kDefHuge + 2);
  a.chunks[0] = chunks;
  a.chunks[1] = chunks + a.chunk_cap;
  a.queue_cap = (uint32_t)n;
  a.slots = (LevelSlot *)(ctrl + kOffSlots);
  a.bar = (GridBarrier *)(ctrl + kOffBar);
  a.err = (uint32_t *)(ctrl + kOffErr);
  a.summary = (Summary *)(ctrl + kOffSummary);
  a.alpha = kDefAlpha;
  a.beta = kDefBeta;
  a.huge = kDefHuge;
  a.bu_scan = kDefBuScan;
  a.timeout_ns = 30000ull * 1000000ull;

  // the array keeps the previous call's control block: start from zero
  GRUS_CUDA_TRY(cudaMemsetAsync(ctrl, 0, kCtrlBytes, s));
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeCooperative;
  attr.val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(device_sm_count() * occ));
  cfg.blockDim = dim3(kBlock);
  cfg.stream = s;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  GRUS_CUDA_TRY(cudaLaunchKernelEx(&cfg, bfs_persistent<4, false>, a));
  if (!stats) return GRUS_OK;
  unsigned char host_ctrl[kCtrlBytes];  // pageable stack copy: no allocation
  GRUS_CUDA_TRY(cudaMemcpyAsync(host_ctrl, ctrl, kCtrlBytes, cudaMemcpyDeviceToHost, s));
  GRUS_CUDA_TRY(cudaStreamSynchronize(s));
  const uint32_t errbits = *(const uint32_t *)(host_ctrl + kOffErr);
  if (errbits) return status_from_device_error(errbits);
  const Summary *sm = (const Summary *)(host_ctrl + kOffSummary);
  std::memset(stats, 0, sizeof(*stats));
  stats->levels = sm->levels;
  stats->bottom_up_levels = sm->bu_levels;
  stats->direction_switches = sm->switches;
  stats->kernel_launches = 1;
  stats->vertices_reached = sm->nr;
  stats->edges_reached = sm->mr;
  return GRUS_OK;
}

namespace grus {
CtrlView bfs_ctrl(grus_graph *g) {
  CtrlView v;
  std::lock_guard<std::mutex> lk(g->mu);
  const Workspace *w = (const Workspace *)g->ws[kWsBfs];
  if (w) {
    v.ctrl = w->ctrl;
    v.bytes = kCtrlBytes;
    v.err_off = kOffErr;
    v.bar_off = kOffBar;
  }
  return v;
}
}  // namespace grus
