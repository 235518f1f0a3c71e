// msssp_core.cuh -- the multi-source SSSP level loop, shared by the
// whole-GPU persistent kernel (msssp.cu, grid barriers) and the cluster
// workers of the batch engine (batch.cu, hardware cluster barriers).
//
// Up to 32 sources advance together and share every adjacency read:
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
// Each (v, s) pair reaches Dijkstra's distance whatever the schedule, so the
// outputs are bit-exact against single-source runs.
//
// Multi-graph launches (kUnion): several graphs share one launch and one
// level loop.  Their vertices are numbered one after another (graph g owns
// ids vb[g] .. vb[g+1]-1), D, F and Far cover all of them, and each graph
// brings its own sources in slots 0..k_g-1.  A vertex's graph is found by a
// binary search over the bases in shared memory; work entries keep the
// graph's own edge indices and a relaxation adds the graph's base to the
// column id.  No edge joins two graphs, so every graph's distances are the
// same as in a launch of its own; the threshold T is shared, which only
// changes the schedule.
#pragma once

#include "device_util.cuh"

namespace grus {
namespace ms {

constexpr uint32_t kPiece = 128;      // edges per work entry
constexpr uint32_t kInf = 4294967294u;

struct Slot {                         // 32 bytes
  uint32_t nent;                      // work entries of the level
  uint32_t moved;                     // pairs moved from far to near by a split
  uint32_t remaining;                 // vertices still holding far pairs after a split
  uint32_t pad0;
  unsigned long long visits;
  uint32_t pad[2];
};

constexpr int kMaxUnion = 64;         // graphs per multi-graph launch

// One graph of a multi-graph launch.
struct UnionGraph {
  const uint32_t *offs, *cols, *wts;
  uint32_t vbase;                     // first id of the graph's vertices
  uint32_t k;                         // its sources (slots 0..k-1)
  uint32_t *out[32];                  // output of slot s: n_g distances
};

struct View {
  const uint32_t *__restrict__ offs;
  const uint32_t *__restrict__ cols;
  const uint32_t *__restrict__ wts;
  uint32_t n, k;
  const uint32_t *srcs;               // k sources
  uint32_t *D;                        // n * KS
  uint32_t *F[2];                     // n each
  uint32_t *far;                      // n
  uint4 *ent;
  uint32_t ent_cap;
  Slot *slots;                        // 4, rotating by level
  uint32_t *minfar;                   // 2, by split parity
  uint32_t *err;
  uint32_t delta;
  // multi-graph launches only: graphs, and the slot of each of the nseeds
  // sources in srcs (global ids)
  const UnionGraph *ug = nullptr;
  uint32_t ngraphs = 0, nseeds = 0;
  const uint32_t *seed_slot = nullptr;
};

// Graph of vertex v: the largest g with vb[g] <= v (vb[ng] is the vertex
// count, above every id).
__device__ __forceinline__ uint32_t graph_of(const uint32_t *vb, uint32_t ng, uint32_t v) {
  uint32_t lo = 0, hi = ng;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (vb[mid] <= v) lo = mid;
    else hi = mid;
  }
  return lo;
}

struct Result {
  uint32_t levels = 0, splits = 0;
  unsigned long long visits = 0, nr = 0, mr = 0;  // nr/mr: this thread's share
};

// Step 1: vertices with a non-empty near mask become work entries.
template <int kBlock, bool kUnion>
__device__ __forceinline__ void build_entries(const View &a, const uint32_t *vb, uint32_t *F,
                                              Slot *sl, uint32_t tid, uint32_t nthreads) {
  const uint32_t rounds = (a.n + nthreads - 1) / nthreads;
  __shared__ uint32_t s_base;
  for (uint32_t r = 0; r < rounds; ++r) {
    const uint32_t v = r * nthreads + tid;
    uint32_t m = 0, b = 0, e = 0, nch = 0;
    if (v < a.n) {
      m = __ldcg(F + v);
      if (m) {
        F[v] = 0u;
        const uint32_t *offs = a.offs;
        uint32_t lv = v;
        if constexpr (kUnion) {
          const uint32_t g = graph_of(vb, a.ngraphs, v);
          offs = a.ug[g].offs;
          lv = v - vb[g];
        }
        b = __ldg(offs + lv);
        e = __ldg(offs + lv + 1);
        nch = (e - b + kPiece - 1) / kPiece;
      }
    }
    uint32_t total = 0;
    const uint32_t off = block_exclusive_scan<kBlock>(nch, &total);
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
// covers floor(32 / p) edges and every lane of it relaxes a live pair.
template <int KS, bool kUnion>
__device__ __forceinline__ unsigned long long relax_entry(const View &a, const uint32_t *vb,
                                                          const uint4 ent, uint32_t *Fn, uint32_t T) {
  const uint32_t lane = lane_id();
  const uint32_t u = ent.x, b = ent.y, e = ent.z, mask = ent.w;
  const uint32_t *cols = a.cols, *wts = a.wts;
  uint32_t vbase = 0;
  if constexpr (kUnion) {
    const uint32_t g = graph_of(vb, a.ngraphs, u);
    cols = a.ug[g].cols;
    wts = a.ug[g].wts;
    vbase = vb[g];
  }
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
    const uint32_t c = xi < e ? __ldg(cols + xi) + vbase : 0u;
    const uint32_t w = xi < e ? __ldg(wts + xi) : 0u;
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

// The whole traversal over the threads [0, nthreads) of one group (a grid or
// a cluster); `sync` is the group barrier (returns false when it gave up) and
// `out(s)` the output array of source s (one graph; a multi-graph launch
// writes through a.ug and takes the vertex bases vb, shared memory, ngraphs+1
// entries).  Returns false if a barrier failed.
template <int KS, int kBlock, bool kUnion = false, class Sync, class Out>
__device__ __forceinline__ bool run(const View &a, uint32_t tid, uint32_t nthreads, Sync &sync,
                                    const Out &out, Result &res, const uint32_t *vb = nullptr) {
  const uint32_t gwarp = tid >> 5, nwarps = nthreads >> 5;
  // prologue
  const size_t dn = (size_t)a.n * KS;
  for (size_t i = tid; i < dn; i += nthreads) a.D[i] = kInf;
  for (uint32_t i = tid; i < a.n; i += nthreads) {
    a.F[0][i] = 0u;
    a.F[1][i] = 0u;
    a.far[i] = 0u;
  }
  if (tid < 4 * sizeof(Slot) / 4) ((uint32_t *)a.slots)[tid] = 0u;
  if (tid < 2) a.minfar[tid] = 0xFFFFFFFFu;
  if (!sync()) return false;
  if constexpr (kUnion) {
    for (uint32_t i = tid; i < a.nseeds; i += nthreads) {
      const uint32_t src = a.srcs[i], slot = a.seed_slot[i];
      a.D[(size_t)src * KS + slot] = 0u;
      atomicOr(a.F[0] + src, 1u << slot);
    }
  } else if (tid < a.k) {
    const uint32_t src = a.srcs[tid];
    a.D[(size_t)src * KS + tid] = 0u;
    atomicOr(a.F[0] + src, 1u << tid);
  }
  if (!sync()) return false;

  uint32_t L = 0, T = a.delta, splits = 0, sel = 0;
  unsigned long long visits = 0;
  while (true) {
    Slot *sl = a.slots + (L & 3u);
    // reset the slot used two levels ahead
    if (tid < sizeof(Slot) / 4) ((uint32_t *)(a.slots + ((L + 2) & 3u)))[tid] = 0u;
    build_entries<kBlock, kUnion>(a, vb, a.F[sel], sl, tid, nthreads);
    if (!sync()) return false;
    const uint32_t nent = min(__ldcg(&sl->nent), a.ent_cap);
    if (nent == 0) {
      // near frontier empty: advance T and split the far masks into F[sel].
      // minfar[j & 1] holds the smallest distance left in the far masks by
      // split j - 1; split j reduces into the other word and resets this one
      // once every thread has read it (after the next barrier).
      const uint32_t Told = T;
      uint32_t Tnew = T + a.delta;
      const uint32_t mf = __ldcg(&a.minfar[splits & 1u]);
      if (mf != 0xFFFFFFFFu && mf >= Tnew) Tnew = (mf / a.delta + 1) * a.delta;
      uint32_t moved = 0, remaining = 0, local_min = 0xFFFFFFFFu;
      for (uint32_t v = tid; v < a.n; v += nthreads) {
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
        if (local_min != 0xFFFFFFFFu) atomicMin(&a.minfar[(splits + 1) & 1u], local_min);
        if (moved) atomicAdd(&sl->moved, moved);
        if (remaining) atomicAdd(&sl->remaining, remaining);
      }
      if (!sync()) return false;
      const uint32_t mv_all = __ldcg(&sl->moved), rem_all = __ldcg(&sl->remaining);
      if (tid == 0) a.minfar[splits & 1u] = 0xFFFFFFFFu;
      T = Tnew;
      ++splits;
      // the slot's counters are read by every thread before they are cleared;
      // the next split adds to them only after the next build's barrier
      if (!sync()) return false;
      if (tid == 0) {
        sl->moved = 0u;
        sl->remaining = 0u;
      }
      if (mv_all == 0 && rem_all == 0) break;  // nothing near, nothing far: done
      continue;  // build entries from the moved pairs (or split again)
    }
    uint32_t *Fn = a.F[sel ^ 1u];
    unsigned long long lv = 0;
    for (uint32_t i = gwarp; i < nent; i += nwarps)
      lv += relax_entry<KS, kUnion>(a, vb, __ldcg(a.ent + i), Fn, T);
    const unsigned long long bv = block_sum_u64<kBlock>(lv);
    if (threadIdx.x == 0 && bv) atomicAdd(&sl->visits, bv);
    if (!sync()) return false;
    visits += __ldcg(&sl->visits);
    sel ^= 1u;
    ++L;
    if (L > 4u * a.n + 64u) {
      if (tid == 0) atomicOr(a.err, kErrLevels);
      break;
    }
  }
  // epilogue: outputs (source-major) and this thread's reach counts
  unsigned long long nr = 0, mr = 0;
  if constexpr (kUnion) {
    for (uint32_t v = tid; v < a.n; v += nthreads) {
      const uint32_t g = graph_of(vb, a.ngraphs, v);
      const UnionGraph &G = a.ug[g];
      const uint32_t lv = v - vb[g];
      const uint32_t deg = __ldg(G.offs + lv + 1) - __ldg(G.offs + lv);
      for (uint32_t s = 0; s < G.k; ++s) {
        const uint32_t d = __ldcg(a.D + (size_t)v * KS + s);
        G.out[s][lv] = d;
        if (d != kInf) {
          ++nr;
          mr += deg;
        }
      }
    }
  } else {
    for (uint32_t v = tid; v < a.n; v += nthreads) {
      const uint32_t deg = __ldg(a.offs + v + 1) - __ldg(a.offs + v);
      for (uint32_t s = 0; s < a.k; ++s) {
        const uint32_t d = __ldcg(a.D + (size_t)v * KS + s);
        out(s)[v] = d;
        if (d != kInf) {
          ++nr;
          mr += deg;
        }
      }
    }
  }
  res.levels = L;
  res.splits = splits;
  res.visits = visits;
  res.nr = nr;
  res.mr = mr;
  return true;
}

}  // namespace ms
}  // namespace grus
