// expand.cuh -- degree-binned frontier expansion shared by the push-direction
// kernels (BFS, SSSP, the drop-in push_kernel).
//
// The reference maps one warp to every active vertex and strides the lanes
// over its list (include/kernel.cuh:42-80): degree<32 vertices leave most
// lanes idle and a hub of 10^5 edges serialises one warp.  Here a frontier
// is two work lists, binned when a vertex is enqueued:
//   queue  : vertex ids of degree 1 .. huge-1
//   chunks : (v, begin, end) pieces of at most kChunk (1024) edges of each vertex of
//            degree >= huge, so hubs spread over every SM
// and a CTA walks a tile of the queue with three cooperative mappings:
//   degree >= kCtaTh : the whole CTA strides the list, one vertex at a time
//   degree >= 32     : a warp strides the list
//   degree <  32     : warp scan-based gather -- the warp's short lists are
//                      laid end to end and each lane takes one edge; the
//                      owner is found by a shuffle binary search over the
//                      inclusive degree scan.
// Column loads are coalesced in every mapping.  A Visitor supplies
//   using aux_t = ...;                         type of the per-source value
//   aux_t aux(uint32_t v)                      per-source value, loaded once
//   void edge(uint32_t src, aux_t aux, uint32_t x)   work on edge index x
#pragma once

#include "device_util.cuh"

namespace grus {

constexpr uint32_t kChunk = 1024;  // edges per chunk work item
constexpr uint32_t kCtaTh = 256;   // CTA-cooperative degree threshold
constexpr uint32_t kWarpTh = 32;   // warp-cooperative degree threshold

// Appends vertex v (adjacency [b,e)) to the binned lists of a frontier.
// Degree-0 vertices are not enqueued (nothing to expand).  Returns false on
// overflow.
__device__ __forceinline__ bool push_binned(uint32_t v, uint32_t b, uint32_t e,
                                            uint32_t huge, uint32_t *q,
                                            uint32_t *qcount, uint32_t qcap,
                                            uint4 *c, uint32_t *ccount,
                                            uint32_t ccap) {
  const uint32_t d = e - b;
  if (d == 0) return true;
  if (d < huge) {
    const uint32_t pos = agg_reserve(qcount);
    if (pos >= qcap) return false;
    q[pos] = v;
    return true;
  }
  const uint32_t nch = (d + kChunk - 1) / kChunk;
  const uint32_t pos = atomicAdd(ccount, nch);
  if (pos + nch > ccap) return false;
  for (uint32_t k = 0; k < nch; ++k)
    c[pos + k] = make_uint4(v, b + k * kChunk, min(e, b + (k + 1) * kChunk), 0u);
  return true;
}

// The set bits of bitmap `bm` (W words) become binned work lists as
// push_binned would build them -- degree 1 .. huge-1 into the vertex queue,
// degree >= huge into kChunk-edge chunks -- and every word is cleared as it
// is read.  CTA `part` of `parts` owns a contiguous range of words and
// reserves queue space once per 256 words (block scan of the counts).
// Must be called by every thread of the CTA.
template <int kBlock>
__device__ __forceinline__ void bitmap_to_binned(uint32_t *bm, uint32_t W,
                                                 const uint32_t *__restrict__ offs, uint32_t huge,
                                                 uint32_t *q, uint32_t *qcount, uint32_t qcap,
                                                 uint4 *c, uint32_t *ccount, uint32_t ccap,
                                                 uint32_t *err, uint32_t part, uint32_t parts) {
  __shared__ uint32_t s_base;
  const uint32_t per = (W + parts - 1) / parts;
  const uint32_t w0 = min(W, part * per), w1 = min(W, w0 + per);
  for (uint32_t base = w0; base < w1; base += kBlock) {
    const uint32_t w = base + threadIdx.x;
    const uint32_t word = w < w1 ? __ldcg(bm + w) : 0u;
    if (word) bm[w] = 0u;
    uint32_t cnt = 0;
    for (uint32_t bits = word; bits; bits &= bits - 1) {
      const uint32_t v = w * 32 + (__ffs(bits) - 1);
      const uint32_t b = __ldg(offs + v), e = __ldg(offs + v + 1);
      const uint32_t d = e - b;
      if (d == 0) continue;
      if (d < huge) {
        ++cnt;
      } else {
        const uint32_t nch = (d + kChunk - 1) / kChunk;
        const uint32_t pos = atomicAdd(ccount, nch);
        if (pos + nch > ccap) {
          atomicOr(err, kErrOverflow);
        } else {
          for (uint32_t k = 0; k < nch; ++k)
            c[pos + k] = make_uint4(v, b + k * kChunk, min(e, b + (k + 1) * kChunk), 0u);
        }
      }
    }
    uint32_t total = 0;
    uint32_t at = block_exclusive_scan<kBlock>(cnt, &total);
    if (threadIdx.x == 0 && total) s_base = atomicAdd(qcount, total);
    __syncthreads();
    if (cnt) {
      at += s_base;
      for (uint32_t bits = word; bits; bits &= bits - 1) {
        const uint32_t v = w * 32 + (__ffs(bits) - 1);
        const uint32_t d = __ldg(offs + v + 1) - __ldg(offs + v);
        if (d == 0 || d >= huge) continue;
        if (at < qcap) q[at] = v;
        else atomicOr(err, kErrOverflow);
        ++at;
      }
    }
    __syncthreads();
  }
}

// One tile: every thread of the CTA brings one source (v, [beg,end), aux);
// an empty range means "no source".  CTA, warp and gather mappings in turn.
// Must be called by every thread of the CTA.
template <int kBlock, class Visitor>
__device__ __forceinline__ void expand_tile(uint32_t v, uint32_t beg, uint32_t end,
                                            typename Visitor::aux_t aux, Visitor &vis) {
  using A = typename Visitor::aux_t;
  __shared__ uint32_t s_owner, s_src, s_beg, s_end;
  __shared__ A s_aux;
  const uint32_t lane = lane_id();
  // CTA-cooperative: one block vote per tile when no source qualifies
  while (__syncthreads_or(end - beg >= kCtaTh)) {
    if (end - beg >= kCtaTh) s_owner = threadIdx.x;  // any qualifying thread wins
    __syncthreads();
    if (threadIdx.x == s_owner) {
      s_src = v;
      s_aux = aux;
      s_beg = beg;
      s_end = end;
      beg = end;
    }
    __syncthreads();
    const uint32_t cs = s_src, cb = s_beg, ce = s_end;
    const A ca = s_aux;
    for (uint32_t x = cb + threadIdx.x; x < ce; x += kBlock) vis.edge(cs, ca, x);
  }
  // warp-cooperative
  while (true) {
    const uint32_t ball = __ballot_sync(0xffffffffu, end - beg >= kWarpTh);
    if (!ball) break;
    const int leader = __ffs(ball) - 1;
    const uint32_t ws = __shfl_sync(0xffffffffu, v, leader);
    const A wa = __shfl_sync(0xffffffffu, aux, leader);
    const uint32_t wb = __shfl_sync(0xffffffffu, beg, leader);
    const uint32_t we = __shfl_sync(0xffffffffu, end, leader);
    if ((int)lane == leader) beg = end;
    for (uint32_t x = wb + lane; x < we; x += 32) vis.edge(ws, wa, x);
  }
  // scan-based gather of the remaining short lists
  const uint32_t deg = end - beg;
  uint32_t incl = deg;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if ((int)lane >= o) incl += t;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  for (uint32_t k0 = 0; k0 < total; k0 += 32) {
    const uint32_t k = k0 + lane;
    int j = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
      const uint32_t pv = __shfl_sync(0xffffffffu, incl, j + step - 1);
      if (pv <= k) j += step;
    }
    const uint32_t os = __shfl_sync(0xffffffffu, v, j);
    const A oa = __shfl_sync(0xffffffffu, aux, j);
    const uint32_t ob = __shfl_sync(0xffffffffu, beg, j);
    const uint32_t oi = __shfl_sync(0xffffffffu, incl, j);
    const uint32_t od = __shfl_sync(0xffffffffu, deg, j);
    if (k < total) vis.edge(os, oa, ob + (k - (oi - od)));
  }
}

// Chunk list: one (v, begin, end) piece per CTA, the whole CTA strides it.
// `part`/`parts` name this CTA among the CTAs sharing the work (the grid, or
// one thread-block cluster).
template <int kBlock, class Visitor>
__device__ __forceinline__ void expand_chunks(const uint4 *ccur, uint32_t ccount, Visitor &vis,
                                              uint32_t part, uint32_t parts) {
  for (uint32_t c = part; c < ccount; c += parts) {
    const uint4 ch = __ldcg(ccur + c);
    const typename Visitor::aux_t a = vis.aux(ch.x);
    for (uint32_t x = ch.y + threadIdx.x; x < ch.z; x += kBlock) vis.edge(ch.x, a, x);
  }
}

template <int kBlock, class Visitor>
__device__ __forceinline__ void expand_chunks(const uint4 *ccur, uint32_t ccount, Visitor &vis) {
  expand_chunks<kBlock>(ccur, ccount, vis, blockIdx.x, gridDim.x);
}

// Expands the queue tile by tile, then the chunk list.  A tile holds
// min(256, ceil(qcount / parts)) entries and tiles are dealt to the CTAs in
// turn, so a small frontier of heavy vertices spreads over as many CTAs as it
// has vertices (whole 256-entry tiles would put a 44-vertex frontier of
// degree-750 vertices on one CTA), while large frontiers keep full tiles.
// Must be called by every thread of the CTA.
template <int kBlock, class Visitor>
__device__ __forceinline__ void expand_binned(const uint32_t *__restrict__ offs,
                                              const uint32_t *qcur, uint32_t qcount,
                                              const uint4 *ccur, uint32_t ccount,
                                              Visitor &vis, uint32_t part, uint32_t parts) {
  const uint32_t tile = min((uint32_t)kBlock, qcount / parts + (qcount % parts != 0));
  for (uint32_t base = part * tile; base < qcount; base += parts * tile) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t hi = min(base + tile, qcount);
    uint32_t v = 0, beg = 0, end = 0;
    typename Visitor::aux_t aux{};
    if (i < hi) {
      v = __ldcg(qcur + i);
      beg = __ldg(offs + v);
      end = __ldg(offs + v + 1);
      aux = vis.aux(v);
    }
    expand_tile<kBlock>(v, beg, end, aux, vis);
  }
  expand_chunks<kBlock>(ccur, ccount, vis, part, parts);
}

template <int kBlock, class Visitor>
__device__ __forceinline__ void expand_binned(const uint32_t *__restrict__ offs,
                                              const uint32_t *qcur, uint32_t qcount,
                                              const uint4 *ccur, uint32_t ccount,
                                              Visitor &vis) {
  expand_binned<kBlock>(offs, qcur, qcount, ccur, ccount, vis, blockIdx.x, gridDim.x);
}

}  // namespace grus
