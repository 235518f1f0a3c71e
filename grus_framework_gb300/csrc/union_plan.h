// union_plan.h -- host logic (no CUDA) of the batch's whole-GPU SSSP lane:
// which SSSP queries on big graphs run together.
//
// Queries on one graph form packs of up to kPackMax sources (one
// multi-source traversal each).  Round r takes every graph's r-th pack; a
// round is cut into launches, in graph order, of at most max_graphs graphs
// whose distance rows -- vertices x the row width of the widest pack (8, 16
// or 32 sources) -- total at most `cap` entries, and whose vertex ids and
// work entries (vertices + edges / piece + 1024) fit 32 bits.  A launch of
// one graph runs as that graph's own multi-source launch; a launch of
// several as one multi-graph launch (msssp.cu).
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

namespace grus {

constexpr size_t kPackMax = 32;

struct UnionPack {
  uint32_t graph;
  std::vector<int> q;  // query indices, in the order given
};

struct UnionPlan {
  std::vector<std::vector<UnionPack>> launches;
  // sizes the multi-graph launches need (launches of one graph excluded)
  uint64_t max_v = 0, max_m = 0;
  uint32_t max_ks = 8;
  int unions = 0;  // launches of more than one graph
};

inline uint32_t union_row_width(size_t k) { return k <= 8 ? 8u : (k <= 16 ? 16u : 32u); }

// sssp: indices of the SSSP queries, grouped by graph (qgraph[i] is the graph
// of query i); gn / gm: vertices and edges per graph.
inline UnionPlan plan_union(const std::vector<int> &sssp, const std::vector<uint32_t> &qgraph,
                            const std::vector<uint64_t> &gn, const std::vector<uint64_t> &gm,
                            uint64_t cap, size_t max_graphs, uint64_t piece) {
  std::vector<std::vector<UnionPack>> rounds;
  for (size_t i = 0; i < sssp.size();) {
    const uint32_t g = qgraph[sssp[i]];
    size_t j = i;
    while (j < sssp.size() && qgraph[sssp[j]] == g) ++j;
    for (size_t r = 0; i + r * kPackMax < j; ++r) {
      if (rounds.size() <= r) rounds.emplace_back();
      UnionPack p;
      p.graph = g;
      p.q.assign(sssp.begin() + i + r * kPackMax,
                 sssp.begin() + std::min(j, i + (r + 1) * kPackMax));
      rounds[r].push_back(std::move(p));
    }
    i = j;
  }
  UnionPlan plan;
  constexpr uint64_t kIdLimit = 0xFFFFFFF0ull;
  for (auto &rd : rounds) {
    std::vector<UnionPack> cur;
    uint64_t v = 0, m = 0;
    size_t kmax = 0;
    auto flush = [&]() {
      if (cur.empty()) return;
      if (cur.size() > 1) {
        plan.max_v = std::max(plan.max_v, v);
        plan.max_m = std::max(plan.max_m, m);
        plan.max_ks = std::max(plan.max_ks, union_row_width(kmax));
        ++plan.unions;
      }
      plan.launches.push_back(std::move(cur));
      cur.clear();
      v = m = 0;
      kmax = 0;
    };
    for (UnionPack &p : rd) {
      const uint64_t n = gn[p.graph], e = gm[p.graph];
      const uint64_t ks = union_row_width(std::max(kmax, p.q.size()));
      if (!cur.empty() &&
          (cur.size() >= max_graphs || (v + n) * ks > cap || v + n >= kIdLimit ||
           v + n + (m + e) / piece + 1024 >= kIdLimit))
        flush();
      kmax = std::max(kmax, p.q.size());
      v += n;
      m += e;
      cur.push_back(std::move(p));
    }
    flush();
  }
  return plan;
}

}  // namespace grus
