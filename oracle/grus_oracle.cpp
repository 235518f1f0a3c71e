// grus_oracle.cpp -- CPU oracle for the Grus frontier-traversal path.
//
// TEST INFRASTRUCTURE ONLY (see grus_oracle.h).  The product never links or
// calls this file; tests, smoke() and bench.py's CPU-baseline legs do.
//
// Plain C++17 + OpenMP.  Every function cites the reference code whose
// behaviour it restates.  Host code only; no architecture intrinsics, so it
// builds and gives the same results on x86_64 and aarch64.
#include "grus_oracle.h"

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <queue>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Generator specification (shared, restated independently by the product's
// CUDA generator in grus_framework_gb300/csrc/graph_gen.cu).
//
//   mix64      = the SplitMix64 output function (Steele, Lea & Flood, 2014).
//   RMAT edge i of seed s: base = mix64(mix64(s) ^ i); level l draws the
//              16-bit lane (l%4) of mix64(base + l/4); quadrant thresholds
//              a=.57, a+b=.76, a+b+c=.95 scaled to 65536 (37356/49807/62259).
//   relabel    = three rounds of (x*odd + c) mod 2^scale, x ^= x >> ceil(s/2),
//              keys from mix64(seed ^ K); a bijection on [0, 2^scale).
//   weight     = mix64(mix64(seed ^ K2) ^ (min<<32 | max)) % 255 + 1, one
//              weight per undirected edge.
// ---------------------------------------------------------------------------
inline uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

constexpr uint32_t kRmatA = 37356, kRmatAB = 49807, kRmatABC = 62259;

inline void rmat_edge(int scale, uint64_t seed, uint64_t i, uint32_t *u,
                      uint32_t *v) {
  const uint64_t base = mix64(mix64(seed) ^ i);
  uint64_t r = 0;
  uint32_t a = 0, b = 0;
  for (int l = 0; l < scale; ++l) {
    if ((l & 3) == 0) r = mix64(base + (uint64_t)(l >> 2));
    const uint32_t x = (uint32_t)((r >> ((l & 3) * 16)) & 0xFFFFu);
    uint32_t ub, vb;
    if (x < kRmatA) { ub = 0; vb = 0; }
    else if (x < kRmatAB) { ub = 0; vb = 1; }
    else if (x < kRmatABC) { ub = 1; vb = 0; }
    else { ub = 1; vb = 1; }
    a = (a << 1) | ub;
    b = (b << 1) | vb;
  }
  *u = a;
  *v = b;
}

inline uint32_t relabel(int scale, uint64_t seed, uint32_t x) {
  const uint64_t mask = (scale >= 32) ? 0xFFFFFFFFull : ((1ull << scale) - 1);
  const uint64_t k0 = mix64(seed ^ 0x5851F42D4C957F2Dull);
  const int sh = (scale + 1) / 2;
  uint64_t y = x;
  for (int round = 0; round < 3; ++round) {
    const uint64_t kr = mix64(k0 + (uint64_t)round);
    const uint64_t mul = (kr & mask) | 1ull;
    const uint64_t add = (kr >> 32) & mask;
    y = (y * mul + add) & mask;
    if (sh > 0) y ^= (y >> sh);
  }
  return (uint32_t)y;
}

inline uint32_t edge_weight(uint64_t seed, uint32_t u, uint32_t v) {
  const uint64_t lo = u < v ? u : v, hi = u < v ? v : u;
  const uint64_t h = mix64(mix64(seed ^ 0x2545F4914F6CDD1Dull) ^ ((lo << 32) | hi));
  return (uint32_t)(h % 255ull) + 1u;
}

// Parallel sort: sorted chunks per thread, then pairwise in-place merges.
void parallel_sort(std::vector<uint64_t> &a) {
#ifdef _OPENMP
  const int T = omp_get_max_threads();
  const size_t n = a.size();
  if (T <= 1 || n < (1u << 16)) {
    std::sort(a.begin(), a.end());
    return;
  }
  int parts = 1;
  while (parts < T) parts <<= 1;
  std::vector<size_t> cut(parts + 1);
  for (int i = 0; i <= parts; ++i) cut[i] = n * (size_t)i / parts;
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < parts; ++i) std::sort(a.begin() + cut[i], a.begin() + cut[i + 1]);
  for (int width = 1; width < parts; width <<= 1) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < parts; i += 2 * width)
      std::inplace_merge(a.begin() + cut[i], a.begin() + cut[i + width],
                         a.begin() + cut[std::min(i + 2 * width, parts)]);
  }
#else
  std::sort(a.begin(), a.end());
#endif
}

// Sorted, de-duplicated (u<<32|v) keys -> CSR arrays.
int keys_to_csr(uint64_t n, std::vector<uint64_t> &keys, uint64_t seed,
                bool weighted, uint64_t *m_out, uint32_t **offs,
                uint32_t **cols, uint32_t **wts) {
  parallel_sort(keys);
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  while (!keys.empty() && keys.back() == UINT64_MAX) keys.pop_back();
  const uint64_t m = keys.size();
  if (m >= 0xFFFFFFFFull) return -EOVERFLOW;
  uint32_t *o = (uint32_t *)std::calloc(n + 1, sizeof(uint32_t));
  uint32_t *c = (uint32_t *)std::malloc((m ? m : 1) * sizeof(uint32_t));
  uint32_t *w = weighted ? (uint32_t *)std::malloc((m ? m : 1) * sizeof(uint32_t)) : nullptr;
  if (!o || !c || (weighted && !w)) {
    std::free(o); std::free(c); std::free(w);
    return -ENOMEM;
  }
#pragma omp parallel for schedule(static)
  for (uint64_t e = 0; e < m; ++e) {
    const uint32_t u = (uint32_t)(keys[e] >> 32), v = (uint32_t)keys[e];
    c[e] = v;
    if (w) w[e] = edge_weight(seed, u, v);
    // offsets: the first edge of each row (and of empty rows before it)
    const uint64_t prev = e ? (keys[e - 1] >> 32) + 1 : 0;
    for (uint64_t x = prev; x <= u; ++x) o[x] = (uint32_t)e;
  }
  const uint64_t last = m ? (keys[m - 1] >> 32) + 1 : 0;
  for (uint64_t x = last; x <= n; ++x) o[x] = (uint32_t)m;
  *m_out = m;
  *offs = o;
  *cols = c;
  *wts = w;
  return 0;
}

}  // namespace

extern "C" {

void orc_rmat_edge(int scale, uint64_t seed, uint64_t i, uint32_t *u,
                   uint32_t *v) {
  rmat_edge(scale, seed, i, u, v);
}
uint32_t orc_relabel(int scale, uint64_t seed, uint32_t x) {
  return relabel(scale, seed, x);
}
uint32_t orc_edge_weight(uint64_t seed, uint32_t u, uint32_t v) {
  return edge_weight(seed, u, v);
}
void orc_free(void *p) { std::free(p); }

int orc_rmat_csr(int scale, int edge_factor, uint64_t seed, uint32_t flags,
                 uint64_t *n_out, uint64_t *m_out, uint32_t **offs,
                 uint32_t **cols, uint32_t **wts) {
  if (scale < 1 || scale > 30 || edge_factor < 1) return -EINVAL;
  const uint64_t n = 1ull << scale;
  const uint64_t E = (uint64_t)edge_factor << scale;
  const bool sym = flags & ORC_GEN_SYMMETRIC;
  const uint64_t per = sym ? 2 : 1;
  // keys (u<<32|v); self-loops become UINT64_MAX and are dropped after sorting
  std::vector<uint64_t> keys(per * E);
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < E; ++i) {
    uint32_t u, v;
    rmat_edge(scale, seed, i, &u, &v);
    if (flags & ORC_GEN_RELABEL) {
      u = relabel(scale, seed, u);
      v = relabel(scale, seed, v);
    }
    const bool loop = u == v;
    keys[per * i] = loop ? UINT64_MAX : (((uint64_t)u << 32) | v);
    if (sym) keys[per * i + 1] = loop ? UINT64_MAX : (((uint64_t)v << 32) | u);
  }
  *n_out = n;
  return keys_to_csr(n, keys, seed, flags & ORC_GEN_WEIGHTED, m_out, offs,
                     cols, wts);
}

int orc_grid_csr(uint32_t rows, uint32_t cols_, uint64_t seed, uint32_t flags,
                 uint64_t *n_out, uint64_t *m_out, uint32_t **offs,
                 uint32_t **cols, uint32_t **wts) {
  if (rows == 0 || cols_ == 0) return -EINVAL;
  const uint64_t n = (uint64_t)rows * cols_;
  if (n >= 0xFFFFFFFFull) return -EOVERFLOW;
  std::vector<uint64_t> keys;
  keys.reserve(4 * n);
  for (uint64_t r = 0; r < rows; ++r)
    for (uint64_t c = 0; c < cols_; ++c) {
      const uint64_t u = r * cols_ + c;
      if (r > 0) keys.push_back((u << 32) | (u - cols_));
      if (c > 0) keys.push_back((u << 32) | (u - 1));
      if (c + 1 < cols_) keys.push_back((u << 32) | (u + 1));
      if (r + 1 < rows) keys.push_back((u << 32) | (u + cols_));
    }
  *n_out = n;
  return keys_to_csr(n, keys, seed, flags & ORC_GEN_WEIGHTED, m_out, offs,
                     cols, wts);
}

// ---------------------------------------------------------------------------
// .gr (Galois v1) reader, include/graph_loader.cuh:65-159: header u64[4] =
// {version=1, sizeEdgeTy, n, m}; u64 end offsets x n (into xadj[1..n], :114-119);
// u32 destinations x m (:122-131); when sizeEdgeTy != 0, 4 bytes of padding if
// m is odd (:139-141) then u32 edge data x m (:142-153), else weights are 1
// (:95-101).  Unlike the reference, every malformed input is an error: bad
// version, sizeEdgeTy not in {0,4}, short reads, non-monotone offsets, a
// destination >= n, or m >= 2^32 (the reference truncates offsets into u32).
// ---------------------------------------------------------------------------
int orc_read_gr(const char *path, uint64_t *n_out, uint64_t *m_out,
                uint32_t **offs, uint32_t **cols, uint32_t **wts) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return -ENOENT;
  uint64_t h[4];
  int rc = 0;
  uint32_t *o = nullptr, *c = nullptr, *w = nullptr;
  uint64_t n = 0, m = 0;
  std::vector<uint64_t> ends;
  if (std::fread(h, sizeof(uint64_t), 4, f) != 4) { rc = -EIO; goto out; }
  if (h[0] != 1) { rc = -EINVAL; goto out; }
  if (h[1] != 0 && h[1] != 4) { rc = -EINVAL; goto out; }
  n = h[2];
  m = h[3];
  if (n >= 0xFFFFFFFFull || m >= 0xFFFFFFFFull) { rc = -EOVERFLOW; goto out; }
  ends.resize(n);
  if (n && std::fread(ends.data(), sizeof(uint64_t), n, f) != n) { rc = -EIO; goto out; }
  o = (uint32_t *)std::malloc((n + 1) * sizeof(uint32_t));
  c = (uint32_t *)std::malloc((m ? m : 1) * sizeof(uint32_t));
  w = (uint32_t *)std::malloc((m ? m : 1) * sizeof(uint32_t));
  if (!o || !c || !w) { rc = -ENOMEM; goto out; }
  o[0] = 0;
  for (uint64_t i = 0; i < n; ++i) {
    if (ends[i] > m || (i && ends[i] < ends[i - 1])) { rc = -EINVAL; goto out; }
    o[i + 1] = (uint32_t)ends[i];
  }
  if (n && o[n] != m) { rc = -EINVAL; goto out; }
  if (!n && m) { rc = -EINVAL; goto out; }
  if (m && std::fread(c, sizeof(uint32_t), m, f) != m) { rc = -EIO; goto out; }
  for (uint64_t e = 0; e < m; ++e)
    if (c[e] >= n) { rc = -EINVAL; goto out; }
  if (h[1]) {
    if (m % 2) {
      uint32_t pad;
      if (std::fread(&pad, 4, 1, f) != 1) { rc = -EIO; goto out; }
    }
    if (m && std::fread(w, sizeof(uint32_t), m, f) != m) { rc = -EIO; goto out; }
  } else {
    for (uint64_t e = 0; e < m; ++e) w[e] = 1;
  }
out:
  std::fclose(f);
  if (rc) {
    std::free(o); std::free(c); std::free(w);
    return rc;
  }
  *n_out = n;
  *m_out = m;
  *offs = o;
  *cols = c;
  *wts = w;
  return 0;
}

int orc_write_gr(const char *path, uint64_t n, uint64_t m,
                 const uint32_t *offs, const uint32_t *cols,
                 const uint32_t *wts) {
  FILE *f = std::fopen(path, "wb");
  if (!f) return -EIO;
  const uint64_t h[4] = {1, wts ? 4ull : 0ull, n, m};
  bool ok = std::fwrite(h, sizeof(uint64_t), 4, f) == 4;
  for (uint64_t i = 0; ok && i < n; ++i) {
    const uint64_t e = offs[i + 1];
    ok = std::fwrite(&e, sizeof(uint64_t), 1, f) == 1;
  }
  if (ok && m) ok = std::fwrite(cols, sizeof(uint32_t), m, f) == m;
  if (ok && wts) {
    if (m % 2) {
      const uint32_t pad = 0;
      ok = std::fwrite(&pad, 4, 1, f) == 1;
    }
    if (ok && m) ok = std::fwrite(wts, sizeof(uint32_t), m, f) == m;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? 0 : -EIO;
}

// Counting-sort transpose, the algorithm of include/graph.cuh:273-303 (column
// counts, exclusive scan, row-ordered scatter, shift back).  The reference's
// scatter of the edge data is commented out (:294); here it is carried.
void orc_csr_to_csc(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                    const uint32_t *wts, uint32_t *t_offs, uint32_t *t_cols,
                    uint32_t *t_wts) {
  const uint64_t nnz = offs[n];
  std::fill(t_offs, t_offs + n + 1, 0u);
  for (uint64_t e = 0; e < nnz; ++e) t_offs[cols[e]]++;
  uint32_t cum = 0;
  for (uint64_t c = 0; c < n; ++c) {
    const uint32_t t = t_offs[c];
    t_offs[c] = cum;
    cum += t;
  }
  t_offs[n] = (uint32_t)nnz;
  for (uint64_t r = 0; r < n; ++r)
    for (uint32_t e = offs[r]; e < offs[r + 1]; ++e) {
      const uint32_t d = t_offs[cols[e]]++;
      t_cols[d] = (uint32_t)r;
      if (t_wts && wts) t_wts[d] = wts[e];
    }
  uint32_t last = 0;
  for (uint64_t c = 0; c <= n; ++c) {
    const uint32_t t = t_offs[c];
    t_offs[c] = last;
    last = t;
  }
}

// First index of maximum out-degree: std::max_element over outDegree exactly
// as include/graph_loader.cuh:132-137 computes it.
uint32_t orc_max_degree_vertex(uint64_t n, const uint32_t *offs) {
  uint32_t best = 0, bd = 0;
  for (uint64_t i = 0; i < n; ++i) {
    const uint32_t d = offs[i + 1] - offs[i];
    if (d > bd) { bd = d; best = (uint32_t)i; }
  }
  return best;
}

// BFS: the fixpoint of samples/bfs/bfs.cu:18-87 -- label[src]=0, every other
// vertex INFINIT (:18-23), and a vertex reached at iteration itr gets itr+1
// (:51-60).  Serial FIFO queue.
int orc_bfs(uint64_t n, const uint32_t *offs, const uint32_t *cols,
            uint32_t src, uint32_t *depth) {
  if (src >= n) return -EINVAL;
  std::fill(depth, depth + n, ORC_INFINIT);
  std::vector<uint32_t> q;
  q.reserve(n);
  depth[src] = 0;
  q.push_back(src);
  for (size_t h = 0; h < q.size(); ++h) {
    const uint32_t u = q[h];
    for (uint32_t e = offs[u]; e < offs[u + 1]; ++e) {
      const uint32_t v = cols[e];
      if (depth[v] == ORC_INFINIT) {
        depth[v] = depth[u] + 1;
        q.push_back(v);
      }
    }
  }
  return 0;
}

// SSSP: the fixpoint of samples/sssp/sssp.cu:51-60 (relax label[dst] >
// label[src] + w) is the shortest-path distance; computed with Dijkstra over
// 64-bit sums.  Unreached stays INFINIT (:18-23).  Distances must stay below
// INFINIT, which holds whenever (n-1)*max_weight < 2^32-1.
int orc_sssp(uint64_t n, const uint32_t *offs, const uint32_t *cols,
             const uint32_t *wts, uint32_t src, uint32_t *dist) {
  if (src >= n) return -EINVAL;
  std::vector<uint64_t> d(n, UINT64_MAX);
  using Item = std::pair<uint64_t, uint32_t>;
  std::priority_queue<Item, std::vector<Item>, std::greater<Item>> pq;
  d[src] = 0;
  pq.push({0, src});
  while (!pq.empty()) {
    const Item it = pq.top();
    pq.pop();
    if (it.first != d[it.second]) continue;
    const uint32_t u = it.second;
    for (uint32_t e = offs[u]; e < offs[u + 1]; ++e) {
      const uint64_t nd = it.first + (wts ? wts[e] : 1u);
      if (nd < d[cols[e]]) {
        d[cols[e]] = nd;
        pq.push({nd, cols[e]});
      }
    }
  }
  for (uint64_t v = 0; v < n; ++v) {
    if (d[v] != UINT64_MAX && d[v] >= ORC_INFINIT) return -EOVERFLOW;
    dist[v] = d[v] == UINT64_MAX ? ORC_INFINIT : (uint32_t)d[v];
  }
  return 0;
}

// CC: on a symmetric graph the fixpoint of samples/cc/cc.cu:69-79 (label=v,
// then atomicMin(label[dst], label[src]) along edges) is the minimum vertex id
// of each connected component.  Union-find, linking the larger root under the
// smaller one so every root is its component's minimum.  Edges are treated as
// undirected.
int orc_cc(uint64_t n, const uint32_t *offs, const uint32_t *cols,
           uint32_t *label) {
  std::vector<uint32_t> p(n);
  for (uint64_t i = 0; i < n; ++i) p[i] = (uint32_t)i;
  auto find = [&](uint32_t x) {
    while (p[x] != x) {
      p[x] = p[p[x]];
      x = p[x];
    }
    return x;
  };
  for (uint64_t u = 0; u < n; ++u)
    for (uint32_t e = offs[u]; e < offs[u + 1]; ++e) {
      uint32_t a = find((uint32_t)u), b = find(cols[e]);
      if (a == b) continue;
      if (a < b) std::swap(a, b);
      p[a] = b;
    }
  for (uint64_t v = 0; v < n; ++v) label[v] = find((uint32_t)v);
  return 0;
}

// Pull PageRank in FP64: r0 = 1/n, r'(v) = (1-d)/n + d * sum_{u->v} r(u)/outdeg(u),
// dangling mass not redistributed (samples/pagerank/pr.cu:29-31,83 never push
// from out-degree-0 vertices).  Computed in push form over the CSR, which
// gives the same sums.
int orc_pagerank(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                 double damping, int iters, double *rank) {
  if (n == 0) return 0;
  std::vector<double> acc(n);
  for (uint64_t v = 0; v < n; ++v) rank[v] = 1.0 / (double)n;
  for (int it = 0; it < iters; ++it) {
    std::fill(acc.begin(), acc.end(), 0.0);
    for (uint64_t u = 0; u < n; ++u) {
      const uint32_t deg = offs[u + 1] - offs[u];
      if (!deg) continue;
      const double c = rank[u] / (double)deg;
      for (uint32_t e = offs[u]; e < offs[u + 1]; ++e) acc[cols[e]] += c;
    }
    for (uint64_t v = 0; v < n; ++v)
      rank[v] = (1.0 - damping) / (double)n + damping * acc[v];
  }
  return 0;
}

// Delta-push PageRank of samples/pagerank/pr.cu:17-90, run sequentially in
// the reference's precision: pr_init (:17-33) sets rank = 1-ALPHA and pushes
// (1-ALPHA)*ALPHA/deg along out-edges; each round prepare()/pr_dd0 (:34-43)
// folds delta into rank and moves it to delta2; the updater (:78-90) adds
// delta2[src]*ALPHA/outdeg(src) to delta[dst] and activates dst when delta
// crosses EPSILON upward.  The full initial frontier is Frontier<BDF> with
// initFull (pr.cu:184).  ALPHA=0.85, EPSILON=0.01 (include/common.cuh:32-33).
int orc_delta_pagerank(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                       float *rank, uint32_t *iterations) {
  const double ALPHA = 0.85, EPSILON = 0.01;
  std::vector<float> delta(n, 0.f), delta2(n, 0.f);
  for (uint64_t v = 0; v < n; ++v) rank[v] = (float)(1.0 - ALPHA);
  for (uint64_t u = 0; u < n; ++u) {
    const uint32_t deg = offs[u + 1] - offs[u];
    const float update = (float)(((1.0 - ALPHA) * ALPHA) / deg);
    for (uint32_t e = offs[u]; e < offs[u + 1]; ++e) delta[cols[e]] += update;
  }
  std::vector<uint32_t> frontier(n);
  for (uint64_t v = 0; v < n; ++v) frontier[v] = (uint32_t)v;
  std::vector<char> flag(n, 0);
  uint32_t itr = 0;
  while (!frontier.empty()) {
    for (uint64_t v = 0; v < n; ++v) {
      const float res = delta[v];
      delta[v] = 0.f;
      delta2[v] = res;
      rank[v] += res;
    }
    for (uint32_t src : frontier) {
      const uint32_t deg = offs[src + 1] - offs[src];
      for (uint32_t e = offs[src]; e < offs[src + 1]; ++e) {
        const uint32_t dst = cols[e];
        const float update = (float)((double)delta2[src] * ALPHA / (double)deg);
        const float dt = delta[dst];
        delta[dst] = dt + update;
        if (((double)(dt + update) > EPSILON) && ((double)dt < EPSILON)) flag[dst] = 1;
      }
    }
    frontier.clear();
    for (uint64_t v = 0; v < n; ++v)
      if (flag[v]) {
        frontier.push_back((uint32_t)v);
        flag[v] = 0;
      }
    ++itr;
  }
  if (iterations) *iterations = itr;
  return 0;
}

uint64_t orc_reached_edges(uint64_t n, const uint32_t *offs,
                           const uint32_t *depth) {
  uint64_t s = 0;
  for (uint64_t v = 0; v < n; ++v)
    if (depth[v] != ORC_INFINIT) s += offs[v + 1] - offs[v];
  return s;
}

int orc_bfs_multi(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                  const uint32_t *srcs, int k, uint32_t *depths) {
  for (int i = 0; i < k; ++i) {
    const int rc = orc_bfs(n, offs, cols, srcs[i], depths + (uint64_t)i * n);
    if (rc) return rc;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// OpenMP baselines: the plain parallel CPU versions of the same algorithms,
// timed as the CPU path (the reference has no host implementation).
// ---------------------------------------------------------------------------
static inline double now_s() {
  return std::chrono::duration<double>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

int orc_omp_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static void set_threads(int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
}

// Level-synchronous top-down BFS with a shared frontier and CAS claims.
double orc_omp_bfs(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                   uint32_t src, uint32_t *depth, int threads) {
  if (src >= n) return -1.0;
  set_threads(threads);
  const double t0 = now_s();
#pragma omp parallel for schedule(static)
  for (uint64_t v = 0; v < n; ++v) depth[v] = ORC_INFINIT;
  std::vector<uint32_t> cur, next(n);
  cur.push_back(src);
  depth[src] = 0;
  uint32_t level = 0;
  while (!cur.empty()) {
    std::atomic<uint64_t> tail{0};
#pragma omp parallel
    {
      std::vector<uint32_t> local;
      local.reserve(4096);
#pragma omp for schedule(dynamic, 64) nowait
      for (size_t i = 0; i < cur.size(); ++i) {
        const uint32_t u = cur[i];
        for (uint32_t e = offs[u]; e < offs[u + 1]; ++e) {
          const uint32_t v = cols[e];
          uint32_t expect = ORC_INFINIT;
          if (__atomic_load_n(&depth[v], __ATOMIC_RELAXED) == ORC_INFINIT &&
              __atomic_compare_exchange_n(&depth[v], &expect, level + 1, false,
                                          __ATOMIC_RELAXED, __ATOMIC_RELAXED))
            local.push_back(v);
          if (local.size() == 4096) {
            const uint64_t at = tail.fetch_add(local.size());
            std::copy(local.begin(), local.end(), next.begin() + at);
            local.clear();
          }
        }
      }
      const uint64_t at = tail.fetch_add(local.size());
      std::copy(local.begin(), local.end(), next.begin() + at);
    }
    cur.assign(next.begin(), next.begin() + tail.load());
    ++level;
  }
  return now_s() - t0;
}

static inline bool atomic_min_u32(uint32_t *p, uint32_t v) {
  uint32_t old = __atomic_load_n(p, __ATOMIC_RELAXED);
  while (v < old) {
    if (__atomic_compare_exchange_n(p, &old, v, true, __ATOMIC_RELAXED,
                                    __ATOMIC_RELAXED))
      return true;
  }
  return false;
}

// Frontier Bellman-Ford with CAS-min relaxations (the algorithm of
// samples/sssp/sssp.cu:51-60 with the lost-update race removed).
double orc_omp_sssp(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                    const uint32_t *wts, uint32_t src, uint32_t *dist,
                    int threads) {
  if (src >= n) return -1.0;
  set_threads(threads);
  const double t0 = now_s();
  std::vector<uint8_t> inq(n, 0);
#pragma omp parallel for schedule(static)
  for (uint64_t v = 0; v < n; ++v) dist[v] = ORC_INFINIT;
  std::vector<uint32_t> cur, next(n);
  dist[src] = 0;
  cur.push_back(src);
  while (!cur.empty()) {
    std::atomic<uint64_t> tail{0};
#pragma omp parallel
    {
      std::vector<uint32_t> local;
#pragma omp for schedule(dynamic, 64) nowait
      for (size_t i = 0; i < cur.size(); ++i) {
        const uint32_t u = cur[i];
        const uint32_t du = __atomic_load_n(&dist[u], __ATOMIC_RELAXED);
        for (uint32_t e = offs[u]; e < offs[u + 1]; ++e) {
          const uint32_t v = cols[e];
          const uint32_t nd = du + (wts ? wts[e] : 1u);
          if (atomic_min_u32(&dist[v], nd)) {
            uint8_t z = 0;
            if (__atomic_compare_exchange_n(&inq[v], &z, (uint8_t)1, false,
                                            __ATOMIC_RELAXED, __ATOMIC_RELAXED))
              local.push_back(v);
          }
        }
      }
      const uint64_t at = tail.fetch_add(local.size());
      std::copy(local.begin(), local.end(), next.begin() + at);
    }
    cur.assign(next.begin(), next.begin() + tail.load());
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < cur.size(); ++i) inq[cur[i]] = 0;
  }
  return now_s() - t0;
}

// Min-label propagation (samples/cc/cc.cu:69-79) iterated to convergence.
double orc_omp_cc(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                  uint32_t *label, int threads) {
  set_threads(threads);
  const double t0 = now_s();
#pragma omp parallel for schedule(static)
  for (uint64_t v = 0; v < n; ++v) label[v] = (uint32_t)v;
  bool changed = true;
  while (changed) {
    changed = false;
#pragma omp parallel for schedule(dynamic, 1024) reduction(|| : changed)
    for (uint64_t v = 0; v < n; ++v) {
      uint32_t best = __atomic_load_n(&label[v], __ATOMIC_RELAXED);
      for (uint32_t e = offs[v]; e < offs[v + 1]; ++e) {
        const uint32_t l = __atomic_load_n(&label[cols[e]], __ATOMIC_RELAXED);
        if (l < best) best = l;
      }
      if (atomic_min_u32(&label[v], best)) changed = true;
    }
  }
  return now_s() - t0;
}

// 20-iteration pull PageRank over the in-edge (CSC) arrays.
double orc_omp_pagerank(uint64_t n, const uint32_t *t_offs,
                        const uint32_t *t_cols, const uint32_t *outdeg,
                        float damping, int iters, float *rank, int threads) {
  set_threads(threads);
  const double t0 = now_s();
  std::vector<float> contrib(n);
  const float base = (1.0f - damping) / (float)n;
#pragma omp parallel for schedule(static)
  for (uint64_t v = 0; v < n; ++v) rank[v] = 1.0f / (float)n;
  for (int it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
    for (uint64_t u = 0; u < n; ++u)
      contrib[u] = outdeg[u] ? rank[u] / (float)outdeg[u] : 0.0f;
#pragma omp parallel for schedule(dynamic, 1024)
    for (uint64_t v = 0; v < n; ++v) {
      double s = 0.0;
      for (uint32_t e = t_offs[v]; e < t_offs[v + 1]; ++e) s += contrib[t_cols[e]];
      rank[v] = base + damping * (float)s;
    }
  }
  return now_s() - t0;
}

}  // extern "C"
