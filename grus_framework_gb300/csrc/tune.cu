// tune.cu -- autotuners: the persistent traversal kernels of one graph, and
// the batched and served forms over a query mix.
//
// Coordinate descent over the launch / heuristic knobs of grus_tuning: for
// each knob in turn, every candidate value is timed (best of `reps` runs,
// CUDA events around the kernel) with the other knobs at their current best,
// and the fastest value is kept.  BFS tunes the push/pull thresholds alpha
// and beta, the pull-level words per warp step, the hub chunking degree and
// the CTAs per SM; SSSP tunes the bucket width Delta, the chunking degree and
// the CTAs per SM.  The winner is stored on the graph (grus_graph_set_tuning)
// and returned.  Results are bit-identical under every candidate (the
// kernels' outputs do not depend on these knobs), so tuning never trades
// correctness.  The reference has no tuning (fixed BLOCK_SIZE, fixed
// thresholds, include/common.cuh:30, include/frontier.cuh:140).
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "grus_internal.cuh"

using namespace grus;

namespace {

struct Knob {
  uint32_t grus_tuning::*u = nullptr;
  float grus_tuning::*f = nullptr;
  std::vector<double> values;
};

void set_knob(grus_tuning &t, const Knob &k, double v) {
  if (k.u) t.*(k.u) = (uint32_t)v;
  else t.*(k.f) = (float)v;
}

}  // namespace

extern "C" int grus_autotune(grus_graph *g, uint32_t algo, uint32_t src, int reps,
                             grus_tuning *best_out, float *best_ms_out) {
  if (!g || src >= g->n || algo > GRUS_ALGO_SSSP) return GRUS_EINVAL;
  if (algo == GRUS_ALGO_SSSP && !g->csr.wts) return GRUS_EINVAL;
  if (reps < 1) reps = 2;
  uint32_t *out = nullptr;
  GRUS_CUDA_TRY(cudaMalloc(&out, g->n * 4));
  std::vector<Knob> knobs;
  if (algo == GRUS_ALGO_BFS) {
    knobs.push_back({nullptr, &grus_tuning::alpha, {6, 15, 40}});
    knobs.push_back({nullptr, &grus_tuning::beta, {8, 18, 48}});
    knobs.push_back({&grus_tuning::bu_words, nullptr, {2, 4}});
    knobs.push_back({&grus_tuning::depth_planes, nullptr, {1, 2}});
    knobs.push_back({&grus_tuning::huge_degree, nullptr, {512, 1024, 4096}});
    knobs.push_back({&grus_tuning::ctas_per_sm, nullptr, {0, 2, 3}});
  } else {
    knobs.push_back({&grus_tuning::sssp_delta, nullptr, {96, 192, 384, 640, 1024}});
    knobs.push_back({&grus_tuning::huge_degree, nullptr, {512, 1024, 4096}});
    knobs.push_back({&grus_tuning::ctas_per_sm, nullptr, {0, 2, 3}});
  }
  grus_tuning best;
  grus_graph_get_tuning(g, &best);
  auto measure = [&](const grus_tuning &t, float *ms) -> int {
    int rc = grus_graph_set_tuning(g, &t);
    if (rc) return rc;
    float bestt = 1e30f;
    for (int r = 0; r < reps + 1; ++r) {  // first run warms the workspace up
      grus_stats st;
      rc = algo == GRUS_ALGO_BFS ? grus_bfs(g, src, out, &st, nullptr)
                                 : grus_sssp(g, src, out, &st, nullptr);
      if (rc) return rc;
      if (r) bestt = std::min(bestt, st.device_ms);
    }
    *ms = bestt;
    return GRUS_OK;
  };
  float best_ms = 0.f;
  int rc = measure(best, &best_ms);
  for (const Knob &k : knobs) {
    if (rc) break;
    for (double v : k.values) {
      grus_tuning cand = best;
      set_knob(cand, k, v);
      float ms = 0.f;
      rc = measure(cand, &ms);
      if (rc) break;
      if (ms < best_ms) {
        best_ms = ms;
        best = cand;
      }
    }
  }
  cudaFree(out);
  if (rc) return rc;
  rc = grus_graph_set_tuning(g, &best);
  if (rc) return rc;
  if (best_out) *best_out = best;
  if (best_ms_out) *best_ms_out = best_ms;
  return GRUS_OK;
}

// ---------------------------------------------------------------------------
// Batched and served forms.  The same coordinate descent, over the knobs of
// grus_batch_config / grus_server_config, timed on the caller's actual query
// mix.  Every candidate gives the same results (each query's result does not
// depend on how queries are scheduled), so tuning never trades correctness.
// ---------------------------------------------------------------------------
namespace {

struct CfgKnob {
  uint32_t grus_batch_config::*b = nullptr;
  uint32_t grus_server_config::*s = nullptr;
  std::vector<uint32_t> values;
};

}  // namespace

extern "C" int grus_batch_autotune(grus_graph *const *graphs, int ngraphs,
                                   const grus_query *queries, int nq, int reps,
                                   grus_batch_config *best_out, float *best_ms_out) {
  if (!graphs || ngraphs < 1 || !queries || nq < 1 || !best_out) return GRUS_EINVAL;
  if (reps < 1) reps = 2;
  uint64_t total = 0;
  for (int i = 0; i < nq; ++i) {
    if (queries[i].graph >= (uint32_t)ngraphs || !graphs[queries[i].graph]) return GRUS_EINVAL;
    total = std::max<uint64_t>(total, queries[i].out_offset + graphs[queries[i].graph]->n);
  }
  uint32_t *out = nullptr;
  GRUS_CUDA_TRY(cudaMalloc(&out, std::max<uint64_t>(total, 1) * 4));
  std::vector<CfgKnob> knobs;
  knobs.push_back({&grus_batch_config::big_edges, nullptr,
                   {1u << 17, 1u << 19, 1u << 21, 1u << 23, 1u << 25}});
  knobs.push_back({&grus_batch_config::launch_entries, nullptr,
                   {1u, 1u << 21, 1u << 22, 1u << 23, 1u << 24}});
  knobs.push_back({&grus_batch_config::cluster_size, nullptr, {8, 16}});
  knobs.push_back({&grus_batch_config::group_sources, nullptr, {1, 8}});
  knobs.push_back({&grus_batch_config::sssp_delta, nullptr, {192, 640, 1024}});
  grus_batch_config best = *best_out;  // the caller's starting point (zeros: defaults)
  auto measure = [&](const grus_batch_config &c, float *ms) -> int {
    grus_batch *b = nullptr;
    int rc = grus_batch_create(graphs, ngraphs, &c, &b);
    if (rc) return rc;
    float bt = 1e30f;
    for (int r = 0; r < reps + 1 && !rc; ++r) {  // the first run captures the graph
      grus_stats st;
      rc = grus_batch_run(b, queries, nq, out, 1, &st, nullptr);
      if (!rc && r) bt = std::min(bt, st.device_ms);
    }
    grus_batch_free(b);
    *ms = bt;
    return rc;
  };
  float best_ms = 0.f;
  int rc = measure(best, &best_ms);
  for (const CfgKnob &k : knobs) {
    if (rc) break;
    for (uint32_t v : k.values) {
      grus_batch_config cand = best;
      cand.*(k.b) = v;
      float ms = 0.f;
      const int crc = measure(cand, &ms);
      if (crc == GRUS_EINVAL || crc == GRUS_ENOMEM) continue;  // not a valid setting here
      if (crc) {
        rc = crc;
        break;
      }
      if (ms < best_ms) {
        best_ms = ms;
        best = cand;
      }
    }
  }
  cudaFree(out);
  if (rc) return rc;
  *best_out = best;
  if (best_ms_out) *best_ms_out = best_ms;
  return GRUS_OK;
}

extern "C" int grus_server_autotune(grus_graph *const *graphs, int ngraphs,
                                    const grus_query *queries, int nq, int reps,
                                    grus_server_config *best_out, float *best_qps_out) {
  if (!graphs || ngraphs < 1 || !queries || nq < 1 || !best_out) return GRUS_EINVAL;
  if (reps < 1) reps = 1;
  for (int i = 0; i < nq; ++i)
    if (queries[i].graph >= (uint32_t)ngraphs || !graphs[queries[i].graph] ||
        queries[i].src >= graphs[queries[i].graph]->n)
      return GRUS_EINVAL;
  // outputs: a few per graph, reused in turn (the results are not read)
  constexpr int kPerGraph = 8;
  std::vector<uint32_t *> outs((size_t)ngraphs * kPerGraph, nullptr);
  int rc = GRUS_OK;
  for (int g = 0; g < ngraphs && !rc; ++g)
    for (int k = 0; k < kPerGraph && !rc; ++k)
      if (cudaMalloc(&outs[(size_t)g * kPerGraph + k], std::max<uint64_t>(graphs[g]->n, 1) * 4) !=
          cudaSuccess) {
        cudaGetLastError();
        rc = GRUS_ENOMEM;
      }
  std::vector<CfgKnob> knobs;
  knobs.push_back({nullptr, &grus_server_config::big_edges, {1u << 18, 1u << 20, 1u << 22, 1u << 24}});
  knobs.push_back({nullptr, &grus_server_config::bfs_pack_min, {0, 2, 4, 8, 16}});
  knobs.push_back({nullptr, &grus_server_config::slots, {8, 16, 32}});
  knobs.push_back({nullptr, &grus_server_config::cluster_size, {4, 8, 16}});
  grus_server_config best = *best_out;
  // saturated throughput: every query submitted at once, host clock to the
  // last completion (best of reps bursts)
  auto measure = [&](const grus_server_config &c, float *qps) -> int {
    grus_server *s = nullptr;
    int r = grus_server_create(graphs, ngraphs, &c, &s);
    if (r) return r;
    std::vector<grus_completion> comp(256);
    float bq = 0.f;
    for (int rep = 0; rep < reps + 1 && !r; ++rep) {  // the first burst warms the lanes up
      std::vector<int> per(ngraphs, 0);
      const auto t0 = std::chrono::steady_clock::now();
      for (int i = 0; i < nq && !r; ++i) {
        const grus_query &q = queries[i];
        uint32_t *o = outs[(size_t)q.graph * kPerGraph + (per[q.graph]++ % kPerGraph)];
        r = grus_server_submit(s, q.graph, q.algo, q.src, o, (uint64_t)i);
      }
      int done = 0, failed = 0;
      while (!r && done < nq) {
        const int k = grus_server_poll(s, comp.data(), (int)comp.size(), 100);
        if (k < 0) {
          r = k;
          break;
        }
        for (int j = 0; j < k; ++j) failed += comp[j].status != GRUS_OK;
        done += k;
        if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(120)) {
          set_last_error("server autotune: a burst did not finish in 120 s");
          r = GRUS_ETIMEDOUT;
        }
      }
      const double sec =
          std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (!r && failed) r = GRUS_ENOMEM;  // a setting that refuses queries is not a candidate
      if (!r && rep) bq = std::max(bq, (float)(nq / sec));
    }
    grus_server_destroy(s);
    *qps = bq;
    return r;
  };
  float best_qps = 0.f;
  if (!rc) rc = measure(best, &best_qps);
  for (const CfgKnob &k : knobs) {
    if (rc) break;
    for (uint32_t v : k.values) {
      grus_server_config cand = best;
      cand.*(k.s) = v;
      float qps = 0.f;
      const int crc = measure(cand, &qps);
      if (crc == GRUS_EINVAL || crc == GRUS_ENOMEM) continue;
      if (crc) {
        rc = crc;
        break;
      }
      if (qps > best_qps) {
        best_qps = qps;
        best = cand;
      }
    }
  }
  for (uint32_t *o : outs) cudaFree(o);
  if (rc) return rc;
  *best_out = best;
  if (best_qps_out) *best_qps_out = best_qps;
  return GRUS_OK;
}
