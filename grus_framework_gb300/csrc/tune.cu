// tune.cu -- autotuner for the persistent traversal kernels.
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
