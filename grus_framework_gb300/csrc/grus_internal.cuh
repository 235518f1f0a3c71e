// grus_internal.cuh -- host-side internals of libgrus (sm_103a): the graph
// handle layout, per-algorithm workspace slots and error plumbing.  The
// device building blocks live in device_util.cuh.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "device_util.cuh"
#include "grus.h"

namespace grus {

constexpr uint32_t kInfinit = 4294967294u;  // include/common.cuh:52

// ---- error plumbing ------------------------------------------------------
int status_from_cuda(cudaError_t e);
int status_from_device_error(uint32_t bits);
void set_last_error(const std::string &msg);

#define GRUS_CUDA_TRY(expr)                                          \
  do {                                                               \
    cudaError_t _e = (expr);                                         \
    if (_e != cudaSuccess) {                                         \
      ::grus::set_last_error(std::string(#expr) + ": " +             \
                             cudaGetErrorString(_e));                \
      return ::grus::status_from_cuda(_e);                           \
    }                                                                \
  } while (0)

// ---- graph handle --------------------------------------------------------
struct Csr {
  uint32_t *offs = nullptr;  // n+1
  uint32_t *cols = nullptr;  // m
  uint32_t *wts = nullptr;   // m or null
};

// Per-algorithm default workspaces cached on the graph handle.
enum WsSlot { kWsBfs = 0, kWsSssp, kWsCc, kWsPr, kWsMsBfs, kWsMsSssp, kWsCount = 8 };

}  // namespace grus

struct grus_graph {
  uint64_t n = 0, m = 0;
  int device = 0;
  int mem_mode = GRUS_MEM_DEVICE;
  uint32_t flags = 0;         // GRUS_GRAPH_* bits
  uint64_t budget_bytes = 0;  // managed mode: device budget
  void *balloon = nullptr;    // managed mode: HBM held back to impose the budget
  grus::Csr csr;              // out-edges
  grus::Csr csc;              // in-edges (built on demand; aliases csr if symmetric)
  uint32_t max_deg_vertex = 0, max_deg = 0;
  // BFS pull index: per vertex {an in-neighbour of high out-degree (kNoRep
  // without in-edges), the vertex's out-degree}, built on demand
  // (grus::build_rep_locked)
  uint2 *bfs_rep = nullptr;
  float bfs_rep_ms = 0.f;
  grus_tuning tuning{};       // zero fields = library defaults
  std::mutex mu;              // guards the workspaces and the csc build
  void *ws[grus::kWsCount] = {};
  void (*ws_free[grus::kWsCount])(void *) = {};
};

namespace grus {

int graph_alloc_array(grus_graph *g, void **p, size_t bytes);
void graph_free_array(grus_graph *g, void *p);
int device_sm_count();
int l2_window(cudaStream_t s, void *base, size_t bytes);
// Share of a window of `bytes` that may persist: 1, or the persisting L2
// set-aside over the window when the window is larger (persisting lines
// beyond the set-aside would only evict one another).
float l2_hit_ratio(size_t bytes);
int build_csc_locked(grus_graph *g);
// Builds g->bfs_rep for the graph's in-edges (the CSR of a symmetric graph,
// else the CSC, which must exist); no-op when built.  Caller holds g->mu.
constexpr uint32_t kNoRep = 0xFFFFFFFFu;
int build_rep_locked(grus_graph *g);

// Effective tuning value: the graph's setting when non-zero, else `def`.
template <typename T>
inline T tune_or(T v, T def) { return v ? v : def; }

// Output buffers may be host or device memory; the call copies as needed.
bool is_device_pointer(const void *p);

int launch_persistent(const void *fn, void **args, int block, int per_sm_req,
                      int occupancy, cudaStream_t s, void *win_base, size_t win_bytes);

// Multi-source BFS (msbfs.cu): outs[i] (device memory, n entries) receives
// the depths from hsrc[i] (host array), 1 <= k <= 64.  With stats the call
// waits for the launch and checks its error word.
int msbfs_run(grus_graph *g, const uint32_t *hsrc, int k, uint32_t *const *outs,
              grus_stats *stats, cudaStream_t s);
// Multi-source SSSP (msssp.cu): as msbfs_run for distances, 1 <= k <= 32.
int msssp_run(grus_graph *g, const uint32_t *hsrc, int k, uint32_t *const *outs,
              grus_stats *stats, cudaStream_t s);

// Fewest BFS queries on one graph of m edges for which one multi-source
// launch (msbfs_run) beats as many single launches.  Measured on RMAT graphs
// with random sources: a 16-source pack costs 2.2-5.3 single launches' time
// up to 2^26 edges, 1.1 at 2^27 and 0.8 at 2^29, where 32 sources reach 1.3
// and 64 sources 2.0.
inline uint32_t bfs_pack_min(uint64_t m) {
  if (m < (1ull << 25)) return 8;
  if (m < (1ull << 27)) return 16;
  if (m < (1ull << 28)) return 24;
  return 32;
}

// Device control block of a graph's workspace for one algorithm (ctrl null
// before the algorithm's first call on the graph), for callers that launch
// without waiting and check the launch's error word later.
struct CtrlView {
  char *ctrl = nullptr;
  size_t bytes = 0, err_off = 0, bar_off = 0;
};
CtrlView bfs_ctrl(grus_graph *g);
CtrlView sssp_ctrl(grus_graph *g);
CtrlView msbfs_ctrl(grus_graph *g);
CtrlView msssp_ctrl(grus_graph *g);
CtrlView pr_ctrl(grus_graph *g);

// Multi-graph multi-source SSSP (msssp.cu): ONE whole-GPU launch over ng
// (<= 64) weighted graphs, graph g with kq[g] (1..32) sources; srcs and outs
// list the sources and their n_g-entry device outputs graph after graph.
// The workspace belongs to the caller: reserve it for `regions` launches of
// at most max_v vertices, max_m edges and ks (8/16/32) sources per graph
// before the first launch of a run; launch i of a run uses region i.  *cv
// receives the launch's control block (error word).
int msssp_union_reserve(void **ws, int regions, uint64_t max_v, uint64_t max_m, uint32_t ks);
int msssp_union_run(void *ws, int region, grus_graph *const *gs, int ng, const uint32_t *kq,
                    const uint32_t *srcs, uint32_t *const *outs, uint32_t delta, cudaStream_t s,
                    CtrlView *cv);
void msssp_union_free(void *ws);
// Clears the control blocks after a failed launch.
void msssp_union_reset(void *ws);

}  // namespace grus
