// batch.cuh -- shared declarations of the cluster-worker query engine
// (batch.cu) and its users (the batch C ABI and the query server).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "grus.h"

struct grus_graph;

namespace grus {

constexpr int kBatchBlock = 256;
constexpr uint32_t kBatchInfinit = 4294967294u;
constexpr uint32_t kAlgoBfs = GRUS_ALGO_BFS, kAlgoSssp = GRUS_ALGO_SSSP;
// Internal task kind: k SSSP queries on one graph run as one multi-source
// traversal; Task.src = first member, Task.pad = k.
constexpr uint32_t kAlgoSsspMulti = 2;
constexpr int kMaxGroup = 32;

// Device view of one resident graph.
struct GraphDesc {
  const uint32_t *offs, *cols, *wts;
  uint32_t n, flags;
  uint64_t m;
};

// One query: output = out_base + out_off (n of the graph entries).
struct Task {
  uint32_t graph, algo, src, pad;
  unsigned long long out_off;
};

// Device state of `workers` cluster workers, each sized for graphs of up to
// (max_n, max_m).
struct BatchState {
  uint32_t *bitmaps = nullptr, *lists = nullptr;
  uint4 *chunks = nullptr;
  void *ctl = nullptr;
  uint32_t *counter = nullptr, *err = nullptr;
  uint64_t Wp = 0;
  uint32_t cap = 0, chunk_cap = 0;
  int workers = 0;
  // multi-source SSSP state per worker: distance matrix (ms_n * ms_ks), near
  // and far masks (3 * ms_n), work entries (ms_ent_cap)
  uint32_t *ms_d = nullptr, *ms_masks = nullptr;
  uint4 *ms_ent = nullptr;
  uint64_t ms_n = 0;
  uint32_t ms_ks = 0, ms_ent_cap = 0;
  int ms_workers = 0;
  int reserve(int nworkers, uint64_t max_n, uint64_t max_m, uint32_t huge);
  int reserve_multi(int nworkers, uint64_t max_n, uint64_t max_m, uint32_t ks);
  void release();
  void release_multi();
  static size_t bytes_per_worker(uint64_t max_n, uint64_t max_m, uint32_t huge);
};

int batch_occupancy(int cluster, int *workers);
// Runs tasks[0..ntasks) with workers [worker0, worker0 + nworkers) of `st`.
// Multi-source tasks read their sources from msrc[Task.src ..] and write
// source i to out + moff[Task.src + i] (both null when there are none).
int batch_launch(BatchState &st, int worker0, int nworkers, int cluster, const GraphDesc *graphs,
                 const Task *tasks, uint32_t ntasks, uint32_t *out, uint32_t huge, uint32_t delta,
                 uint32_t *counter, cudaStream_t s, const uint32_t *msrc = nullptr,
                 const unsigned long long *moff = nullptr);
GraphDesc describe(const grus_graph *g);

}  // namespace grus
