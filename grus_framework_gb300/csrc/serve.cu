// serve.cu -- a query server over device-resident graphs (continuous batching).
//
// Requests (graph, BFS|SSSP, source, device output) are queued by
// grus_server_submit from any host thread and served by two lanes.
//   Small graphs: a scheduler thread admits each request into a worker slot:
//     one cluster worker of the batch engine (batch.cu) with its own
//     per-query device state and CUDA stream.  A slot's state is allocated the
//     first time it is used, and only if free HBM (cudaMemGetInfo) covers it
//     plus a reserve -- admission by free HBM.  Each admitted query is one
//     single-worker launch on its slot's stream, so queries that arrive while
//     others run start as soon as a slot is free and overlap on the device.
//   Big graphs (at least big_edges edges): one cluster would take many times
//     longer than the whole GPU, so a second thread runs the whole-GPU
//     persistent kernels (grus_bfs / grus_sssp) one launch at a time, and
//     packs the queued SSSP requests on the same graph -- up to 32 -- into one
//     multi-source launch (msssp.cu) that writes each request's own output.
//     BFS requests on one graph are packed -- up to 64, msbfs.cu -- once
//     enough are queued for the pack to beat single direction-optimising
//     launches on a graph of that size, else they run alone.
//     A graph's workspace is allocated only if free HBM covers it plus the
//     reserve.  Up to four launches are queued on the lane's stream; each
//     copies its error word to pinned memory and records an event, so the
//     lane never waits on the host between queries.
// Completion is observed with an event per slot (small lane) or per queued
// launch (big lane); latency is completion time minus
// submission time on the host clock.
// The reference has no serving path (one query per process run).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "batch.cuh"
#include "grus_internal.cuh"

namespace grus {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t tag;
  uint32_t graph, algo, src;
  uint32_t *out;
  Clock::time_point t_submit;
};

struct Slot {
  BatchState state;        // one worker
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  Task *d_task = nullptr;
  Task *h_task = nullptr;  // pinned staging
  uint32_t *h_err = nullptr;  // pinned copy of the worker's error word
  uint32_t *counter = nullptr;
  bool ready = false;      // device state allocated
  bool busy = false;
  Request req{};
};

}  // namespace
}  // namespace grus

struct grus_server {
  std::vector<grus_graph *> graphs;
  std::vector<uint8_t> big;  // per graph: served by the whole-GPU lane
  grus::GraphDesc *d_graphs = nullptr;
  uint64_t max_n = 0, max_m = 0;  // over the small graphs
  uint64_t big_edges = 1ull << 20;
  uint32_t bfs_pack_min = 0;  // 0: grus::bfs_pack_min(m)
  int cluster = 8;
  uint32_t huge = 1024, delta = 192;
  uint64_t reserve = 1ull << 30;
  std::vector<grus::Slot> slots;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<grus::Request> pending;      // small lane
  std::deque<grus::Request> big_pending;  // big lane
  std::deque<grus_completion> completed;
  std::thread worker, big_worker;
  cudaStream_t big_stream = nullptr;
  uint64_t big_launches = 0, big_queries = 0;
  std::atomic<uint64_t> kernel_launches{0};  // kernels launched for queries, both lanes
  std::atomic<bool> stop{false};
  int device = 0;
  uint64_t admitted = 0, finished = 0, rejected = 0;
  int slots_ready = 0;
  int error = GRUS_OK;
};

namespace grus {
namespace {

int slot_prepare(grus_server *s, Slot &sl) {
  if (sl.ready) return GRUS_OK;
  size_t free_b = 0, total_b = 0;
  GRUS_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
  const size_t need = BatchState::bytes_per_worker(s->max_n, s->max_m, s->huge) + 4096;
  if (free_b < need + s->reserve) return GRUS_ENOMEM;  // not admitted: wait for a slot
  int rc = sl.state.reserve(1, s->max_n, s->max_m, s->huge);
  if (rc) return rc;
  GRUS_CUDA_TRY(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking));
  GRUS_CUDA_TRY(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
  GRUS_CUDA_TRY(cudaMalloc(&sl.d_task, sizeof(Task)));
  GRUS_CUDA_TRY(cudaMallocHost(&sl.h_task, sizeof(Task)));
  GRUS_CUDA_TRY(cudaMallocHost(&sl.h_err, 4));
  GRUS_CUDA_TRY(cudaMalloc(&sl.counter, 4));
  GRUS_CUDA_TRY(cudaMemset(sl.state.err, 0, 4));
  sl.ready = true;
  ++s->slots_ready;
  return GRUS_OK;
}

int slot_launch(grus_server *s, Slot &sl, const Request &r) {
  Task &t = *sl.h_task;
  t.graph = r.graph;
  t.algo = r.algo;
  t.src = r.src;
  t.pad = 0;
  t.out_off = 0;
  GRUS_CUDA_TRY(cudaMemcpyAsync(sl.d_task, sl.h_task, sizeof(Task), cudaMemcpyHostToDevice, sl.stream));
  GRUS_CUDA_TRY(cudaMemsetAsync(sl.counter, 0, 4, sl.stream));
  int rc = batch_launch(sl.state, 0, 1, s->cluster, s->d_graphs, sl.d_task, 1, r.out, s->huge,
                        s->delta, sl.counter, sl.stream);
  if (rc) return rc;
  s->kernel_launches += 1;
  GRUS_CUDA_TRY(cudaMemcpyAsync(sl.h_err, sl.state.err, 4, cudaMemcpyDeviceToHost, sl.stream));
  GRUS_CUDA_TRY(cudaMemsetAsync(sl.state.err, 0, 4, sl.stream));
  GRUS_CUDA_TRY(cudaEventRecord(sl.done, sl.stream));
  return GRUS_OK;
}

void scheduler(grus_server *s) {
  cudaSetDevice(s->device);
  while (!s->stop.load()) {
    bool idle = true;
    // completions
    for (auto &sl : s->slots) {
      if (!sl.busy) continue;
      const cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaErrorNotReady) continue;
      idle = false;
      grus_completion c;
      std::memset(&c, 0, sizeof(c));
      c.tag = sl.req.tag;
      c.status = q == cudaSuccess ? GRUS_OK : status_from_cuda(q);
      if (q == cudaSuccess && *sl.h_err) c.status = status_from_device_error(*sl.h_err);
      const auto now = Clock::now();
      c.latency_us = std::chrono::duration<double, std::micro>(now - sl.req.t_submit).count();
      sl.busy = false;
      std::lock_guard<std::mutex> lk(s->mu);
      s->completed.push_back(c);
      ++s->finished;
      s->cv.notify_all();
    }
    // admissions
    for (auto &sl : s->slots) {
      if (sl.busy) continue;
      Request r;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->pending.empty()) break;
        r = s->pending.front();
      }
      if (!sl.ready) {
        const int rc = slot_prepare(s, sl);
        if (rc == GRUS_ENOMEM && s->slots_ready > 0) continue;  // wait for a busy slot
        if (rc == GRUS_ENOMEM) {
          // not even one query fits in free HBM: refuse it rather than queue forever
          grus_completion c;
          std::memset(&c, 0, sizeof(c));
          c.tag = r.tag;
          c.status = GRUS_ENOMEM;
          std::lock_guard<std::mutex> lk(s->mu);
          s->pending.pop_front();
          s->completed.push_back(c);
          ++s->finished;
          ++s->rejected;
          s->cv.notify_all();
          continue;
        }
        if (rc) {
          std::lock_guard<std::mutex> lk(s->mu);
          s->error = rc;
          continue;
        }
      }
      {
        std::lock_guard<std::mutex> lk(s->mu);
        s->pending.pop_front();
        ++s->admitted;
      }
      sl.req = r;
      const int rc = slot_launch(s, sl, r);
      if (rc) {
        grus_completion c;
        std::memset(&c, 0, sizeof(c));
        c.tag = r.tag;
        c.status = rc;
        std::lock_guard<std::mutex> lk(s->mu);
        s->completed.push_back(c);
        ++s->finished;
        s->cv.notify_all();
        continue;
      }
      sl.busy = true;
      idle = false;
    }
    if (idle) {
      std::unique_lock<std::mutex> lk(s->mu);
      bool any_busy = false;
      for (auto &sl : s->slots) any_busy |= sl.busy;
      if (!any_busy && s->pending.empty())
        s->cv.wait_for(lk, std::chrono::milliseconds(2));
      else
        std::this_thread::yield();
    }
  }
}

// Rough device bytes of a graph's whole-GPU workspace for `algo` (BFS also
// covers the multi-source one), used for admission before the first launch.
size_t big_workspace_bytes(const grus_graph *g, uint32_t algo, bool multi) {
  const size_t n = g->n, m = g->m;
  if (algo == GRUS_ALGO_SSSP && multi) return 128 * n + 16 * n + m / 8 + (1u << 20);
  // a BFS pack also keeps 64 depth bytes per vertex
  return (algo == GRUS_ALGO_SSSP ? 20 * n : (multi ? 104 * n : 40 * n)) + m / 32 + (1u << 20);
}

bool big_workspace_ready(const grus_graph *g, uint32_t algo, bool multi) {
  if (algo == GRUS_ALGO_SSSP) return (multi ? g->ws[kWsMsSssp] : g->ws[kWsSssp]) != nullptr;
  if (multi) return g->ws[kWsMsBfs] != nullptr;
  return multi ? g->ws[kWsMsBfs] != nullptr : g->ws[kWsBfs] != nullptr;
}

void complete(grus_server *s, const Request &r, int status, Clock::time_point now) {
  grus_completion c;
  std::memset(&c, 0, sizeof(c));
  c.tag = r.tag;
  c.status = status;
  c.latency_us = std::chrono::duration<double, std::micro>(now - r.t_submit).count();
  s->completed.push_back(c);
  ++s->finished;
}

// One whole-GPU launch of the big lane, in flight on the lane's stream.
struct BigJob {
  std::vector<Request> group;
  cudaEvent_t done = nullptr;
  uint32_t *h_err = nullptr;  // pinned copy of the launch's error word
  CtrlView ctrl;
};

// Launches one group without waiting: the kernel, a copy of its error word
// into pinned memory and a reset of that word, then an event.  Launches
// queue back to back on the lane's stream, so the GPU runs them without the
// host round trip between queries.
int big_launch(grus_server *s, BigJob &j) {
  const Request &r = j.group[0];
  grus_graph *g = s->graphs[r.graph];
  const bool multi = j.group.size() > 1;
  if (!big_workspace_ready(g, r.algo, multi)) {
    size_t free_b = 0, total_b = 0;
    GRUS_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    if (free_b < big_workspace_bytes(g, r.algo, multi) + s->reserve) return GRUS_ENOMEM;
  }
  int rc;
  if (!multi) {
    rc = r.algo == GRUS_ALGO_SSSP ? grus_sssp(g, r.src, r.out, nullptr, s->big_stream)
                                  : grus_bfs(g, r.src, r.out, nullptr, s->big_stream);
  } else {
    uint32_t srcs[64];
    uint32_t *outs[64];
    for (size_t i = 0; i < j.group.size(); ++i) {
      srcs[i] = j.group[i].src;
      outs[i] = j.group[i].out;
    }
    rc = r.algo == GRUS_ALGO_SSSP
             ? msssp_run(g, srcs, (int)j.group.size(), outs, nullptr, s->big_stream)
             : msbfs_run(g, srcs, (int)j.group.size(), outs, nullptr, s->big_stream);
  }
  if (rc) return rc;
  // a single BFS is the persistent kernel and its narrow-tail kernel
  s->kernel_launches += (!multi && r.algo != GRUS_ALGO_SSSP) ? 2 : 1;
  j.ctrl = r.algo == GRUS_ALGO_SSSP ? (multi ? msssp_ctrl(g) : sssp_ctrl(g))
                                    : (multi ? msbfs_ctrl(g) : bfs_ctrl(g));
  *j.h_err = 0;
  if (j.ctrl.ctrl) {
    GRUS_CUDA_TRY(cudaMemcpyAsync(j.h_err, j.ctrl.ctrl + j.ctrl.err_off, 4, cudaMemcpyDeviceToHost,
                                  s->big_stream));
    GRUS_CUDA_TRY(cudaMemsetAsync(j.ctrl.ctrl + j.ctrl.err_off, 0, 4, s->big_stream));
  }
  GRUS_CUDA_TRY(cudaEventRecord(j.done, s->big_stream));
  return GRUS_OK;
}

void big_finish(grus_server *s, std::vector<Request> &group, int rc) {
  const auto now = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (rc == GRUS_ENOMEM) {
    s->rejected += group.size();
  } else {
    ++s->big_launches;
    s->big_queries += group.size();
    s->admitted += group.size();
  }
  for (const Request &q : group) complete(s, q, rc, now);
  s->cv.notify_all();
}

void big_scheduler(grus_server *s) {
  cudaSetDevice(s->device);
  constexpr int kDepth = 4;  // launches queued on the lane's stream
  std::vector<BigJob> jobs(kDepth);
  for (BigJob &j : jobs) {
    cudaError_t e = cudaEventCreateWithFlags(&j.done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost(&j.h_err, 4);
    if (e != cudaSuccess) {
      // no lane state: fail every big-graph request from now on
      cudaGetLastError();
      std::lock_guard<std::mutex> lk(s->mu);
      s->error = status_from_cuda(e);
      set_last_error(std::string("server big lane: ") + cudaGetErrorString(e));
      for (const Request &q : s->big_pending) complete(s, q, s->error, Clock::now());
      s->big_pending.clear();
      s->cv.notify_all();
      for (BigJob &k : jobs) {
        if (k.done) cudaEventDestroy(k.done);
        if (k.h_err) cudaFreeHost(k.h_err);
      }
      return;
    }
    j.group.reserve(64);
  }
  std::deque<int> inflight, spare;
  for (int i = 0; i < kDepth; ++i) spare.push_back(i);
  while (!s->stop.load()) {
    bool progress = false;
    // completions, in launch order
    while (!inflight.empty()) {
      BigJob &j = jobs[inflight.front()];
      const cudaError_t q = cudaEventQuery(j.done);
      if (q == cudaErrorNotReady) break;
      int rc = q == cudaSuccess ? GRUS_OK : status_from_cuda(q);
      if (rc == GRUS_OK && *j.h_err) {
        rc = status_from_device_error(*j.h_err);
        // the failed launch may have left its barrier state behind: drain the
        // lane and clear the control block before the next launch on it
        cudaStreamSynchronize(s->big_stream);
        if (j.ctrl.ctrl) cudaMemset(j.ctrl.ctrl, 0, j.ctrl.bytes);
      }
      big_finish(s, j.group, rc);
      spare.push_back(inflight.front());
      inflight.pop_front();
      progress = true;
    }
    // launches
    while (!spare.empty()) {
      BigJob &j = jobs[spare.front()];
      j.group.clear();
      {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->big_pending.empty()) break;
        const Request first = s->big_pending.front();
        s->big_pending.pop_front();
        j.group.push_back(first);
        // SSSP requests on one graph share a multi-source launch (it
        // amortises the adjacency reads over up to 32 sources); BFS requests
        // share one (up to 64) only when enough are queued: a direction-
        // optimising BFS skips most edges, so a small pack on a big graph
        // costs more than the single launches it replaces
        size_t cap = 32;
        if (first.algo == GRUS_ALGO_BFS) {
          size_t same = 1;
          for (const Request &q : s->big_pending)
            if (q.graph == first.graph && q.algo == GRUS_ALGO_BFS && ++same >= 64) break;
          const uint32_t pmin =
              s->bfs_pack_min ? s->bfs_pack_min : bfs_pack_min(s->graphs[first.graph]->m);
          cap = same >= pmin ? 64 : 1;
        }
        for (auto it = s->big_pending.begin(); it != s->big_pending.end() && j.group.size() < cap;) {
          if (it->graph == first.graph && it->algo == first.algo) {
            j.group.push_back(*it);
            it = s->big_pending.erase(it);
          } else {
            ++it;
          }
        }
      }
      progress = true;
      const int rc = big_launch(s, j);
      if (rc) {
        big_finish(s, j.group, rc);
        continue;
      }
      inflight.push_back(spare.front());
      spare.pop_front();
    }
    if (progress) continue;
    std::unique_lock<std::mutex> lk(s->mu);
    if (inflight.empty())
      s->cv.wait_for(lk, std::chrono::milliseconds(50),
                     [&] { return s->stop.load() || !s->big_pending.empty(); });
    else
      s->cv.wait_for(lk, std::chrono::microseconds(20));
  }
  cudaStreamSynchronize(s->big_stream);
  for (BigJob &j : jobs) {
    cudaEventDestroy(j.done);
    cudaFreeHost(j.h_err);
  }
}

}  // namespace
}  // namespace grus

using namespace grus;

extern "C" {

int grus_server_create(grus_graph *const *graphs, int ngraphs, const grus_server_config *cfg,
                       grus_server **out) {
  if (!graphs || ngraphs < 1 || !out) return GRUS_EINVAL;
  grus_server *s = new grus_server();
  cudaGetDevice(&s->device);
  std::vector<GraphDesc> descs;
  int nslots = 16;
  if (cfg) {
    if (cfg->slots) nslots = (int)cfg->slots;
    if (cfg->cluster_size) s->cluster = (int)cfg->cluster_size;
    if (cfg->hbm_reserve_bytes) s->reserve = cfg->hbm_reserve_bytes;
    if (cfg->sssp_delta) s->delta = cfg->sssp_delta;
    if (cfg->big_edges) s->big_edges = cfg->big_edges == 0xFFFFFFFFu ? ~0ull : cfg->big_edges;
    s->bfs_pack_min = cfg->bfs_pack_min;
  }
  bool any_small = false;
  for (int i = 0; i < ngraphs; ++i) {
    if (!graphs[i]) {
      delete s;
      return GRUS_EINVAL;
    }
    s->graphs.push_back(graphs[i]);
    descs.push_back(describe(graphs[i]));
    const bool big = graphs[i]->m >= s->big_edges;
    s->big.push_back(big ? 1 : 0);
    if (!big) {
      any_small = true;
      s->max_n = std::max<uint64_t>(s->max_n, graphs[i]->n);
      s->max_m = std::max<uint64_t>(s->max_m, graphs[i]->m);
    }
  }
  if (s->cluster < 1 || s->cluster > 16 || nslots < 1 || nslots > 1024) {
    delete s;
    return GRUS_EINVAL;
  }
  s->slots.resize(nslots);
  int probe_workers = 0;
  if (any_small && (batch_occupancy(s->cluster, &probe_workers) != GRUS_OK || probe_workers < 1)) {
    delete s;
    set_last_error("server: no cluster of this size can be resident");
    return GRUS_EINVAL;
  }
  cudaError_t e = cudaMalloc(&s->d_graphs, ngraphs * sizeof(GraphDesc));
  if (e == cudaSuccess)
    e = cudaMemcpy(s->d_graphs, descs.data(), ngraphs * sizeof(GraphDesc), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(s->d_graphs);
    delete s;
    set_last_error(cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  // The big lane's persistent launches need all their CTAs resident at once
  // while the small lane keeps launching cluster workers on other streams:
  // at the highest stream priority their pending CTAs take freed SM
  // resources before new small-lane work does, so a grid barrier is never
  // left waiting behind a stream of small launches.
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  e = cudaStreamCreateWithPriority(&s->big_stream, cudaStreamNonBlocking, prio_greatest);
  if (e != cudaSuccess) {
    cudaFree(s->d_graphs);
    delete s;
    set_last_error(cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  s->worker = std::thread(scheduler, s);
  s->big_worker = std::thread(big_scheduler, s);
  *out = s;
  return GRUS_OK;
}

int grus_server_submit(grus_server *s, uint32_t graph, uint32_t algo, uint32_t src, uint32_t *out,
                       uint64_t tag) {
  if (!s || !out || graph >= s->graphs.size() || algo > GRUS_ALGO_SSSP) return GRUS_EINVAL;
  const grus_graph *g = s->graphs[graph];
  if (src >= g->n) return GRUS_EINVAL;
  if (algo == GRUS_ALGO_SSSP && !g->csr.wts) return GRUS_EINVAL;
  if (!is_device_pointer(out)) {
    set_last_error("server outputs must be device (or managed) memory");
    return GRUS_EINVAL;
  }
  Request r{tag, graph, algo, src, out, Clock::now()};
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->error) return s->error;
    (s->big[graph] ? s->big_pending : s->pending).push_back(r);
  }
  s->cv.notify_all();
  return GRUS_OK;
}

int grus_server_poll(grus_server *s, grus_completion *out, int max, int wait_ms) {
  if (!s || (!out && max > 0) || max < 0) return GRUS_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->completed.empty() && wait_ms > 0)
    s->cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->completed.empty(); });
  int k = 0;
  while (k < max && !s->completed.empty()) {
    out[k++] = s->completed.front();
    s->completed.pop_front();
  }
  return k;
}

int grus_server_get_stats(grus_server *s, grus_server_stats *st) {
  if (!s || !st) return GRUS_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(st, 0, sizeof(*st));
  st->pending = s->pending.size() + s->big_pending.size();
  st->submitted = s->admitted + s->rejected + st->pending;
  st->admitted = s->admitted;
  st->completed = s->finished;
  st->big_launches = s->big_launches;
  st->big_queries = s->big_queries;
  st->kernel_launches = s->kernel_launches.load();
  st->slots_ready = (uint32_t)s->slots_ready;
  st->rejected = s->rejected;
  st->slots = (uint32_t)s->slots.size();
  return GRUS_OK;
}

int grus_server_destroy(grus_server *s) {
  if (!s) return GRUS_EINVAL;
  s->stop.store(true);
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  if (s->big_worker.joinable()) s->big_worker.join();
  if (s->big_stream) {
    cudaStreamSynchronize(s->big_stream);
    cudaStreamDestroy(s->big_stream);
  }
  for (auto &sl : s->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    sl.state.release();
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.done) cudaEventDestroy(sl.done);
    cudaFree(sl.d_task);
    if (sl.h_task) cudaFreeHost(sl.h_task);
    if (sl.h_err) cudaFreeHost(sl.h_err);
    cudaFree(sl.counter);
  }
  cudaFree(s->d_graphs);
  delete s;
  return GRUS_OK;
}

}  // extern "C"
