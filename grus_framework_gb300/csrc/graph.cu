// graph.cu -- graph handles: HBM / managed CSR, the .gr loader, the budget
// balloon, device CSR->CSC transpose, info and copy-back.
//
// Reference behaviour replaced (paths relative to the Grus project root):
//   include/graph_loader.cuh:65-166  ReadGraphGR / Load  (Galois v1 .gr)
//   include/graph.cuh:170-251        Set_Mem_Policy      (UM prefetch/advise)
//   include/graph.cuh:273-320        csr_tocsc / CSR2CSC (host-serial, no weights)
//   tools/mem_limit.cu:1-19          HBM balloon imposing a device budget
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "grus_internal.cuh"

namespace grus {

static thread_local std::string g_last_error;

void set_last_error(const std::string &msg) { g_last_error = msg; }

int status_from_cuda(cudaError_t e) {
  if (e == cudaSuccess) return GRUS_OK;
  if (e == cudaErrorMemoryAllocation) return GRUS_ENOMEM;
  if (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice) return GRUS_ENODEV;
  if (e == cudaErrorInvalidValue) return GRUS_EINVAL;
  return GRUS_ECUDA;
}

int status_from_device_error(uint32_t bits) {
  if (bits & kErrTimeout) {
    set_last_error("a device-side wait exceeded its time limit");
    return GRUS_ETIMEDOUT;
  }
  if (bits & kErrAborted) {
    set_last_error("the launch was abandoned at a grid barrier after a wait timed out");
    return GRUS_ETIMEDOUT;
  }
  if (bits & (kErrOverflow | kErrLevels)) {
    set_last_error("a device queue or level bound overflowed");
    return GRUS_EOVERFLOW;
  }
  return GRUS_OK;
}

int device_sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  if (!cached[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = v;
  }
  return cached[dev];
}

bool is_device_pointer(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int graph_alloc_array(grus_graph *g, void **p, size_t bytes) {
  if (bytes == 0) bytes = 4;
  if (g->mem_mode == GRUS_MEM_MANAGED) {
    GRUS_CUDA_TRY(cudaMallocManaged(p, bytes));
  } else {
    GRUS_CUDA_TRY(cudaMalloc(p, bytes));
  }
  return GRUS_OK;
}

void graph_free_array(grus_graph *, void *p) {
  if (p) cudaFree(p);
}

// Scan of in-degrees / row expansion helpers for the transpose.
__global__ void k_expand_rows(const uint32_t *__restrict__ offs, uint64_t n,
                              uint32_t *__restrict__ rowid) {
  // one warp per row; lanes write the row id over the row's edge range
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t u = warp; u < n; u += nwarps) {
    const uint32_t b = offs[u], e = offs[u + 1];
    for (uint32_t x = b + lane; x < e; x += 32) rowid[x] = (uint32_t)u;
  }
}

__global__ void k_iota(uint32_t *__restrict__ a, uint64_t m) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x)
    a[i] = (uint32_t)i;
}

// Boundaries of sorted keys -> offsets: offs[x] = first index whose key >= x.
__global__ void k_offsets_from_sorted(const uint32_t *__restrict__ keys,
                                      uint64_t m, uint64_t n,
                                      uint32_t *__restrict__ offs) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e <= m;
       e += (uint64_t)gridDim.x * blockDim.x) {
    const int64_t prev = e == 0 ? -1 : (int64_t)keys[e - 1];
    const int64_t cur = e == m ? (int64_t)n : (int64_t)keys[e];
    for (int64_t x = prev + 1; x <= cur && x <= (int64_t)n; ++x) offs[x] = (uint32_t)e;
  }
}

__global__ void k_gather_csc(const uint32_t *__restrict__ perm,
                             const uint32_t *__restrict__ rowid,
                             const uint32_t *__restrict__ wts, uint64_t m,
                             uint32_t *__restrict__ t_cols,
                             uint32_t *__restrict__ t_wts) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t e = perm[i];
    t_cols[i] = rowid[e];
    if (t_wts) t_wts[i] = wts[e];
  }
}

__global__ void k_u64_to_u32_offsets(const uint64_t *__restrict__ ends,
                                     uint64_t n, uint32_t *__restrict__ offs,
                                     uint32_t *__restrict__ bad, uint64_t m) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t e = ends[i];
    const uint64_t p = i ? ends[i - 1] : 0;
    if (e > m || e < p) atomicOr(bad, 1u);
    offs[i + 1] = (uint32_t)e;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) offs[0] = 0;
}

__global__ void k_check_cols(const uint32_t *__restrict__ cols, uint64_t m,
                             uint64_t n, uint32_t *__restrict__ bad) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x)
    if (cols[i] >= n) atomicOr(bad, 2u);
}

__global__ void k_fill_u32(uint32_t *__restrict__ a, uint64_t m, uint32_t v) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x)
    a[i] = v;
}

// Max out-degree vertex, first index on ties (include/graph_loader.cuh:132-137):
// packed key (degree << 32) | ~index, reduced with atomicMax.
__global__ void k_max_degree(const uint32_t *__restrict__ offs, uint64_t n,
                             unsigned long long *__restrict__ best) {
  unsigned long long local = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long d = offs[i + 1] - offs[i];
    const unsigned long long key = (d << 32) | (0xFFFFFFFFull - i);
    local = key > local ? key : local;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_down_sync(0xffffffffu, local, o);
    local = t > local ? t : local;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(best, local);
}

// One CTA enters the persistent kernels' grid barrier; the host presets its
// arrival count so the episode cannot complete and the wait must time out.
__global__ void k_wait_limit(GridBarrier *bar, uint32_t *err, uint64_t timeout_ns) {
  grid_sync(bar, err, timeout_ns);
}

// The same one-CTA wait on a workspace's own control block: the CTA first
// counts one phantom arrival, so its wait must time out, and the block is
// left as a launch that timed out leaves it (abort raised, arrival count
// stale, error word set).
__global__ void k_stale_barrier(GridBarrier *bar, uint32_t *err, uint64_t timeout_ns) {
  if (threadIdx.x == 0) {
    bar->count = 1u;
    bar->abort = 0u;
    __threadfence();
  }
  grid_sync(bar, err, timeout_ns);
}

static int grid_for(uint64_t work, int block = 256) {
  const int sms = std::max(device_sm_count(), 1);
  const uint64_t want = (work + block - 1) / block;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)sms * 16));
}

int finalize_graph(grus_graph *g) {
  unsigned long long *d_best = nullptr, best = 0;
  GRUS_CUDA_TRY(cudaMalloc(&d_best, sizeof(unsigned long long)));
  cudaMemset(d_best, 0, sizeof(unsigned long long));
  if (g->n) k_max_degree<<<grid_for(g->n), 256>>>(g->csr.offs, g->n, d_best);
  cudaError_t e = cudaMemcpy(&best, d_best, sizeof(best), cudaMemcpyDeviceToHost);
  cudaFree(d_best);
  GRUS_CUDA_TRY(e);
  g->max_deg = (uint32_t)(best >> 32);
  g->max_deg_vertex = g->n ? (uint32_t)(0xFFFFFFFFull - (best & 0xFFFFFFFFull)) : 0;
  if (g->max_deg == 0) g->max_deg_vertex = 0;
  return GRUS_OK;
}

// Managed mode: the reference's --opt policy (include/graph.cuh:173-205):
// prefetch the offsets, then as much of the columns (and weights) as the
// device budget allows, and mark everything AccessedBy the device so the rest
// is read in place over the host link rather than faulted back and forth.
// The budget itself is imposed the way tools/mem_limit.cu does it: a balloon
// cudaMalloc leaves only `budget` bytes of free HBM beside what is already
// allocated.
int apply_mem_policy(grus_graph *g, cudaStream_t s) {
  if (g->mem_mode != GRUS_MEM_MANAGED) return GRUS_OK;
  int dev = 0;
  GRUS_CUDA_TRY(cudaGetDevice(&dev));
  cudaMemLocation loc{};
  loc.type = cudaMemLocationTypeDevice;
  loc.id = dev;
  const uint64_t ob = (g->n + 1) * 4ull, cb = g->m * 4ull;
  const uint64_t wb = g->csr.wts ? g->m * 4ull : 0ull;
  const uint64_t total = ob + cb + wb;
  uint64_t budget = g->budget_bytes ? g->budget_bytes : total;
  GRUS_CUDA_TRY(cudaMemAdvise(g->csr.offs, ob, cudaMemAdviseSetAccessedBy, loc));
  GRUS_CUDA_TRY(cudaMemAdvise(g->csr.cols, cb ? cb : 4, cudaMemAdviseSetAccessedBy, loc));
  if (wb) GRUS_CUDA_TRY(cudaMemAdvise(g->csr.wts, wb, cudaMemAdviseSetAccessedBy, loc));
  uint64_t left = budget;
  const uint64_t po = std::min(ob, left);
  if (po) GRUS_CUDA_TRY(cudaMemPrefetchAsync(g->csr.offs, po, loc, 0, s));
  left -= po;
  if (wb) {
    const uint64_t half = left / 2;
    const uint64_t pc = std::min(cb, half), pw = std::min(wb, left - pc);
    if (pc) GRUS_CUDA_TRY(cudaMemPrefetchAsync(g->csr.cols, pc, loc, 0, s));
    if (pw) GRUS_CUDA_TRY(cudaMemPrefetchAsync(g->csr.wts, pw, loc, 0, s));
  } else {
    const uint64_t pc = std::min(cb, left);
    if (pc) GRUS_CUDA_TRY(cudaMemPrefetchAsync(g->csr.cols, pc, loc, 0, s));
  }
  // whatever lies beyond the budget starts on the host, wherever it was
  // written (a graph generated on the device is first touched there)
  if (g->budget_bytes) {
    cudaMemLocation host{};
    host.type = cudaMemLocationTypeHost;
    host.id = 0;
    const uint64_t po2 = std::min(ob, budget);
    uint64_t left2 = budget - po2;
    uint64_t pc2 = 0, pw2 = 0;
    if (wb) {
      pc2 = std::min(cb, left2 / 2);
      pw2 = std::min(wb, left2 - pc2);
    } else {
      pc2 = std::min(cb, left2);
    }
    if (ob > po2)
      GRUS_CUDA_TRY(cudaMemPrefetchAsync((char *)g->csr.offs + po2, ob - po2, host, 0, s));
    if (cb > pc2)
      GRUS_CUDA_TRY(cudaMemPrefetchAsync((char *)g->csr.cols + pc2, cb - pc2, host, 0, s));
    if (wb > pw2)
      GRUS_CUDA_TRY(cudaMemPrefetchAsync((char *)g->csr.wts + pw2, wb - pw2, host, 0, s));
  }
  GRUS_CUDA_TRY(cudaStreamSynchronize(s));
  if (g->budget_bytes && !g->balloon) {
    size_t free_b = 0, total_b = 0;
    GRUS_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    // keep `budget` plus a fixed reserve for workspaces free; hold the rest
    const uint64_t reserve = 4ull << 30;
    const uint64_t keep = g->budget_bytes + reserve;
    if (free_b > keep + (64ull << 20)) {
      if (cudaMalloc(&g->balloon, free_b - keep) != cudaSuccess) {
        cudaGetLastError();
        g->balloon = nullptr;
      }
    }
  }
  return GRUS_OK;
}

// Upload host CSR arrays into a new handle (device or managed memory).
int graph_from_host(uint64_t n, uint64_t m, const uint32_t *offs,
                    const uint32_t *cols, const uint32_t *wts, uint32_t flags,
                    int mem_mode, uint64_t budget, grus_graph **out) {
  if (!out || (!offs && n) || (!cols && m)) return GRUS_EINVAL;
  if (n >= 0xFFFFFFFFull || m >= 0xFFFFFFFFull) return GRUS_EOVERFLOW;
  if (mem_mode != GRUS_MEM_DEVICE && mem_mode != GRUS_MEM_MANAGED) return GRUS_EINVAL;
  if (offs[0] != 0 || offs[n] != m) {
    set_last_error("offsets must start at 0 and end at m");
    return GRUS_EINVAL;
  }
  grus_graph *g = new grus_graph();
  g->n = n;
  g->m = m;
  g->flags = flags | (wts ? GRUS_GRAPH_WEIGHTED : 0u);
  g->mem_mode = mem_mode;
  g->budget_bytes = budget;
  cudaGetDevice(&g->device);
  int rc = graph_alloc_array(g, (void **)&g->csr.offs, (n + 1) * 4);
  if (!rc) rc = graph_alloc_array(g, (void **)&g->csr.cols, m * 4);
  if (!rc && wts) rc = graph_alloc_array(g, (void **)&g->csr.wts, m * 4);
  if (rc) {
    grus_graph_free(g);
    return rc;
  }
  cudaError_t e = cudaMemcpy(g->csr.offs, offs, (n + 1) * 4, cudaMemcpyDefault);
  if (e == cudaSuccess && m) e = cudaMemcpy(g->csr.cols, cols, m * 4, cudaMemcpyDefault);
  if (e == cudaSuccess && wts && m) e = cudaMemcpy(g->csr.wts, wts, m * 4, cudaMemcpyDefault);
  uint32_t *bad = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&bad, 4);
  if (e == cudaSuccess) e = cudaMemset(bad, 0, 4);
  uint32_t hbad = 0;
  if (e == cudaSuccess) {
    if (m) k_check_cols<<<grid_for(m), 256>>>(g->csr.cols, m, n, bad);
    e = cudaMemcpy(&hbad, bad, 4, cudaMemcpyDeviceToHost);
  }
  if (bad) cudaFree(bad);
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    grus_graph_free(g);
    return status_from_cuda(e);
  }
  if (hbad) {
    set_last_error("a column index is >= n");
    grus_graph_free(g);
    return GRUS_EINVAL;
  }
  rc = finalize_graph(g);
  if (!rc) rc = apply_mem_policy(g, 0);
  if (rc) {
    grus_graph_free(g);
    return rc;
  }
  *out = g;
  return GRUS_OK;
}

// rep[v].x: among the first kRepScan in-neighbours of v, one of largest
// out-degree (the first such), or kNoRep; rep[v].y: v's out-degree, so one
// 8-byte load gives a pull level both the test and the frontier's edge
// count (a random vertex's entry is one sector, where the representative
// and the offsets were two).  One warp per vertex; the key
// (out-degree, -position) is reduced across the lanes.  A BFS pull level tests
// this vertex's frontier bit before reading v's adjacency: high-degree
// neighbours are reached early, so for nearly every vertex found at a pull
// level (99.4-100 % on RMAT-20) the representative is already in the
// frontier and the scattered read of the list is skipped.  Any in-neighbour
// would keep results exact; the bound keeps the build at one pass.
constexpr uint32_t kRepScan = 256;
__global__ void k_build_rep(const uint32_t *__restrict__ ioffs, const uint32_t *__restrict__ icols,
                            const uint32_t *__restrict__ offs, uint32_t n, uint2 *rep) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += nw) {
    const uint32_t b = ioffs[v], e = min(ioffs[v + 1], b + kRepScan);
    unsigned long long best = 0;
    for (uint32_t x = b + lane; x < e; x += 32) {
      const uint32_t u = icols[x];
      const unsigned long long key =
          ((unsigned long long)(offs[u + 1] - offs[u] + 1u) << 32) | (0xFFFFFFFFu - (x - b));
      best = key > best ? key : best;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_xor_sync(0xffffffffu, best, o);
      best = t > best ? t : best;
    }
    if (lane == 0)
      rep[v] = make_uint2(best ? icols[b + (0xFFFFFFFFu - (uint32_t)best)] : kNoRep,
                          offs[v + 1] - offs[v]);
  }
}

int build_rep_locked(grus_graph *g) {
  if (g->bfs_rep) return GRUS_OK;
  const bool sym = (g->flags & GRUS_GRAPH_SYMMETRIC) != 0;
  const uint32_t *io = sym ? g->csr.offs : g->csc.offs;
  const uint32_t *ic = sym ? g->csr.cols : g->csc.cols;
  if (!io) return GRUS_EINVAL;
  uint2 *rep = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&rep, std::max<uint64_t>(g->n, 1) * sizeof(uint2));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float ms = 0.f;
  if (e == cudaSuccess) {
    cudaEventRecord(e0, 0);
    const int sms = std::max(device_sm_count(), 1);
    if (g->n) k_build_rep<<<sms * 8, 256>>>(io, ic, g->csr.offs, (uint32_t)g->n, rep);
    cudaEventRecord(e1, 0);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) {
    if (rep) cudaFree(rep);
    set_last_error(std::string("bfs pull index: ") + cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  g->bfs_rep = rep;
  g->bfs_rep_ms = ms;
  return GRUS_OK;
}

// Device transpose: stable radix sort of column ids carrying edge ids, so each
// CSC column lists its rows in ascending order exactly as the counting sort of
// include/graph.cuh:273-303 does; weights are permuted along (the reference
// drops them, :294).
int build_csc_locked(grus_graph *g) {
  if (g->csc.offs) return GRUS_OK;
  if (g->flags & GRUS_GRAPH_SYMMETRIC) {
    g->csc = g->csr;  // symmetric: in-edges == out-edges (aliased, not owned)
    return GRUS_OK;
  }
  const uint64_t n = g->n, m = g->m;
  uint32_t *keys_in = nullptr, *keys_out = nullptr, *vals_in = nullptr,
           *vals_out = nullptr, *rowid = nullptr;
  void *tmp = nullptr;
  size_t tmp_bytes = 0;
  Csr t;
  int rc = GRUS_OK;
  int bits = 1;
  while (bits < 32 && (1ull << bits) < n) ++bits;
  cudaError_t e = cudaSuccess;
#define GRUS_TRY_E(x) do { e = (x); if (e != cudaSuccess) goto fail; } while (0)
  GRUS_TRY_E(cudaMalloc(&keys_out, std::max<uint64_t>(m, 1) * 4));
  GRUS_TRY_E(cudaMalloc(&vals_in, std::max<uint64_t>(m, 1) * 4));
  GRUS_TRY_E(cudaMalloc(&vals_out, std::max<uint64_t>(m, 1) * 4));
  GRUS_TRY_E(cudaMalloc(&rowid, std::max<uint64_t>(m, 1) * 4));
  GRUS_TRY_E(cudaMalloc(&keys_in, std::max<uint64_t>(m, 1) * 4));
  rc = graph_alloc_array(g, (void **)&t.offs, (n + 1) * 4);
  if (!rc) rc = graph_alloc_array(g, (void **)&t.cols, m * 4);
  if (!rc && g->csr.wts) rc = graph_alloc_array(g, (void **)&t.wts, m * 4);
  if (rc) goto fail_rc;
  if (m) {
    GRUS_TRY_E(cudaMemcpy(keys_in, g->csr.cols, m * 4, cudaMemcpyDeviceToDevice));
    k_iota<<<grid_for(m), 256>>>(vals_in, m);
    k_expand_rows<<<grid_for(n * 32), 256>>>(g->csr.offs, n, rowid);
    GRUS_TRY_E(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys_in, keys_out,
                                               vals_in, vals_out, (int64_t)m, 0, bits));
    GRUS_TRY_E(cudaMalloc(&tmp, tmp_bytes));
    GRUS_TRY_E(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys_in, keys_out,
                                               vals_in, vals_out, (int64_t)m, 0, bits));
    k_gather_csc<<<grid_for(m), 256>>>(vals_out, rowid, g->csr.wts, m, t.cols, t.wts);
  }
  k_offsets_from_sorted<<<grid_for(m + 1), 256>>>(keys_out, m, n, t.offs);
  GRUS_TRY_E(cudaGetLastError());
  GRUS_TRY_E(cudaDeviceSynchronize());
  cudaFree(tmp);
  cudaFree(keys_in);
  cudaFree(keys_out);
  cudaFree(vals_in);
  cudaFree(vals_out);
  cudaFree(rowid);
  g->csc = t;
  return GRUS_OK;
fail:
  set_last_error(std::string("csc build: ") + cudaGetErrorString(e));
  rc = status_from_cuda(e);
fail_rc:
  cudaFree(tmp);
  cudaFree(keys_in);
  cudaFree(keys_out);
  cudaFree(vals_in);
  cudaFree(vals_out);
  cudaFree(rowid);
  if (t.offs) cudaFree(t.offs);
  if (t.cols) cudaFree(t.cols);
  if (t.wts) cudaFree(t.wts);
  return rc;
#undef GRUS_TRY_E
}

// L2 persistence: reserve the set-aside once per process and return the
// window size usable for `bytes` starting at `base` (0 = unsupported).
int l2_window(cudaStream_t, void *, size_t bytes) {
  static int max_window = -1;
  static size_t set_aside = 0;
  if (max_window < 0) {
    int dev = 0, w = 0, p = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&w, cudaDevAttrMaxAccessPolicyWindowSize, dev);
    cudaDeviceGetAttribute(&p, cudaDevAttrMaxPersistingL2CacheSize, dev);
    max_window = w;
    set_aside = (size_t)p;
    if (p > 0 && cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, set_aside) != cudaSuccess) {
      cudaGetLastError();
      set_aside = 0;
    }
  }
  if (!set_aside || max_window <= 0) return 0;
  return (int)std::min<size_t>(bytes, (size_t)max_window);
}

float l2_hit_ratio(size_t bytes) {
  static int p = -1;
  if (p < 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxPersistingL2CacheSize, dev) != cudaSuccess) {
      cudaGetLastError();
      v = 0;
    }
    p = v;
  }
  if (p <= 0 || bytes <= (size_t)p) return 1.0f;
  return (float)((double)p / (double)bytes);
}

}  // namespace grus

using namespace grus;

extern "C" {

const char *grus_version(void) { return "grus-gb300 0.1 (sm_103a)"; }

const char *grus_strerror(int s) {
  switch (s) {
    case GRUS_OK: return "ok";
    case GRUS_ENOENT: return "no such file";
    case GRUS_EIO: return "i/o error or truncated file";
    case GRUS_ENOMEM: return "out of memory";
    case GRUS_EBUSY: return "resource busy";
    case GRUS_ENODEV: return "no CUDA device";
    case GRUS_EINVAL: return "invalid argument";
    case GRUS_EOVERFLOW: return "value or capacity overflow";
    case GRUS_ETIMEDOUT: return "device wait timed out";
    case GRUS_ECUDA: return "CUDA error";
    default: return "unknown status";
  }
}

const char *grus_last_error(void) { return g_last_error.c_str(); }

int grus_device_init(int device) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    set_last_error("no CUDA device visible");
    return GRUS_ENODEV;
  }
  if (device < 0 || device >= count) return GRUS_EINVAL;
  GRUS_CUDA_TRY(cudaSetDevice(device));
  GRUS_CUDA_TRY(cudaFree(nullptr));
  return GRUS_OK;
}

int grus_check_wait_limit(uint32_t timeout_ms) {
  if (timeout_ms < 1 || timeout_ms > 10000) return GRUS_EINVAL;
  constexpr size_t kErrOff = sizeof(GridBarrier), kBytes = kErrOff + 64;
  char *ctrl = nullptr;
  GRUS_CUDA_TRY(cudaMalloc(&ctrl, kBytes));
  // barrier at offset 0, error word after it; one arrival already counted, so
  // the single CTA of the launch never sees the episode complete
  GridBarrier preset{};
  preset.count = 1u;
  cudaError_t e = cudaMemset(ctrl, 0, kBytes);
  if (e == cudaSuccess) e = cudaMemcpy(ctrl, &preset, sizeof(preset), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_wait_limit<<<1, 32>>>((GridBarrier *)ctrl, (uint32_t *)(ctrl + kErrOff),
                            (uint64_t)timeout_ms * 1000000ull);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  uint32_t err = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&err, ctrl + kErrOff, 4, cudaMemcpyDeviceToHost);
  cudaFree(ctrl);
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return status_from_cuda(e);
  }
  if (err & kErrTimeout) {
    set_last_error("device wait ended at its time limit (as intended by this check)");
    return GRUS_ETIMEDOUT;
  }
  set_last_error("device wait did not report its time limit");
  return GRUS_ECUDA;
}

int grus_check_stale_barrier(grus_graph *g, uint32_t which, uint32_t timeout_ms, void *stream) {
  if (!g || timeout_ms < 1 || timeout_ms > 10000) return GRUS_EINVAL;
  CtrlView v;
  switch (which) {
    case GRUS_CHECK_BFS: v = bfs_ctrl(g); break;
    case GRUS_CHECK_SSSP: v = sssp_ctrl(g); break;
    case GRUS_CHECK_BFS_MULTI: v = msbfs_ctrl(g); break;
    case GRUS_CHECK_SSSP_MULTI: v = msssp_ctrl(g); break;
    case GRUS_CHECK_PAGERANK: v = pr_ctrl(g); break;
    default: return GRUS_EINVAL;
  }
  if (!v.ctrl) {
    set_last_error("the graph has no workspace for this algorithm yet (run it once first)");
    return GRUS_EINVAL;
  }
  GRUS_CUDA_TRY(cudaSetDevice(g->device));
  k_stale_barrier<<<1, 32, 0, (cudaStream_t)stream>>>((GridBarrier *)(v.ctrl + v.bar_off),
                                                       (uint32_t *)(v.ctrl + v.err_off),
                                                       (uint64_t)timeout_ms * 1000000ull);
  GRUS_CUDA_TRY(cudaGetLastError());
  return GRUS_OK;
}

int grus_graph_from_csr(uint64_t n, uint64_t m, const uint32_t *offsets,
                        const uint32_t *cols, const uint32_t *weights,
                        uint32_t flags, int mem_mode, uint64_t budget_bytes,
                        grus_graph **out) {
  // host-side validation of the offsets' monotonicity (cheap, O(n))
  if (!offsets || (m && !cols) || !out) return GRUS_EINVAL;
  if (!is_device_pointer(offsets)) {
    for (uint64_t i = 0; i < n; ++i)
      if (offsets[i + 1] < offsets[i]) {
        set_last_error("offsets are not monotone");
        return GRUS_EINVAL;
      }
  }
  return graph_from_host(n, m, offsets, cols, weights, flags, mem_mode,
                         budget_bytes, out);
}

// .gr loader: the layout of include/graph_loader.cuh:65-159 read with large
// freads into pinned staging, offsets converted u64->u32 on the device.
// Every malformed input is reported (the reference prints and continues,
// :72-76,110-111,125-126,146-147; assumes sizeEdgeTy==4, :143).
int grus_graph_load_gr(const char *path, int need_weights, int mem_mode,
                       uint64_t budget_bytes, grus_graph **out) {
  if (!path || !out) return GRUS_EINVAL;
  FILE *f = std::fopen(path, "rb");
  if (!f) {
    set_last_error(std::string("cannot open ") + path);
    return GRUS_ENOENT;
  }
  uint64_t h[4];
  if (std::fread(h, 8, 4, f) != 4) {
    std::fclose(f);
    set_last_error("unable to read .gr header");
    return GRUS_EIO;
  }
  if (h[0] != 1 || (h[1] != 0 && h[1] != 4)) {
    std::fclose(f);
    set_last_error("unsupported .gr version or edge size");
    return GRUS_EINVAL;
  }
  const uint64_t n = h[2], m = h[3];
  if (n >= 0xFFFFFFFFull || m >= 0xFFFFFFFFull) {
    std::fclose(f);
    set_last_error(".gr graph too large for uint32 ids/offsets");
    return GRUS_EOVERFLOW;
  }
  grus_graph *g = new grus_graph();
  g->n = n;
  g->m = m;
  g->mem_mode = mem_mode;
  g->budget_bytes = budget_bytes;
  cudaGetDevice(&g->device);
  const bool weighted = h[1] != 0;
  const bool want_w = need_weights != 0;
  if (want_w) g->flags |= GRUS_GRAPH_WEIGHTED;
  int rc = graph_alloc_array(g, (void **)&g->csr.offs, (n + 1) * 4);
  if (!rc) rc = graph_alloc_array(g, (void **)&g->csr.cols, m * 4);
  if (!rc && want_w) rc = graph_alloc_array(g, (void **)&g->csr.wts, m * 4);
  uint64_t *d_ends = nullptr;
  uint32_t *d_bad = nullptr;
  void *stage = nullptr;
  const size_t kStage = 64ull << 20;
  uint32_t hbad = 0;
  cudaError_t e = cudaSuccess;
  auto read_to = [&](void *dst, uint64_t bytes) -> int {
    uint64_t done = 0;
    while (done < bytes) {
      const size_t chunk = (size_t)std::min<uint64_t>(kStage, bytes - done);
      if (std::fread(stage, 1, chunk, f) != chunk) return GRUS_EIO;
      e = cudaMemcpy((char *)dst + done, stage, chunk, cudaMemcpyDefault);
      if (e != cudaSuccess) return status_from_cuda(e);
      done += chunk;
    }
    return GRUS_OK;
  };
  if (!rc && cudaMallocHost(&stage, kStage) != cudaSuccess) rc = GRUS_ENOMEM;
  if (!rc && cudaMalloc(&d_ends, std::max<uint64_t>(n, 1) * 8) != cudaSuccess) rc = GRUS_ENOMEM;
  if (!rc && cudaMalloc(&d_bad, 4) != cudaSuccess) rc = GRUS_ENOMEM;
  if (!rc) cudaMemset(d_bad, 0, 4);
  if (!rc) rc = read_to(d_ends, n * 8);
  if (!rc && n) {
    k_u64_to_u32_offsets<<<grid_for(n), 256>>>(d_ends, n, g->csr.offs, d_bad, m);
  } else if (!rc) {
    cudaMemset(g->csr.offs, 0, 4);
  }
  if (!rc) rc = read_to(g->csr.cols, m * 4);
  if (!rc && m) k_check_cols<<<grid_for(m), 256>>>(g->csr.cols, m, n, d_bad);
  if (!rc && want_w) {
    if (weighted) {
      if (m % 2) {
        uint32_t pad;
        if (std::fread(&pad, 4, 1, f) != 1) rc = GRUS_EIO;
      }
      if (!rc) rc = read_to(g->csr.wts, m * 4);
    } else if (m) {
      k_fill_u32<<<grid_for(m), 256>>>(g->csr.wts, m, 1u);  // :95-101
    }
  }
  if (!rc) {
    e = cudaMemcpy(&hbad, d_bad, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = status_from_cuda(e);
  }
  if (!rc) {
    uint32_t last = 0;
    e = cudaMemcpy(&last, g->csr.offs + n, 4, cudaMemcpyDefault);
    if (e != cudaSuccess) rc = status_from_cuda(e);
    else if (last != m) hbad |= 4u;
  }
  std::fclose(f);
  if (stage) cudaFreeHost(stage);
  if (d_ends) cudaFree(d_ends);
  if (d_bad) cudaFree(d_bad);
  if (!rc && hbad) {
    set_last_error(".gr offsets or destinations out of range");
    rc = GRUS_EINVAL;
  }
  if (rc == GRUS_EIO) set_last_error("truncated .gr file");
  if (!rc) rc = finalize_graph(g);
  if (!rc) rc = apply_mem_policy(g, 0);
  if (rc) {
    grus_graph_free(g);
    return rc;
  }
  *out = g;
  return GRUS_OK;
}

int grus_graph_save_gr(const grus_graph *g, const char *path) {
  if (!g || !path) return GRUS_EINVAL;
  std::vector<uint32_t> offs(g->n + 1), cols(g->m), wts(g->csr.wts ? g->m : 0);
  int rc = grus_graph_copy_csr(g, offs.data(), cols.data(),
                               g->csr.wts ? wts.data() : nullptr);
  if (rc) return rc;
  FILE *f = std::fopen(path, "wb");
  if (!f) return GRUS_EIO;
  const uint64_t h[4] = {1, g->csr.wts ? 4ull : 0ull, g->n, g->m};
  bool ok = std::fwrite(h, 8, 4, f) == 4;
  std::vector<uint64_t> ends(g->n);
  for (uint64_t i = 0; i < g->n; ++i) ends[i] = offs[i + 1];
  if (ok && g->n) ok = std::fwrite(ends.data(), 8, g->n, f) == g->n;
  if (ok && g->m) ok = std::fwrite(cols.data(), 4, g->m, f) == g->m;
  if (ok && g->csr.wts) {
    if (g->m % 2) {
      const uint32_t pad = 0;
      ok = std::fwrite(&pad, 4, 1, f) == 1;
    }
    if (ok && g->m) ok = std::fwrite(wts.data(), 4, g->m, f) == g->m;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GRUS_OK : GRUS_EIO;
}

int grus_graph_get_info(const grus_graph *g, grus_graph_info *info) {
  if (!g || !info) return GRUS_EINVAL;
  std::memset(info, 0, sizeof(*info));
  info->n = g->n;
  info->m = g->m;
  info->max_degree_vertex = g->max_deg_vertex;
  info->max_degree = g->max_deg;
  info->flags = g->flags;
  info->mem_mode = g->mem_mode;
  info->offsets = g->csr.offs;
  info->cols = g->csr.cols;
  info->weights = g->csr.wts;
  info->t_offsets = g->csc.offs;
  info->t_cols = g->csc.cols;
  info->t_weights = g->csc.wts;
  info->budget_bytes = g->budget_bytes;
  return GRUS_OK;
}

int grus_graph_copy_csr(const grus_graph *g, uint32_t *offsets, uint32_t *cols,
                        uint32_t *weights) {
  if (!g) return GRUS_EINVAL;
  if (offsets) GRUS_CUDA_TRY(cudaMemcpy(offsets, g->csr.offs, (g->n + 1) * 4, cudaMemcpyDefault));
  if (cols && g->m) GRUS_CUDA_TRY(cudaMemcpy(cols, g->csr.cols, g->m * 4, cudaMemcpyDefault));
  if (weights) {
    if (!g->csr.wts) return GRUS_EINVAL;
    if (g->m) GRUS_CUDA_TRY(cudaMemcpy(weights, g->csr.wts, g->m * 4, cudaMemcpyDefault));
  }
  return GRUS_OK;
}

int grus_graph_build_csc(grus_graph *g) {
  if (!g) return GRUS_EINVAL;
  std::lock_guard<std::mutex> lk(g->mu);
  return build_csc_locked(g);
}

int grus_graph_build_index(grus_graph *g, float *build_ms) {
  if (!g) return GRUS_EINVAL;
  std::lock_guard<std::mutex> lk(g->mu);
  if (!(g->flags & GRUS_GRAPH_SYMMETRIC)) {
    const int rc = build_csc_locked(g);
    if (rc) return rc;
  }
  const int rc = build_rep_locked(g);
  if (rc) return rc;
  if (build_ms) *build_ms = g->bfs_rep_ms;
  return GRUS_OK;
}

int grus_graph_set_tuning(grus_graph *g, const grus_tuning *t) {
  if (!g || !t) return GRUS_EINVAL;
  if (t->alpha < 0.f || t->beta < 0.f || t->multi_alpha < 0.f || t->ctas_per_sm > 64 ||
      t->depth_planes > 2 || t->tail_cluster > 2)
    return GRUS_EINVAL;
  std::lock_guard<std::mutex> lk(g->mu);
  if (t->huge_degree != g->tuning.huge_degree) {
    // hub chunk lists are sized from the chunking degree: rebuild workspaces
    cudaDeviceSynchronize();
    for (int i = 0; i < kWsCount; ++i)
      if (g->ws[i] && g->ws_free[i]) {
        g->ws_free[i](g->ws[i]);
        g->ws[i] = nullptr;
      }
  }
  g->tuning = *t;
  return GRUS_OK;
}

int grus_graph_get_tuning(const grus_graph *g, grus_tuning *t) {
  if (!g || !t) return GRUS_EINVAL;
  *t = g->tuning;
  return GRUS_OK;
}

int grus_graph_free(grus_graph *g) {
  if (!g) return GRUS_EINVAL;
  cudaDeviceSynchronize();
  for (int i = 0; i < kWsCount; ++i)
    if (g->ws[i] && g->ws_free[i]) g->ws_free[i](g->ws[i]);
  if (g->csc.offs && g->csc.offs != g->csr.offs) {
    cudaFree(g->csc.offs);
    cudaFree(g->csc.cols);
    if (g->csc.wts) cudaFree(g->csc.wts);
  }
  if (g->csr.offs) cudaFree(g->csr.offs);
  if (g->csr.cols) cudaFree(g->csr.cols);
  if (g->csr.wts) cudaFree(g->csr.wts);
  if (g->bfs_rep) cudaFree(g->bfs_rep);
  if (g->balloon) cudaFree(g->balloon);
  delete g;
  return GRUS_OK;
}

int grus_graph_copy_csc(const grus_graph *g, uint32_t *t_offsets,
                        uint32_t *t_cols, uint32_t *t_weights) {
  if (!g || !g->csc.offs) return GRUS_EINVAL;
  if (t_offsets) GRUS_CUDA_TRY(cudaMemcpy(t_offsets, g->csc.offs, (g->n + 1) * 4, cudaMemcpyDefault));
  if (t_cols && g->m) GRUS_CUDA_TRY(cudaMemcpy(t_cols, g->csc.cols, g->m * 4, cudaMemcpyDefault));
  if (t_weights) {
    if (!g->csc.wts) return GRUS_EINVAL;
    if (g->m) GRUS_CUDA_TRY(cudaMemcpy(t_weights, g->csc.wts, g->m * 4, cudaMemcpyDefault));
  }
  return GRUS_OK;
}

}  // extern "C"

namespace grus {

// Cooperative launch of a persistent kernel: SMs x min(occupancy, requested)
// CTAs, with an L2 persisting access-policy window over [win_base, +win_bytes)
// attached to this launch only (the caller's stream is left untouched).
int launch_persistent(const void *fn, void **args, int block, int per_sm_req,
                      int occupancy, cudaStream_t s, void *win_base, size_t win_bytes) {
  int per_sm = occupancy;
  if (per_sm_req > 0) per_sm = std::min(per_sm, per_sm_req);
  if (per_sm < 1) {
    set_last_error("persistent kernel cannot be resident");
    return GRUS_ECUDA;
  }
  cudaLaunchAttribute attrs[2];
  int nattr = 0;
  attrs[nattr].id = cudaLaunchAttributeCooperative;
  attrs[nattr].val.cooperative = 1;
  ++nattr;
  const int win = win_base ? l2_window(s, win_base, win_bytes) : 0;
  if (win > 0) {
    attrs[nattr].id = cudaLaunchAttributeAccessPolicyWindow;
    attrs[nattr].val.accessPolicyWindow.base_ptr = win_base;
    attrs[nattr].val.accessPolicyWindow.num_bytes = (size_t)win;
    attrs[nattr].val.accessPolicyWindow.hitRatio = l2_hit_ratio((size_t)win);
    attrs[nattr].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attrs[nattr].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    ++nattr;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(device_sm_count() * per_sm));
  cfg.blockDim = dim3((unsigned)block);
  cfg.stream = s;
  cfg.attrs = attrs;
  cfg.numAttrs = nattr;
  GRUS_CUDA_TRY(cudaLaunchKernelExC(&cfg, fn, args));
  return GRUS_OK;
}

}  // namespace grus
