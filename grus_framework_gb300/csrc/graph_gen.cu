// graph_gen.cu -- seeded RMAT and 2-D grid graphs built directly in HBM.
//
// The reference ships no generator (it reads Galois-converted .gr files,
// README.md:14-27); the configurations it is measured on are synthetic RMAT
// and grid graphs, so the library generates them on the device:
//   1. one thread per raw edge draws its RMAT endpoints from a counter-based
//      hash (no RNG state, so any edge can be regenerated independently),
//   2. CUB radix-sorts the packed (u << scale | v) keys, de-duplicates,
//   3. rows become offsets by a boundary scan, weights are a hash of the
//      undirected edge.
// Specification (shared with the CPU oracle, which restates it):
//   mix64   = SplitMix64 output function (Steele, Lea & Flood 2014).
//   edge i  : base = mix64(mix64(seed) ^ i); level l uses 16-bit lane l%4 of
//             mix64(base + l/4); quadrant thresholds 37356 / 49807 / 62259
//             of 65536 (a=.57, b=.19, c=.19, d=.05).
//   relabel : 3 rounds of x = (x*odd + c) mod 2^s; x ^= x >> ceil(s/2).
//   weight  : mix64(mix64(seed ^ 0x2545F4914F6CDD1D) ^ (min<<32|max)) % 255 + 1.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

#include <algorithm>

#include "grus_internal.cuh"

namespace grus {

int finalize_graph(grus_graph *g);
int apply_mem_policy(grus_graph *g, cudaStream_t s);

namespace {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ void rmat_edge(int scale, uint64_t seed, uint64_t i,
                                          uint32_t &u, uint32_t &v) {
  const uint64_t base = mix64(mix64(seed) ^ i);
  uint64_t r = 0;
  uint32_t a = 0, b = 0;
  for (int l = 0; l < scale; ++l) {
    if ((l & 3) == 0) r = mix64(base + (uint64_t)(l >> 2));
    const uint32_t x = (uint32_t)((r >> ((l & 3) * 16)) & 0xFFFFu);
    const uint32_t ub = x >= 49807u;                  // quadrants c, d
    const uint32_t vb = (x >= 37356u && x < 49807u) || x >= 62259u;  // b, d
    a = (a << 1) | ub;
    b = (b << 1) | vb;
  }
  u = a;
  v = b;
}

__device__ __forceinline__ uint32_t relabel(int scale, uint64_t k0, uint32_t x) {
  const uint64_t mask = (1ull << scale) - 1;
  const int sh = (scale + 1) / 2;
  uint64_t y = x;
#pragma unroll
  for (int round = 0; round < 3; ++round) {
    const uint64_t kr = mix64(k0 + (uint64_t)round);
    y = (y * ((kr & mask) | 1ull) + ((kr >> 32) & mask)) & mask;
    y ^= (y >> sh);
  }
  return (uint32_t)y;
}

__device__ __forceinline__ uint32_t edge_weight(uint64_t wseed, uint32_t u, uint32_t v) {
  const uint64_t lo = u < v ? u : v, hi = u < v ? v : u;
  return (uint32_t)(mix64(wseed ^ ((lo << 32) | hi)) % 255ull) + 1u;
}

// Self-loops map to the all-ones key (the pair (n-1, n-1), itself a loop),
// which sorts last and is dropped.
__global__ void k_rmat_keys(int scale, uint64_t seed, uint64_t E, bool sym,
                            bool rel, uint64_t *__restrict__ keys) {
  const uint64_t k0 = mix64(seed ^ 0x5851F42D4C957F2Dull);
  const uint64_t sentinel = (1ull << (2 * scale)) - 1;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t u, v;
    rmat_edge(scale, seed, i, u, v);
    if (rel) {
      u = relabel(scale, k0, u);
      v = relabel(scale, k0, v);
    }
    const bool loop = u == v;
    if (sym) {
      keys[2 * i] = loop ? sentinel : (((uint64_t)u << scale) | v);
      keys[2 * i + 1] = loop ? sentinel : (((uint64_t)v << scale) | u);
    } else {
      keys[i] = loop ? sentinel : (((uint64_t)u << scale) | v);
    }
  }
}

__global__ void k_keys_to_csr(const uint64_t *__restrict__ keys, uint64_t m,
                              int scale, uint64_t n, uint32_t *__restrict__ offs,
                              uint32_t *__restrict__ cols, uint32_t *__restrict__ wts,
                              uint64_t wseed) {
  const uint64_t vmask = (1ull << scale) - 1;
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e <= m;
       e += (uint64_t)gridDim.x * blockDim.x) {
    const int64_t prev = e == 0 ? -1 : (int64_t)(keys[e - 1] >> scale);
    const int64_t cur = e == m ? (int64_t)n : (int64_t)(keys[e] >> scale);
    for (int64_t x = prev + 1; x <= cur; ++x) offs[x] = (uint32_t)e;
    if (e < m) {
      const uint32_t v = (uint32_t)(keys[e] & vmask);
      cols[e] = v;
      if (wts) wts[e] = edge_weight(wseed, (uint32_t)cur, v);
    }
  }
}

__global__ void k_grid_degree(uint32_t rows, uint32_t ncols, uint32_t *__restrict__ deg) {
  const uint64_t n = (uint64_t)rows * ncols;
  for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < n;
       u += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = (uint32_t)(u / ncols), c = (uint32_t)(u % ncols);
    deg[u] = (r > 0) + (c > 0) + (c + 1 < ncols) + (r + 1 < rows);
  }
}

__global__ void k_grid_fill(uint32_t rows, uint32_t ncols, const uint32_t *__restrict__ offs,
                            uint32_t *__restrict__ cols, uint32_t *__restrict__ wts,
                            uint64_t wseed) {
  const uint64_t n = (uint64_t)rows * ncols;
  for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < n;
       u += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = (uint32_t)(u / ncols), c = (uint32_t)(u % ncols);
    uint32_t e = offs[u];
    uint32_t nb[4];
    int k = 0;
    if (r > 0) nb[k++] = (uint32_t)(u - ncols);
    if (c > 0) nb[k++] = (uint32_t)(u - 1);
    if (c + 1 < ncols) nb[k++] = (uint32_t)(u + 1);
    if (r + 1 < rows) nb[k++] = (uint32_t)(u + ncols);
    for (int j = 0; j < k; ++j, ++e) {
      cols[e] = nb[j];
      if (wts) wts[e] = edge_weight(wseed, (uint32_t)u, nb[j]);
    }
  }
}

int grid_for(uint64_t work, int block = 256) {
  const int sms = std::max(device_sm_count(), 1);
  const uint64_t want = (work + block - 1) / block;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)sms * 16));
}

}  // namespace
}  // namespace grus

using namespace grus;

extern "C" {

int grus_graph_rmat(int scale, int edge_factor, uint64_t seed,
                    uint32_t gen_flags, int mem_mode, uint64_t budget_bytes,
                    grus_graph **out) {
  if (!out || scale < 1 || scale > 30 || edge_factor < 1) return GRUS_EINVAL;
  if (mem_mode != GRUS_MEM_DEVICE && mem_mode != GRUS_MEM_MANAGED) return GRUS_EINVAL;
  const bool sym = gen_flags & GRUS_GEN_SYMMETRIC;
  const uint64_t n = 1ull << scale;
  const uint64_t E = (uint64_t)edge_factor << scale;
  const uint64_t K = sym ? 2 * E : E;
  uint64_t *keys = nullptr, *keys_alt = nullptr;
  void *tmp = nullptr;
  size_t tmp_sort = 0, tmp_uniq = 0;
  int64_t *d_num = nullptr;
  int64_t num = 0;
  grus_graph *g = nullptr;
  int rc = GRUS_OK;
  cudaError_t e = cudaSuccess;
#define GRUS_GEN_TRY(x) do { e = (x); if (e != cudaSuccess) goto fail; } while (0)
  GRUS_GEN_TRY(cudaMalloc(&keys, K * 8));
  GRUS_GEN_TRY(cudaMalloc(&keys_alt, K * 8));
  GRUS_GEN_TRY(cudaMalloc(&d_num, sizeof(int64_t)));
  k_rmat_keys<<<grid_for(E), 256>>>(scale, seed, E, sym, gen_flags & GRUS_GEN_RELABEL, keys);
  GRUS_GEN_TRY(cudaGetLastError());
  GRUS_GEN_TRY(cub::DeviceRadixSort::SortKeys(nullptr, tmp_sort, keys, keys_alt, (int64_t)K, 0, 2 * scale));
  GRUS_GEN_TRY(cub::DeviceSelect::Unique(nullptr, tmp_uniq, keys_alt, keys, d_num, (int64_t)K));
  GRUS_GEN_TRY(cudaMalloc(&tmp, std::max(tmp_sort, tmp_uniq)));
  GRUS_GEN_TRY(cub::DeviceRadixSort::SortKeys(tmp, tmp_sort, keys, keys_alt, (int64_t)K, 0, 2 * scale));
  GRUS_GEN_TRY(cub::DeviceSelect::Unique(tmp, tmp_uniq, keys_alt, keys, d_num, (int64_t)K));
  GRUS_GEN_TRY(cudaMemcpy(&num, d_num, sizeof(num), cudaMemcpyDeviceToHost));
  if (num > 0) {
    uint64_t last = 0;
    GRUS_GEN_TRY(cudaMemcpy(&last, keys + (num - 1), 8, cudaMemcpyDeviceToHost));
    if (last == (1ull << (2 * scale)) - 1) --num;  // drop the self-loop sentinel
  }
  cudaFree(tmp);
  tmp = nullptr;
  cudaFree(keys_alt);
  keys_alt = nullptr;
  if ((uint64_t)num >= 0xFFFFFFFFull) {
    rc = GRUS_EOVERFLOW;
    goto fail_rc;
  }
  g = new grus_graph();
  g->n = n;
  g->m = (uint64_t)num;
  g->mem_mode = mem_mode;
  g->budget_bytes = budget_bytes;
  g->flags = (sym ? GRUS_GRAPH_SYMMETRIC : 0u) |
             ((gen_flags & GRUS_GEN_WEIGHTED) ? GRUS_GRAPH_WEIGHTED : 0u);
  cudaGetDevice(&g->device);
  rc = graph_alloc_array(g, (void **)&g->csr.offs, (n + 1) * 4);
  if (!rc) rc = graph_alloc_array(g, (void **)&g->csr.cols, g->m * 4);
  if (!rc && (gen_flags & GRUS_GEN_WEIGHTED)) rc = graph_alloc_array(g, (void **)&g->csr.wts, g->m * 4);
  if (rc) goto fail_rc;
  k_keys_to_csr<<<grid_for(g->m + 1), 256>>>(keys, g->m, scale, n, g->csr.offs, g->csr.cols,
                                             g->csr.wts, mix64(seed ^ 0x2545F4914F6CDD1Dull));
  GRUS_GEN_TRY(cudaGetLastError());
  GRUS_GEN_TRY(cudaDeviceSynchronize());
  cudaFree(keys);
  keys = nullptr;
  cudaFree(d_num);
  d_num = nullptr;
  rc = finalize_graph(g);
  if (!rc) rc = apply_mem_policy(g, 0);
  if (rc) goto fail_rc;
  *out = g;
  return GRUS_OK;
fail:
  set_last_error(std::string("rmat: ") + cudaGetErrorString(e));
  rc = status_from_cuda(e);
fail_rc:
  cudaFree(tmp);
  cudaFree(keys);
  cudaFree(keys_alt);
  cudaFree(d_num);
  if (g) grus_graph_free(g);
  return rc;
#undef GRUS_GEN_TRY
}

int grus_graph_grid2d(uint32_t rows, uint32_t cols, uint64_t seed,
                      uint32_t gen_flags, grus_graph **out) {
  if (!out || rows == 0 || cols == 0) return GRUS_EINVAL;
  const uint64_t n = (uint64_t)rows * cols;
  if (n >= 0xFFFFFFFFull) return GRUS_EOVERFLOW;
  const uint64_t m = 4ull * n - 2ull * rows - 2ull * cols;
  grus_graph *g = new grus_graph();
  g->n = n;
  g->m = m;
  g->flags = GRUS_GRAPH_SYMMETRIC | ((gen_flags & GRUS_GEN_WEIGHTED) ? GRUS_GRAPH_WEIGHTED : 0u);
  cudaGetDevice(&g->device);
  uint32_t *deg = nullptr;
  void *tmp = nullptr;
  size_t tb = 0;
  cudaError_t e = cudaSuccess;
  int rc = graph_alloc_array(g, (void **)&g->csr.offs, (n + 1) * 4);
  if (!rc) rc = graph_alloc_array(g, (void **)&g->csr.cols, m * 4);
  if (!rc && (gen_flags & GRUS_GEN_WEIGHTED)) rc = graph_alloc_array(g, (void **)&g->csr.wts, m * 4);
  if (rc) {
    grus_graph_free(g);
    return rc;
  }
  e = cudaMalloc(&deg, (n + 1) * 4);
  if (e == cudaSuccess) e = cudaMemset(deg + n, 0, 4);
  if (e == cudaSuccess) {
    k_grid_degree<<<grid_for(n), 256>>>(rows, cols, deg);
    e = cub::DeviceScan::ExclusiveSum(nullptr, tb, deg, g->csr.offs, (int64_t)(n + 1));
  }
  if (e == cudaSuccess) e = cudaMalloc(&tmp, tb);
  if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(tmp, tb, deg, g->csr.offs, (int64_t)(n + 1));
  if (e == cudaSuccess) {
    k_grid_fill<<<grid_for(n), 256>>>(rows, cols, g->csr.offs, g->csr.cols, g->csr.wts,
                                      mix64(seed ^ 0x2545F4914F6CDD1Dull));
    e = cudaDeviceSynchronize();
  }
  cudaFree(tmp);
  cudaFree(deg);
  if (e != cudaSuccess) {
    set_last_error(std::string("grid: ") + cudaGetErrorString(e));
    grus_graph_free(g);
    return status_from_cuda(e);
  }
  rc = finalize_graph(g);
  if (rc) {
    grus_graph_free(g);
    return rc;
  }
  *out = g;
  return GRUS_OK;
}

}  // extern "C"
