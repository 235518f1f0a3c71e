/*
 * grus.h -- C ABI of libgrus, the GB300 (sm_103a) frontier-traversal core.
 *
 * The reference (Grus) exposes no C ABI: its path sits behind C++ templates
 * (include/kernel.cuh, frontier.cuh, graph.cuh, graph_loader.cuh) and the
 * samples' command lines.  Each entry point below names the reference
 * interface whose job it takes over, so a maintainer can bind the path from
 * C, ctypes or any FFI.  The mgg drop-in headers in
 * grus_framework_gb300/mgg/ keep the template API itself.
 *
 * Conventions
 *   - Every call returns an int status: 0 on success, a negative code below
 *     on failure.  The library never calls exit() (unlike H_ERR,
 *     include/common.cuh:57-68).  grus_last_error() gives a detail string.
 *   - The library owns graph handles; the caller owns output buffers.  An
 *     output pointer may be host memory (pinned or pageable) or device
 *     memory; the call detects which and copies as needed.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy stream).
 *     Calls with host outputs or a non-NULL stats pointer return after the
 *     work has finished; calls with device outputs and no stats are
 *     asynchronous on `stream`.
 *   - Vertex ids and CSR arrays are uint32 (vtx_t, include/common.cuh:48);
 *     unreached vertices read GRUS_INFINIT (INFINIT, include/common.cuh:52).
 */
#ifndef GRUS_H
#define GRUS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define GRUS_OK 0
#define GRUS_ENOENT (-2)
#define GRUS_EIO (-5)
#define GRUS_ENOMEM (-12)
#define GRUS_EBUSY (-16)
#define GRUS_ENODEV (-19)
#define GRUS_EINVAL (-22)
#define GRUS_EOVERFLOW (-75)
#define GRUS_ETIMEDOUT (-110)
#define GRUS_ECUDA (-1000)

#define GRUS_INFINIT 4294967294u

/* memory modes (include/graph.cuh:170-251 Set_Mem_Policy) */
#define GRUS_MEM_DEVICE 0  /* CSR in HBM (cudaMalloc) */
#define GRUS_MEM_MANAGED 1 /* CSR in managed memory, prefetched up to a budget */

/* graph flags */
#define GRUS_GRAPH_SYMMETRIC 1u /* every edge (u,v) has (v,u): CSR == CSC */
#define GRUS_GRAPH_WEIGHTED 2u  /* uint32 edge weights present */

/* query kinds (batches, server, autotuner) */
#define GRUS_ALGO_BFS 0u
#define GRUS_ALGO_SSSP 1u

/* generator flags */
#define GRUS_GEN_SYMMETRIC 1u
#define GRUS_GEN_WEIGHTED 2u
#define GRUS_GEN_RELABEL 4u

#if defined(__GNUC__)
#define GRUS_API __attribute__((visibility("default")))
#else
#define GRUS_API
#endif

typedef struct grus_graph grus_graph;

typedef struct grus_graph_info {
  uint64_t n;                   /* numNode (include/graph.cuh:116) */
  uint64_t m;                   /* numEdge (include/graph.cuh:117) */
  uint32_t max_degree_vertex;   /* first vertex of maximum out-degree */
  uint32_t max_degree;
  uint32_t flags;               /* GRUS_GRAPH_* */
  int32_t mem_mode;             /* GRUS_MEM_* */
  const uint32_t *offsets;      /* xadj   (device-accessible, n+1) */
  const uint32_t *cols;         /* adjncy (device-accessible, m)   */
  const uint32_t *weights;      /* adjwgt (device-accessible, m) or NULL */
  const uint32_t *t_offsets;    /* CSC arrays, NULL until built */
  const uint32_t *t_cols;
  const uint32_t *t_weights;
  uint64_t budget_bytes;        /* managed mode device budget, else 0 */
} grus_graph_info;

typedef struct grus_stats {
  uint32_t levels;              /* frontier iterations (job.itr at loop end) */
  uint32_t bottom_up_levels;    /* iterations run in pull direction */
  uint32_t direction_switches;
  uint32_t kernel_launches;     /* device kernels launched by this call */
  uint64_t vertices_reached;
  uint64_t edges_reached;       /* m_r: sum of out-degree of reached vertices */
  uint64_t edges_relaxed;       /* SSSP: edge relaxations performed */
  float device_ms;              /* CUDA-event time of the device work */
  uint32_t reserved0;
} grus_stats;

/* Autotunable launch/heuristic parameters (0 fields mean "default"). */
typedef struct grus_tuning {
  float alpha;            /* push->pull when m_f > m_u / alpha (Beamer) */
  float beta;             /* pull->push when n_f < n / beta */
  uint32_t ctas_per_sm;   /* persistent grid = SMs x ctas_per_sm (<= occupancy) */
  uint32_t huge_degree;   /* degree at/above which a vertex is split into chunks */
  uint32_t bu_scan;       /* neighbours a pull thread checks before deferring */
  uint32_t timeout_ms;    /* bound on every device-side wait */
  uint32_t sssp_delta;    /* SSSP near/far bucket width (distance units) */
  uint32_t bu_words;      /* BFS pull levels: bitmap words per warp step (2 or 4) */
  float multi_alpha;      /* multi-source BFS: push->pull when the union frontier's
                             out-edges exceed m / multi_alpha (0: 10 up to 32
                             sources, 6 above) */
  uint32_t depth_planes;  /* BFS: keep depths as bit planes in L2 and write the
                             depth array once at the end (1), or store each
                             depth as its vertex is found (2); 0: planes from
                             2^22 vertices on */
  uint32_t tail_cluster;  /* BFS: hand a long traversal whose push frontier has
                             become small to the thread-block-cluster tail (0
                             or 1), or run every level in the persistent
                             kernel (2) */
} grus_tuning;

/* ---- library ------------------------------------------------------------- */
GRUS_API const char *grus_version(void);
/* Text of a status code. */
GRUS_API const char *grus_strerror(int status);
/* Detail of the last failing call on this host thread. */
GRUS_API const char *grus_last_error(void);
/* Select and initialise a device (FLAGS_device, include/app.cuh:18). */
GRUS_API int grus_device_init(int device);
/* Diagnostic of the bounded device waits, no counterpart in the reference
 * (whose kernels never wait on one another): runs the grid barrier of the
 * persistent kernels in a one-CTA launch whose barrier can never complete
 * (its arrival count is preset), so the wait must end by its time limit.
 * Returns GRUS_ETIMEDOUT after about timeout_ms (1..10000) with the device
 * context still usable, or another status if the wait did not behave. */
GRUS_API int grus_check_wait_limit(uint32_t timeout_ms);
/* Diagnostic of the barrier reset between launches, no counterpart in the
 * reference: queues on `stream`, without waiting, the same one-CTA wait on
 * the control block of one of the graph's workspaces (`which`, below; the
 * workspace exists once that algorithm has run on the graph), so the block
 * is left as a launch that timed out at a grid barrier leaves it: abort flag
 * raised, arrival count stale, error word set.  Every launch clears its
 * block's barrier and error word in its own stream first, so a call queued
 * behind this one runs normally.  Returns GRUS_OK once queued, GRUS_EINVAL
 * when the workspace does not exist or timeout_ms is outside 1..10000. */
#define GRUS_CHECK_BFS 0u
#define GRUS_CHECK_SSSP 1u
#define GRUS_CHECK_BFS_MULTI 2u
#define GRUS_CHECK_SSSP_MULTI 3u
#define GRUS_CHECK_PAGERANK 4u
GRUS_API int grus_check_stale_barrier(grus_graph *g, uint32_t which, uint32_t timeout_ms,
                                      void *stream);

/* ---- graphs -------------------------------------------------------------- */
/* CSR from host arrays.  Replaces graph_t<CSR> filled by
 * graph_loader::ReadGraphGR (include/graph_loader.cuh:65-159). */
GRUS_API int grus_graph_from_csr(uint64_t n, uint64_t m, const uint32_t *offsets,
                        const uint32_t *cols, const uint32_t *weights,
                        uint32_t flags, int mem_mode, uint64_t budget_bytes,
                        grus_graph **out);
/* Builds the BFS pull index of g ahead of its first BFS (grus_bfs builds it
 * on demand otherwise) and reports the device time it took.  No counterpart
 * in the reference.  Per vertex, one in-neighbour of high out-degree and the
 * vertex's out-degree (8 bytes per vertex, freed with the graph; built from
 * the CSC on a directed graph, which it builds too): a pull level tests that
 * neighbour's frontier bit before reading the vertex's adjacency, which
 * settles nearly every vertex found at the level without the scattered read.
 * Results do not change. */
GRUS_API int grus_graph_build_index(grus_graph *g, float *build_ms);
/* Load a Galois v1 .gr file.  Replaces graph_loader::Load
 * (include/graph_loader.cuh:160-166) + Set_Mem_Policy
 * (include/graph.cuh:170-251).  need_weights mirrors Load's _needweight. */
GRUS_API int grus_graph_load_gr(const char *path, int need_weights, int mem_mode,
                       uint64_t budget_bytes, grus_graph **out);
/* Write the graph as .gr (the layout graph_loader.cuh:65-159 reads). */
GRUS_API int grus_graph_save_gr(const grus_graph *g, const char *path);
/* Seeded RMAT (a,b,c,d = .57,.19,.19,.05) generated on the device; the
 * reference has no generator (it reads Galois-converted files, README.md). */
GRUS_API int grus_graph_rmat(int scale, int edge_factor, uint64_t seed,
                    uint32_t gen_flags, int mem_mode, uint64_t budget_bytes,
                    grus_graph **out);
/* rows x cols 4-neighbour grid, vertex id r*cols+c. */
GRUS_API int grus_graph_grid2d(uint32_t rows, uint32_t cols, uint64_t seed,
                      uint32_t gen_flags, grus_graph **out);
GRUS_API int grus_graph_get_info(const grus_graph *g, grus_graph_info *info);
/* Copy CSR (and CSC when built) back to host arrays (any may be NULL). */
GRUS_API int grus_graph_copy_csr(const grus_graph *g, uint32_t *offsets, uint32_t *cols,
                        uint32_t *weights);
/* Device transpose CSR->CSC with weights.  Replaces the host-serial
 * csr_tocsc/CSR2CSC (include/graph.cuh:273-320), which drops weights. */
GRUS_API int grus_graph_build_csc(grus_graph *g);
GRUS_API int grus_graph_copy_csc(const grus_graph *g, uint32_t *t_offsets,
                        uint32_t *t_cols, uint32_t *t_weights);
GRUS_API int grus_graph_set_tuning(grus_graph *g, const grus_tuning *t);
GRUS_API int grus_graph_get_tuning(const grus_graph *g, grus_tuning *t);
GRUS_API int grus_graph_free(grus_graph *g);

/* ---- traversals ----------------------------------------------------------- */
/* Single-source BFS depths.  Replaces the BFS_single_gpu level loop
 * (samples/bfs/bfs.cu:135-173) over kernel<...,Frontier<BDF>> / kernel_pull
 * (include/kernel.cuh:124-165): one persistent direction-optimising launch. */
GRUS_API int grus_bfs(grus_graph *g, uint32_t src, uint32_t *depth, grus_stats *stats,
             void *stream);

/* Multi-source BFS: k <= 64 sources advance together in one persistent
 * launch, one bit per source in a 64-bit word per vertex.  `srcs` (host or
 * device, k entries) may repeat vertices; `depths` holds k*n uint32,
 * source-major (depths[i*n + v] = depth of v from srcs[i], GRUS_INFINIT if
 * unreached).  The reference answers one source per run of its BFS sample
 * (samples/bfs/bfs.cu:135-173).  stats->vertices_reached / edges_reached are
 * summed over the sources. */
GRUS_API int grus_bfs_multi(grus_graph *g, const uint32_t *srcs, int k, uint32_t *depths,
                   grus_stats *stats, void *stream);

/* Multi-source SSSP: k <= 32 sources advance together in one persistent
 * launch over one vertex-major distance matrix, sharing every adjacency
 * read.  `srcs` (host or device) may repeat vertices; `dists` holds k*n
 * uint32, source-major, bit-exact with k grus_sssp calls.  The reference
 * answers one source per run of its SSSP sample (samples/sssp/sssp.cu:
 * 123-170).  stats: levels, threshold advances (direction_switches),
 * relaxations, and reach counts summed over the sources. */
GRUS_API int grus_sssp_multi(grus_graph *g, const uint32_t *srcs, int k, uint32_t *dists,
                    grus_stats *stats, void *stream);

/* Per-level record of the last grus_bfs call made with stats: level i ends
 * end_ns after the kernel started; `vertices` were discovered into level i+1
 * with `edges` out-edges in total; `pull` is 1 for a bottom-up level. */
typedef struct grus_level_trace {
  uint64_t end_ns;
  uint64_t edges;
  uint32_t vertices;
  uint32_t pull;
} grus_level_trace;
/* Copies up to max_levels records; returns how many (>= 0) or a status. */
GRUS_API int grus_bfs_trace(grus_graph *g, grus_level_trace *out, int max_levels);
/* Per-level records of the last grus_sssp call on g made with stats: end
 * time, relaxations (edges), frontier entries (vertices) and the number of
 * threshold advances so far (pull).  Same return convention. */
GRUS_API int grus_sssp_trace(grus_graph *g, grus_level_trace *out, int max_levels);

/* Allocation-free BFS.  No counterpart in the reference.  For callers that
 * cannot allocate device memory (a host process that owns the whole device
 * budget through its own pool, or loops where cudaMalloc's device-wide
 * synchronisation is not acceptable): same algorithm and results as
 * grus_bfs, but on raw device CSR arrays (offsets, cols, depth must be device
 * or managed memory; `symmetric` != 0 lets pull levels use the CSR as
 * in-edges, else the BFS runs push-only) with its scratch in a fixed
 * file-scope device array held by every GPU that loads the library (about
 * 10 MB).  Graphs above the limits below are rejected with GRUS_EOVERFLOW.
 * The arrays must form a valid CSR: offsets[0] == 0, offsets monotone,
 * offsets[n] == m and every cols entry < n.  This is NOT checked (the arrays
 * stay on the device); a column id >= n makes the kernel write past the
 * depth array and past its own scratch, which later calls on that GPU share.
 * The first call on a device (and the first after a cudaDeviceReset) looks
 * the array up; make it before any stream capture.  All calls share the
 * array: calls that overlap on the GPU race.  Asynchronous on `stream` unless
 * `stats` is given; then it waits and reports device-side errors (a grid
 * barrier that timed out).  With stats == NULL such errors are dropped: the
 * next call clears the control block before anyone reads it, so callers who
 * need them must pass stats, which makes the call synchronous. */
#define GRUS_STATIC_MAX_VERTICES (1u << 20)
#define GRUS_STATIC_MAX_EDGES (1u << 25)
GRUS_API int grus_bfs_static(uint64_t n, uint64_t m, const uint32_t *offsets,
                    const uint32_t *cols, int symmetric, uint32_t src, uint32_t *depth,
                    grus_stats *stats, void *stream);

/* Exact single-source shortest paths over uint32 weights (dist in the same
 * units; GRUS_INFINIT unreached).  Replaces SSSP_single_gpu
 * (samples/sssp/sssp.cu:123-170), whose non-atomic relax (:51-60) can lose
 * updates: here a persistent near/far label-correcting launch with atomicMin.
 * stats->edges_relaxed counts edge relaxations attempted. */
GRUS_API int grus_sssp(grus_graph *g, uint32_t src, uint32_t *dist, grus_stats *stats,
              void *stream);

/* Connected components, label[v] = minimum vertex id of v's component (edges
 * taken as undirected).  On a symmetric graph this is the fixpoint of the
 * reference's min-label propagation (samples/cc/cc.cu:69-79, driver :124-190);
 * computed with a min-hooking union-find (Afforest sampling + giant-component
 * skip), bit-exact whatever the schedule. */
GRUS_API int grus_cc(grus_graph *g, uint32_t *label, grus_stats *stats, void *stream);

/* Pull PageRank: r0 = 1/n, r' = (1-d)/n + d * sum r(u)/outdeg(u) over in-edges,
 * `iters` iterations, FP32 ranks with compensated sums; dangling mass is not
 * redistributed (samples/pagerank/pr.cu:29-31,83 never pushes from
 * out-degree-0 vertices).  Builds the CSC on first use.  The reference's own
 * delta-push PR (pr.cu:17-90) is kept by the drop-in headers. */
GRUS_API int grus_pagerank(grus_graph *g, float damping, int iters, float *rank,
                  grus_stats *stats, void *stream);

/* Autotuner: coordinate descent over the grus_tuning knobs of the BFS
 * (alpha, beta, bu_words, huge_degree, ctas_per_sm) or SSSP (sssp_delta,
 * huge_degree, ctas_per_sm) persistent kernel on this graph from `src`, each
 * candidate timed best-of-`reps` with CUDA events.  Stores the fastest on the
 * graph and returns it (and its time).  Outputs do not depend on the knobs.
 * The reference has fixed launch shapes and thresholds. */
GRUS_API int grus_autotune(grus_graph *g, uint32_t algo, uint32_t src, int reps,
                  grus_tuning *best, float *best_ms);

/* ---- batched queries ------------------------------------------------------ */
/* Many BFS / SSSP queries over many resident graphs in one launch.  A worker
 * is one thread-block cluster that takes queries from a device counter and
 * runs each to completion (levels separated by the hardware cluster
 * barrier); per-worker device state is sized for the largest graph.  The
 * reference answers one query per process run. */
typedef struct grus_query {
  uint32_t graph;        /* index into the graphs given at creation */
  uint32_t algo;         /* GRUS_ALGO_BFS or GRUS_ALGO_SSSP */
  uint32_t src;
  uint32_t reserved;
  uint64_t out_offset;   /* result = out + out_offset, n of the graph entries */
} grus_query;

typedef struct grus_batch_config {
  uint32_t cluster_size; /* CTAs per worker (1..16, default 16) */
  uint32_t workers;      /* 0 = as many as fit */
  uint32_t huge_degree;  /* hub chunking threshold */
  uint32_t sssp_delta;   /* SSSP bucket width */
  uint32_t group_sources;/* SSSP queries on one graph packed per multi-source
                            task (1..32; default 1 = no packing: on a 16-CTA
                            worker a pack of 8 costs about 3.3 single
                            queries, so packing pays only when workers would
                            otherwise idle, e.g. many queries on few small
                            graphs) */
  uint32_t big_edges;    /* queries on graphs with at least this many edges
                            run as whole-GPU launches before the cluster
                            workers start: SSSP packed up to 32 sources
                            per graph, BFS up to 64 per launch when enough
                            share a graph, else one launch each (default
                            2^21; 0xFFFFFFFF: never) */
  uint32_t launch_entries;/* the SSSP packs of several of those graphs share
                            one launch while their distance rows (vertices
                            x 8/16/32 sources) total at most this many
                            entries (default 2^23 = 32 MiB, which stays in
                            L2; 1: one graph per launch) */
} grus_batch_config;

typedef struct grus_batch grus_batch;

GRUS_API int grus_batch_create(grus_graph *const *graphs, int ngraphs,
                      const grus_batch_config *cfg, grus_batch **out);
/* Runs queries[0..nq); `out` is device memory.  use_graph != 0 replays a
 * captured CUDA graph (task upload, counter reset, kernel) re-captured only
 * when nq, out or stream change.  Asynchronous unless stats is given. */
GRUS_API int grus_batch_run(grus_batch *b, const grus_query *queries, int nq, uint32_t *out,
                   int use_graph, grus_stats *stats, void *stream);
GRUS_API int grus_batch_get_info(const grus_batch *b, grus_batch_config *info);
GRUS_API int grus_batch_free(grus_batch *b);

/* ---- tooling ----------------------------------------------------------------- */
/* Converts a text edge list ("u v [w]" per line, 0-based, '#' comments) or a
 * Matrix Market coordinate file (1-based; "symmetric" in its header implies
 * GRUS_GEN_SYMMETRIC, "pattern" drops weights) to the Galois v1 .gr layout.
 * flags: GRUS_GEN_SYMMETRIC adds reverse edges and keeps one (u, v) per pair
 * (the lightest); GRUS_GEN_WEIGHTED keeps the third column as uint32 weights
 * (1 where absent).  The reference relies on Galois' graph-convert for this
 * (README.md:14-27). */
GRUS_API int grus_convert_edgelist(const char *in_path, const char *out_path, uint32_t flags);

/* Binary dump of a result array (host or device): "GRUSRES1", uint32 type,
 * uint32 element size (4), uint64 n, then the n values.  Beside the
 * reference's text SaveResults (include/print.cuh:36-45). */
#define GRUS_RESULT_U32 0u
#define GRUS_RESULT_F32 1u
GRUS_API int grus_save_result(const char *path, const void *values, uint64_t n, uint32_t type);

/* Device telemetry of the current device, the quantities the reference's
 * tools/pcie.py polls: device memory (CUDA), and through NVML, opened at run
 * time, host-link throughput (NVML's PCIe counters, KB/s, sampled over about
 * 20 ms), SM and memory clocks, power, temperature, driver version.  Only
 * reads; `valid` tells which fields were available.  GRUS_ENODEV without a
 * device. */
#define GRUS_TEL_HBM 1u
#define GRUS_TEL_LINK 2u
#define GRUS_TEL_CLOCKS 4u
#define GRUS_TEL_POWER 8u
#define GRUS_TEL_TEMP 16u
#define GRUS_TEL_DRIVER 32u
typedef struct grus_telemetry {
  uint64_t hbm_total_bytes, hbm_free_bytes;
  uint32_t link_tx_kbps, link_rx_kbps;
  uint32_t sm_clock_mhz, mem_clock_mhz;
  uint32_t power_mw, temperature_c;
  uint32_t valid, reserved;
  char driver_version[32];
} grus_telemetry;
GRUS_API int grus_telemetry_sample(grus_telemetry *out);

/* ---- serving --------------------------------------------------------------- */
/* A query server over device-resident graphs.  Requests queue on the host
 * and are served by two lanes.  Small graphs (fewer than big_edges edges): a
 * scheduler thread admits each query into a worker slot (one cluster worker
 * of the batch engine with its own device state and stream) as soon as a slot
 * is free, allocating a slot's state only if free HBM covers it plus
 * hbm_reserve_bytes; admitted queries overlap on the device.  Big graphs: a
 * second thread queues whole-GPU persistent launches back to back on a
 * high-priority stream, and packs the queued SSSP queries on the same graph
 * (up to 32) into one multi-source launch, and the queued BFS queries on it
 * (up to 64) when enough are queued; a graph's workspace is allocated only
 * if free HBM covers it plus the reserve.  Latency is measured from submit to observed completion on the
 * host clock. */
typedef struct grus_server grus_server;

typedef struct grus_server_config {
  uint32_t slots;            /* concurrent queries (default 16) */
  uint32_t cluster_size;     /* CTAs per query (1..16, default 8) */
  uint64_t hbm_reserve_bytes;/* free HBM kept back at admission (default 1 GiB) */
  uint32_t sssp_delta;
  uint32_t big_edges;        /* graphs with at least this many edges run on the
                                whole-GPU lane (default 2^20; 0xFFFFFFFF: never) */
  uint32_t bfs_pack_min;     /* whole-GPU lane: fewest queued BFS requests on one
                                graph that share one multi-source launch (up to
                                64); 0 = by graph size (8 below 2^25 edges, 16
                                below 2^27, 24 below 2^28, else 32) */
} grus_server_config;

typedef struct grus_completion {
  uint64_t tag;
  int32_t status;
  uint32_t reserved;
  double latency_us;
} grus_completion;

typedef struct grus_server_stats {
  uint64_t submitted, admitted, completed, pending, rejected;
  uint32_t slots, slots_ready;
  uint64_t big_launches;     /* whole-GPU launches of the big-graph lane */
  uint64_t big_queries;      /* queries they served (SSSP queries on one graph
                                share a multi-source launch) */
  uint64_t kernel_launches;  /* kernels launched for queries, both lanes */
} grus_server_stats;

GRUS_API int grus_server_create(grus_graph *const *graphs, int ngraphs,
                       const grus_server_config *cfg, grus_server **out);
/* Queues one query; `out` (device memory, n of the graph entries) receives
 * the depths (BFS) or distances (SSSP).  Returns at once. */
GRUS_API int grus_server_submit(grus_server *s, uint32_t graph, uint32_t algo, uint32_t src,
                       uint32_t *out, uint64_t tag);
/* Collects up to max completions, waiting up to wait_ms for the first;
 * returns how many were written. */
GRUS_API int grus_server_poll(grus_server *s, grus_completion *out, int max, int wait_ms);
GRUS_API int grus_server_get_stats(grus_server *s, grus_server_stats *st);
GRUS_API int grus_server_destroy(grus_server *s);

/* ---- autotuning of the batched and served forms ------------------------------ */
/* No counterpart in the reference, whose thresholds are fixed constants
 * (include/common.cuh:30, include/frontier.cuh:140).  Both run coordinate
 * descent over their engine's knobs on the caller's own query mix, starting
 * from *best (zeros: defaults), and write the fastest setting back to *best.
 * Results are the same under every setting, so tuning never trades
 * correctness.  The graphs must stay unchanged while tuning runs.
 *
 * grus_batch_autotune: big_edges, launch_entries, cluster_size,
 * group_sources and sssp_delta, each candidate timed as grus_batch_run with
 * CUDA-graph replay (best of `reps` device times, *best_ms).  The query
 * offsets define the output layout; the tuner allocates its own output. */
GRUS_API int grus_batch_autotune(grus_graph *const *graphs, int ngraphs,
                                 const grus_query *queries, int nq, int reps,
                                 grus_batch_config *best, float *best_ms);
/* grus_server_autotune: big_edges, bfs_pack_min, slots and cluster_size,
 * each candidate a fresh server given every query at once (saturated
 * throughput, host clock, best of `reps` bursts after a warm-up burst,
 * *best_qps).  out_offset of the queries is ignored; a setting under which
 * admission refuses queries is skipped. */
GRUS_API int grus_server_autotune(grus_graph *const *graphs, int ngraphs,
                                  const grus_query *queries, int nq, int reps,
                                  grus_server_config *best, float *best_qps);

#ifdef __cplusplus
}
#endif
#endif /* GRUS_H */
