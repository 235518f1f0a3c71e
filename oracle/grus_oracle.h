/*
 * grus_oracle.h -- CPU oracle for the Grus frontier-traversal path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the grus_framework_gb300
 * package, libgrus.so, the mgg drop-in headers) links, loads or calls this
 * library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * legs use it, and only as the checker or as the timed CPU baseline.
 *
 * What it restates (reference paths are relative to the Grus project root):
 *   - the Galois v1 .gr layout read by include/graph_loader.cuh:65-159,
 *   - the serial CSR->CSC transpose of include/graph.cuh:273-303 (plus the
 *     weight permutation the reference leaves commented out at :294),
 *   - the fixpoints of the sample operators:
 *       BFS  samples/bfs/bfs.cu:18-87      (depth from src, INFINIT unreached)
 *       SSSP samples/sssp/sssp.cu:51-60    (exact shortest paths = Dijkstra)
 *       CC   samples/cc/cc.cu:69-79        (minimum vertex id per component)
 *       PR   pull PageRank in FP64 (r0=1/n, r'=(1-d)/n + d*sum r/outdeg,
 *            dangling mass not redistributed, matching samples/pagerank/pr.cu
 *            which never pushes from out-degree-0 vertices, :29-31,83),
 *       delta-PR, the algorithm of samples/pagerank/pr.cu:17-90 (sequential).
 *   - seeded RMAT / 2-D grid generators, restated from the generator
 *     specification in grus_framework_gb300 (the reference ships none).
 *   - OpenMP "same algorithm" baselines that are timed as the CPU path.
 *
 * Parity pins: the .gr reader and the transpose are pinned against the
 * reference's own host code compiled and run in the build container
 * (oracle/ref_pin.cu -> tests/golden/ref_pin_*.txt).  The traversal oracles
 * are pinned against hand-computed known answers and networkx; the reference
 * has no CPU implementation, no tests and no golden vectors for them, so
 * against the reference itself their parity is unpinned.
 *
 * All functions return 0 on success and a negative errno-style code on error.
 */
#ifndef GRUS_ORACLE_H
#define GRUS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_INFINIT 4294967294u /* include/common.cuh:52, UINT_MAX-1 */

/* generator flag bits (same meaning as GRUS_GEN_* in include/grus.h) */
#define ORC_GEN_SYMMETRIC 1u
#define ORC_GEN_WEIGHTED 2u
#define ORC_GEN_RELABEL 4u

/* ---- graph construction ------------------------------------------------ */
/* Builds a CSR with malloc'ed arrays (free with orc_free).  *wts is NULL when
 * ORC_GEN_WEIGHTED is not set. */
int orc_rmat_csr(int scale, int edge_factor, uint64_t seed, uint32_t flags,
                 uint64_t *n, uint64_t *m, uint32_t **offs, uint32_t **cols,
                 uint32_t **wts);
int orc_grid_csr(uint32_t rows, uint32_t cols_, uint64_t seed, uint32_t flags,
                 uint64_t *n, uint64_t *m, uint32_t **offs, uint32_t **cols,
                 uint32_t **wts);
/* Raw RMAT endpoints of edge i before relabelling (for generator tests). */
void orc_rmat_edge(int scale, uint64_t seed, uint64_t i, uint32_t *u,
                   uint32_t *v);
uint32_t orc_relabel(int scale, uint64_t seed, uint32_t x);
uint32_t orc_edge_weight(uint64_t seed, uint32_t u, uint32_t v);
void orc_free(void *p);

/* ---- .gr file I/O (include/graph_loader.cuh:65-159) ------------------- */
int orc_read_gr(const char *path, uint64_t *n, uint64_t *m, uint32_t **offs,
                uint32_t **cols, uint32_t **wts);
int orc_write_gr(const char *path, uint64_t n, uint64_t m,
                 const uint32_t *offs, const uint32_t *cols,
                 const uint32_t *wts);

/* ---- transpose (include/graph.cuh:273-303) ----------------------------- */
void orc_csr_to_csc(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                    const uint32_t *wts, uint32_t *t_offs, uint32_t *t_cols,
                    uint32_t *t_wts);

/* ---- serial oracles ---------------------------------------------------- */
uint32_t orc_max_degree_vertex(uint64_t n, const uint32_t *offs);
int orc_bfs(uint64_t n, const uint32_t *offs, const uint32_t *cols,
            uint32_t src, uint32_t *depth);
int orc_sssp(uint64_t n, const uint32_t *offs, const uint32_t *cols,
             const uint32_t *wts, uint32_t src, uint32_t *dist);
int orc_cc(uint64_t n, const uint32_t *offs, const uint32_t *cols,
           uint32_t *label);
int orc_pagerank(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                 double damping, int iters, double *rank);
int orc_delta_pagerank(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                       float *rank, uint32_t *iterations);
/* Reached-edge accounting: m_r = sum of out-degrees over reached vertices. */
uint64_t orc_reached_edges(uint64_t n, const uint32_t *offs,
                           const uint32_t *depth);
/* Multi-source BFS oracle: k serial BFS runs, depths[k*n]. */
int orc_bfs_multi(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                  const uint32_t *srcs, int k, uint32_t *depths);

/* ---- OpenMP baselines (timed CPU path); return seconds or <0 on error -- */
double orc_omp_bfs(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                   uint32_t src, uint32_t *depth, int threads);
double orc_omp_sssp(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                    const uint32_t *wts, uint32_t src, uint32_t *dist,
                    int threads);
double orc_omp_cc(uint64_t n, const uint32_t *offs, const uint32_t *cols,
                  uint32_t *label, int threads);
double orc_omp_pagerank(uint64_t n, const uint32_t *t_offs,
                        const uint32_t *t_cols, const uint32_t *outdeg,
                        float damping, int iters, float *rank, int threads);
int orc_omp_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
