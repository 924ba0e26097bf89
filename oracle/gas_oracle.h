/*
 * TEST INFRASTRUCTURE ONLY -- the oracle.
 *
 * A plain-C restatement of vertexAPI2's sequential CPU engine
 * GASEngineRef (refgas.h:31-225), its host CSR/CSC builder
 * (util.h:44-121) and the example vertex programs (bfs.cu:31-78,
 * sssp.cu:25-64, connected_component.cu:25-63, pagerank.cu:27-73), driven
 * exactly as the example drivers drive them (bfs.cu:91-112, sssp.cu:67-82,
 * connected_component.cu:66-81, pagerank.cu:76-101).
 *
 * It is the checker for the CUDA engine in tests/, in smoke() and in the
 * CPU-baseline leg of bench.py.  Nothing in the product links or calls it.
 *
 * Parity of this restatement is pinned two ways:
 *   - against the reference engine itself: oracle/build.py compiles
 *     refgas.h + util.h in place into oracle/_ref/libgas_ref.so and
 *     tests/test_oracle.py compares both engines on the reference's own
 *     fixture graphs and on synthetic graphs;
 *   - against golden vectors produced by that compiled reference engine
 *     (tests/golden/make_golden.py), which travel with the repository.
 *
 * One documented difference: util.h:48-72 orders the edges of one vertex
 * with std::sort (unstable), whose tie order is a libstdc++ detail.  This
 * restatement uses a stable counting sort (ties keep edge-list order).
 * Integer programs (BFS, SSSP, CC) are order independent; FP32 PageRank
 * sums in a different order and agrees to within FP32 rounding.
 */
#ifndef GAS_ORACLE_H
#define GAS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-run instrumentation (outside the engine's own loop, mirroring the
 * counts the GPU engine reports so per-iteration bytes can be compared). */
typedef struct {
  int32_t iterations;        /* gather/apply/scatter rounds executed       */
  int32_t capacity;          /* entries available in the arrays below      */
  int64_t *active;           /* |A_k|: active vertices at iteration k      */
  int64_t *edges_gathered;   /* sum of in-degrees of A_k                   */
  int64_t *ret;              /* |R_k|: vertices whose apply returned true  */
  int64_t *edges_scattered;  /* sum of out-degrees of R_k                  */
  int64_t run_ns;            /* wall time of run()+getResults()            */
} ora_stats;

/* util.h:79-110 edgeListToCSR (stable within a key). offsets has nV+1
 * entries; out_dsts / sort_idx may be NULL. */
void ora_edge_list_to_csr(int32_t nV, int32_t nE, const int32_t *srcs,
                          const int32_t *dsts, int32_t *offsets,
                          int32_t *out_dsts, int32_t *sort_idx);

/* bfs.cu:148-166: first vertex with the strictly largest out-degree. */
int32_t ora_max_outdegree_vertex(int32_t nV, int32_t nE, const int32_t *srcs);

/* All run functions return 0 on success, nonzero on bad arguments.
 * stats may be NULL. */
int ora_run_bfs(int32_t nV, int32_t nE, const int32_t *srcs,
                const int32_t *dsts, int32_t source, int32_t *depth,
                ora_stats *stats);

int ora_run_sssp(int32_t nV, int32_t nE, const int32_t *srcs,
                 const int32_t *dsts, const int32_t *weights, int32_t source,
                 int32_t *dist, ora_stats *stats);

/* SSSP whose Program::scatter writes each visited edge (visits += 1,
 * last = source distance): the engine's scatter call (refgas.h:171-197). */
int ora_run_sssp_visits(int32_t nV, int32_t nE, const int32_t *srcs,
                        const int32_t *dsts, const int32_t *weights, int32_t source,
                        int32_t *dist, int32_t *visits, int32_t *last, ora_stats *stats);

int ora_run_cc(int32_t nV, int32_t nE, const int32_t *srcs,
               const int32_t *dsts, int32_t *label, ora_stats *stats);

/* PageRank as pagerank.cu:27-101; max_iters <= 0 means "until no vertex
 * is active" (the reference's run()), otherwise an explicit capped loop. */
int ora_run_pagerank_f32(int32_t nV, int32_t nE, const int32_t *srcs,
                         const int32_t *dsts, int32_t max_iters, float *rank,
                         ora_stats *stats);
int ora_run_pagerank_f64(int32_t nV, int32_t nE, const int32_t *srcs,
                         const int32_t *dsts, int32_t max_iters,
                         double *rank, ora_stats *stats);

/* Personalised PageRank (no counterpart in the reference; written against
 * the same Program contract, modelled on pagerank.cu:27-73):
 *   rank_v <- alpha*[v==source] + (1-alpha) * sum_{u->v} rank_u/outdeg_u
 * starting from rank = [v==source], every vertex active, `iters` rounds. */
int ora_run_ppr_f32(int32_t nV, int32_t nE, const int32_t *srcs,
                    const int32_t *dsts, int32_t source, float alpha,
                    int32_t iters, float *rank, ora_stats *stats);
int ora_run_ppr_f64(int32_t nV, int32_t nE, const int32_t *srcs,
                    const int32_t *dsts, int32_t source, double alpha,
                    int32_t iters, double *rank, ora_stats *stats);

/* Seeded synthetic graphs (gas_oracle_gen.c): an implementation of the
 * benchmark's R-MAT and lattice generators independent of the product
 * library, so that CPU-only measurements never load it.  Outputs are
 * malloc'd; release them with ora_graph_free.  Return 0 on success. */
typedef struct {
  int32_t nVertices;
  int64_t nEdges;
  int32_t *srcs, *dsts, *weights; /* weights NULL when none were asked for */
} ora_graph;

int ora_gen_rmat(int32_t scale, int32_t edgeFactor, double a, double b, double c,
                 uint64_t seed, int32_t symmetrize, int32_t wLo, int32_t wHi, ora_graph *out);
int ora_gen_grid(int32_t rows, int32_t cols, double pDelete, uint64_t seed, int32_t wLo,
                 int32_t wHi, ora_graph *out);
void ora_graph_free(ora_graph *g);

#ifdef __cplusplus
}
#endif
#endif
