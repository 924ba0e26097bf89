/*
 * gas_gb300.h -- C ABI of the GB300 Gather-Apply-Scatter engine.
 *
 * Two layers, both plain C (pointers, sizes, status codes; no C++ or torch
 * types), exported from libgas_gb300.so:
 *
 *  1. The engine layer (gas_engine_*): one call per method of vertexAPI2's
 *     GASEngineGPU (gpugas.h:74-773), for the built-in vertex programs
 *     (BFS, SSSP, connected components, PageRank, personalised PageRank).
 *     This is what an FFI binding (ctypes, cgo, JNI) of the reference path
 *     would bind.
 *
 *  2. The core layer (gas_core_*, declared in gas_gb300_core.h): the
 *     Program-independent half of the engine.  The C++ header
 *     gas_gb300/gpugas.cuh drives it for user-written vertex programs,
 *     whose gather/apply kernels are instantiated in the user's own
 *     translation unit (Programs are compile-time types, as in gpugas.h).
 *
 * Every function returns a gas_status (0 = GAS_OK).  No function aborts the
 * process; gas_last_error() gives a one-line description of the most recent
 * failure on the calling thread.  An engine or state object is used by one
 * host thread at a time.
 */
#ifndef GAS_GB300_H
#define GAS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GAS_API __attribute__((visibility("default")))
#else
#define GAS_API
#endif

typedef int32_t gas_status;
enum {
  GAS_OK = 0,
  GAS_ERR_INVALID = 1,      /* bad argument (null pointer, id out of range, ...) */
  GAS_ERR_OOM = 2,          /* device or host allocation failed                   */
  GAS_ERR_CUDA = 3,         /* a CUDA runtime call failed                          */
  GAS_ERR_TIMEOUT = 4,      /* a bounded device-side wait gave up                  */
  GAS_ERR_STATE = 5,        /* call out of order (e.g. no graph set)               */
  GAS_ERR_UNSUPPORTED = 6,  /* feature not available for this program / size       */
  GAS_ERR_NO_DEVICE = 7     /* no CUDA device, or the device is not sm_103         */
};

/* Program ids of the built-in vertex programs (engine layer). */
enum {
  GAS_PROGRAM_BFS = 1,       /* bfs.cu:31-78                       VertexData int32 depth      */
  GAS_PROGRAM_SSSP = 2,      /* sssp.cu:25-64                      VertexData int32, EdgeData int32 */
  GAS_PROGRAM_CC = 3,        /* connected_component.cu:25-63       VertexData int32 label      */
  GAS_PROGRAM_PAGERANK = 4,  /* pagerank.cu:27-73                  VertexData {float rank; int32 numOutEdges} */
  GAS_PROGRAM_PPR = 5        /* personalised PageRank, alpha 0.15 (no reference counterpart)
                                VertexData {float rank; int32 numOutEdges; float teleport} */
};

typedef struct gas_engine_s gas_engine;

/* ---------------- engine layer (GASEngineGPU, gpugas.h) ------------------ */

/* Replaces the GASEngineGPU constructor (gpugas.h:144-172), which bound the
 * engine to device 0 and the default stream.  `stream` is a cudaStream_t
 * (NULL = the legacy default stream). */
GAS_API gas_status gas_engine_create(int32_t program, int32_t device, void *stream,
                                     gas_engine **out);

/* Replaces ~GASEngineGPU (gpugas.h:175-197). NULL is accepted. */
GAS_API gas_status gas_engine_destroy(gas_engine *e);

/* Replaces setGraph (gpugas.h:212-322): builds CSC (gather) and CSR
 * (scatter) on the device from the edge list, sorts edge data into CSC order
 * and copies vertex data to the device.  vertexData / edgeData are borrowed
 * host arrays of the program's VertexData / EdgeData (either may be NULL,
 * as in the reference); getResults writes back into them. */
GAS_API gas_status gas_engine_set_graph(gas_engine *e, int32_t nVertices, void *vertexData,
                                        int32_t nEdges, void *edgeData,
                                        const int32_t *edgeListSrcs,
                                        const int32_t *edgeListDsts);

/* Replaces getResults (gpugas.h:329-338): copies vertex data (and edge
 * data, in the caller's original edge order) back to the host arrays. */
GAS_API gas_status gas_engine_get_results(gas_engine *e);

/* Re-uploads vertex data from `host` (nVertices elements) without rebuilding
 * the graph; the vertex-data half of setGraph (gpugas.h:221-226). */
GAS_API gas_status gas_engine_set_vertex_data(gas_engine *e, const void *host);

/* Replaces setActive (gpugas.h:342-349): active set = [start, end).
 * Starts a new traversal: the round number handed to programs that take
 * one (BFS depth) restarts at 0. */
GAS_API gas_status gas_engine_set_active(gas_engine *e, int32_t vertexStart, int32_t vertexEnd);

/* Replaces countActive (gpugas.h:353-356).  Waits for queued work. */
GAS_API gas_status gas_engine_count_active(gas_engine *e, int32_t *nActive);

/* Replaces gatherApply (gpugas.h:421-513).  Asynchronous. */
GAS_API gas_status gas_engine_gather_apply(gas_engine *e, int32_t haveGather);

/* Replaces scatterActivate (gpugas.h:669-751).  Asynchronous: the next
 * active set is built on the device (no host round trip). */
GAS_API gas_status gas_engine_scatter_activate(gas_engine *e, int32_t haveScatter);

/* Replaces nextIter (gpugas.h:754-758).  nActive may be NULL (then the
 * call does not wait); otherwise it waits and returns the new count. */
GAS_API gas_status gas_engine_next_iter(gas_engine *e, int32_t *nActive);

/* Replaces run (gpugas.h:764-772): iterate until no vertex is active, or
 * for at most maxIters rounds when maxIters > 0.  iterations (may be NULL)
 * receives the number of non-empty rounds executed.  After a run that
 * stopped at maxIters, a later run or the stepwise calls continue from the
 * next round's frontier. */
GAS_API gas_status gas_engine_run(gas_engine *e, int32_t maxIters, int32_t *iterations);

/* Replaces the BFS driver's setIterationCount<true> (bfs.cu:81-88,
 * cudaMemcpyToSymbol of g_iterationCountGPU): the iteration number the
 * built-in BFS program writes as depth on the next gatherApply. */
GAS_API gas_status gas_engine_set_iteration(gas_engine *e, int32_t iteration);

/* Per-round counts of the last run()/stepwise sequence since setActive:
 * for round k, active[k] = |A_k|, gathered[k] = in-edges of A_k,
 * ret[k] = vertices whose apply returned true, scattered[k] = their
 * out-edges.  Arrays may be NULL; `capacity` bounds what is written.
 * *rounds receives the number of rounds recorded. */
GAS_API gas_status gas_engine_round_stats(gas_engine *e, int32_t capacity, int64_t *active,
                                          int64_t *gathered, int64_t *ret,
                                          int64_t *scattered, int32_t *rounds);

/* Elapsed device time (ms, CUDA events on the engine's stream) of the most
 * recent gas_engine_run call. */
GAS_API gas_status gas_engine_last_run_ms(gas_engine *e, float *ms);

/* Device-side copy of the current vertex data (saved once, restored any
 * number of times, asynchronously on the engine's stream): repeated runs
 * on a resident graph without a host round trip. */
GAS_API gas_status gas_engine_save_vertex_data(gas_engine *e);
GAS_API gas_status gas_engine_restore_vertex_data(gas_engine *e);

/* Per-kernel timing of run(): when enabled, every gather/apply and
 * scatter/activate launch of run() is bracketed by CUDA events on the
 * engine's stream; gas_engine_kernel_times returns the summed device
 * milliseconds and launch counts of the most recent run(). */
GAS_API gas_status gas_engine_set_profiling(gas_engine *e, int32_t enabled);
GAS_API gas_status gas_engine_kernel_times(gas_engine *e, float *gatherMs, float *scatterMs,
                                           int32_t *gatherLaunches, int32_t *scatterLaunches);

/* Launch shape of run(): persistent != 0 runs every round in one
 * cooperative kernel (the default), 0 launches each phase of each round;
 * runBlocksPerSM bounds the persistent kernel's CTAs per SM (0 = the
 * default: 2 on graphs whose degrees are all <= 8, else 4).  Results do not
 * depend on either. */
GAS_API gas_status gas_engine_set_launch_config(gas_engine *e, int32_t persistent,
                                                int32_t runBlocksPerSM);

/* Frontier policy of run(): a round runs dense -- one pull pass over every
 * vertex's in-edges, the reference's dense path (gpugas.h:689-717) without
 * its scan -- when the previous round's apply-returned-true vertices have
 * more than nEdges/alpha out-edges (the reference switches at nEdges/100);
 * 0 keeps every round on frontier lists.  Results do not depend on it. */
GAS_API gas_status gas_engine_set_dense_policy(gas_engine *e, int32_t alpha);
/* One-phase list rounds on graphs whose degrees are all <= 8 (default on);
 * see gas_core_set_fused_rounds.  Results do not depend on it. */
GAS_API gas_status gas_engine_set_fused_rounds(gas_engine *e, int32_t on);

/* Breadth-first search that allocates nothing (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc -- device memory
 * already claimed by another allocator, or a serving thread that must not
 * pay cudaMalloc's device synchronisation -- the graph and the result live
 * in device memory the caller owns: outOffsets[nVertices+1] and
 * outDests[nEdges] (CSR), depth[nVertices] (written: -1 unreached, else the
 * round at which the vertex was reached, as bfs.cu:31-78).  All scratch is
 * one fixed file-scope __device__ array (about 3.4 MB), so graphs are
 * limited to GAS_NOALLOC_MAX_VERTICES vertices and GAS_NOALLOC_MAX_EDGES
 * edges; larger ones are rejected with GAS_ERR_INVALID.  A GPU holds the
 * array from the time the library's device code is loaded on it until the
 * process exits; under CUDA's default lazy loading that is the first call
 * on the device, which can therefore fail with an out-of-memory status when
 * another allocator has already taken the free memory.  That first call on
 * a device also looks up the array's device address (kept for the process's
 * life: calls after a cudaDeviceReset are not supported), so make it before
 * any stream capture.  Every call reuses the same array: calls that overlap
 * on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  Runs on `stream` (a cudaStream_t, NULL =
 * legacy default stream) and blocks until the search is done; *rounds (may
 * be NULL) receives the number of rounds. */
#define GAS_NOALLOC_MAX_VERTICES 65536
#define GAS_NOALLOC_MAX_EDGES 2097152
GAS_API gas_status gas_bfs_noalloc(int32_t nVertices, int32_t nEdges, const int32_t *outOffsets,
                                   const int32_t *outDests, int32_t source, int32_t *depth,
                                   void *stream, int32_t *rounds);

/* ---------------- batched multi-source queries --------------------------- */
/* Many BFS, SSSP or personalised PageRank queries with their own sources on
 * one resident graph (no counterpart in the reference, which runs one
 * source per engine).  Each group of up to 256 queries is one persistent
 * launch, captured once per shape into a CUDA graph and replayed; every BFS
 * or SSSP query's result equals its single-source gas_engine_run result bit
 * for bit, and every PPR query's ranks equal the served PPR query's (the
 * same sums in the same order: a left fold in CSC order for vertices of
 * in-degree <= 4096, bit for bit the FP32 oracle's). */
typedef struct gas_batch_s gas_batch;

GAS_API gas_status gas_batch_create(int32_t device, void *stream, gas_batch **out);
GAS_API gas_status gas_batch_destroy(gas_batch *b);
/* Edge list as gas_engine_set_graph; weights (int32, may be NULL) are the
 * SSSP edge lengths. */
GAS_API gas_status gas_batch_set_graph(gas_batch *b, int32_t nVertices, int32_t nEdges,
                                       const int32_t *srcs, const int32_t *dsts,
                                       const int32_t *weights);
/* program = GAS_PROGRAM_BFS, GAS_PROGRAM_SSSP or GAS_PROGRAM_PPR (alpha
 * 0.15, teleport to the source, 20 rounds, every vertex active at the
 * start as the serving loop runs it).  results (may be NULL) is a host
 * array of nQueries * nVertices 4-byte values, query-major: BFS depth
 * (int32, -1 = unreached), SSSP distance (int32, 2147383647 = unreached,
 * sssp.cu:32-33) or PPR rank (float32).  *rounds receives the largest round
 * count of the batches. */
GAS_API gas_status gas_batch_run(gas_batch *b, int32_t program, int32_t nQueries,
                                 const int32_t *sources, int32_t *results, int32_t *rounds);
/* Work units of at most chunkEdges in-edges, CTAs per SM (0 = as many as
 * fit), CUDA-graph replay on/off.  Results do not depend on them. */
GAS_API gas_status gas_batch_set_config(gas_batch *b, int32_t chunkEdges, int32_t blocksPerSM,
                                        int32_t useGraphs);
/* Times candidate configurations on nQueries random sources and keeps the
 * fastest, one setting at a time: for SSSP the bucket width
 * (gas_batch_set_delta); for BFS and SSSP the frontier form
 * (gas_batch_set_frontier, where pairs are allowed) and, for vertex-mask
 * frontiers, the push/pull switch alpha (gas_batch_set_policy); then the
 * work-unit chunk (edges per warp unit, i.e. warps per high-degree vertex)
 * and CTAs per SM (PPR: CTAs per SM only).  Reports the chosen chunk size
 * and CTAs per SM; gas_batch_get_tuning reads every setting. */
GAS_API gas_status gas_batch_autotune(gas_batch *b, int32_t program, int32_t nQueries,
                                      int32_t *chunkEdges, int32_t *blocksPerSM);
/* The current settings: chunk edges, CTAs per SM, alpha, frontier form,
 * SSSP bucket width (any pointer may be NULL). */
GAS_API gas_status gas_batch_get_tuning(gas_batch *b, int32_t *chunkEdges, int32_t *blocksPerSM,
                                        int32_t *alpha, int32_t *frontier, int32_t *delta);
/* Round policy: a round pushes from the vertices that changed last round
 * when their out-degree total times alpha is at most nEdges, otherwise it
 * pulls over every vertex (default alpha 10; 0 = always push).  Results do
 * not depend on it. */
GAS_API gas_status gas_batch_set_policy(gas_batch *b, int32_t alpha);
/* SSSP bucket width: 0 relaxes every changed (vertex, query) pair each
 * round (Bellman-Ford rounds, the reference's order); delta > 0 relaxes a
 * query's pairs in order of distance, delta at a time (delta-stepping),
 * which cuts repeated relaxations on high-diameter weighted graphs.
 * Results do not depend on it.  gas_batch_autotune sets it for SSSP. */
GAS_API gas_status gas_batch_set_delta(gas_batch *b, int32_t delta);
/* Frontier representation: 0 = changed vertices with query masks (any
 * graph); 1 = changed (vertex, query) pairs, one lane each (used when every
 * out-degree is <= 64 and vertices x queries < 2^31, else masks); -1 =
 * automatic (the default: pairs where allowed).  Results do not depend on
 * it. */
GAS_API gas_status gas_batch_set_frontier(gas_batch *b, int32_t mode);
GAS_API gas_status gas_batch_get_delta(gas_batch *b, int32_t *delta);
/* Device milliseconds of the most recent gas_batch_run. */
GAS_API gas_status gas_batch_last_ms(gas_batch *b, float *ms);

/* ---------------- serving loop ------------------------------------------ */
/* A request loop over graphs kept resident on one device (no counterpart in
 * the reference).  Queries -- BFS, SSSP or personalised PageRank (PPR:
 * alpha 0.15, teleport to the source, 20 rounds) from one source on one
 * resident graph -- are submitted at any time from any thread.  A
 * scheduler thread batches the queries waiting for the same graph and
 * program into one batch (up to maxBatch queries) whenever one of `lanes`
 * streams is free and device memory admits it, and advances every batch in
 * flight round by round, so batches on different lanes share the device
 * and new queries start while others run (continuous batching).
 *
 * Admission by free device memory: a batch of n queries on a graph of V
 * vertices, with rows of Q queries (the next power of two >= n; at least 32
 * for BFS and SSSP) and E edges, needs working state of (BFS) V*Q*4 +
 * V*(Q/8)*4 + 28*V + 24*E/512 bytes, (SSSP) V*Q*4 + V*(Q/32)*12 + 28*V +
 * 24*E/512, (PPR) V*Q*16 plus Q*4 bytes per 4096 in-edges of vertices
 * above 4096, plus V*n*4 for its results.  It starts only
 * when cudaMemGetInfo's free bytes plus the server pool's cached bytes,
 * minus reserveBytes, cover it; otherwise the batch shrinks (in steps of
 * 32 queries) or waits for a running batch to release memory.  A query
 * that cannot fit even alone on an idle device fails with GAS_ERR_OOM.
 *
 * Results: BFS depth (-1 unreached) and SSSP distance (2147383647
 * unreached) as int32, PPR rank as float, nVertices values per query; each
 * equals the query's single-source result (BFS, SSSP: bit for bit with
 * gas_engine_run; PPR: bit for bit with the reference engine's CPU loop in
 * FP32) whatever the batch it ran in.  They stay in device memory until
 * gas_server_wait fetches them. */
typedef struct gas_server_s gas_server;

typedef struct {
  int32_t lanes;         /* batches in flight at once, one stream each (1..16; default 4) */
  int32_t maxBatch;      /* queries per batch (1..256; default 256)                     */
  int64_t reserveBytes;  /* device memory admission leaves free (default 1 GiB)          */
} gas_server_config;

typedef struct {
  int32_t status;     /* gas_status of the query                           */
  int32_t program;
  int32_t graph;
  int32_t source;
  int32_t rounds;     /* rounds its batch ran                              */
  int32_t batchSize;  /* queries in that batch                             */
  int32_t lane;
  int32_t pad;
  int64_t submitNs;   /* steady-clock nanoseconds: submitted, batch        */
  int64_t admitNs;    /* admitted, results complete in device memory        */
  int64_t doneNs;
} gas_query_info;

typedef struct {
  int64_t submitted, completed, failed;
  int64_t batches;           /* batches started                               */
  int64_t batchedQueries;    /* queries in them (mean batch = this / batches) */
  int64_t memoryWaits;       /* admissions deferred or shrunk for memory      */
  int64_t bytesInUse;        /* device bytes held by batches and results      */
  int64_t peakBytesInUse;
  int64_t pending;           /* queries submitted and not yet in a batch      */
  int64_t running;           /* batches in flight                              */
  int64_t kernelLaunches;    /* kernels the scheduler has launched             */
} gas_server_stats;

/* cfg may be NULL (defaults).  Starts the scheduler thread. */
GAS_API gas_status gas_server_create(int32_t device, const gas_server_config *cfg,
                                     gas_server **out);
/* Stops the scheduler after the batches in flight; queries not yet started
 * and results not yet fetched are dropped. */
GAS_API gas_status gas_server_destroy(gas_server *s);
/* Uploads a graph (edge list as gas_engine_set_graph; int32 weights, may be
 * NULL, are the SSSP edge lengths) and keeps it resident; GAS_ERR_OOM when
 * it does not fit in free device memory minus reserveBytes. */
GAS_API gas_status gas_server_add_graph(gas_server *s, int32_t nVertices, int32_t nEdges,
                                        const int32_t *srcs, const int32_t *dsts,
                                        const int32_t *weights, int32_t *graphId);
/* Non-blocking.  program = GAS_PROGRAM_BFS, _SSSP (graph with weights) or
 * _PPR. */
GAS_API gas_status gas_server_submit(gas_server *s, int32_t graphId, int32_t program,
                                     int32_t source, uint64_t *ticket);
/* Waits up to timeoutMs (< 0: no limit) for the query; GAS_ERR_TIMEOUT if
 * it is still running (wait again later).  On completion copies its
 * nVertices results into `result` (host memory of resultBytes, may be
 * NULL), fills `info` (may be NULL), releases the query and returns the
 * query's own status. */
GAS_API gas_status gas_server_wait(gas_server *s, uint64_t ticket, int32_t timeoutMs,
                                   void *result, int64_t resultBytes, gas_query_info *info);
/* *done = 1 when the query has completed (successfully or not). */
GAS_API gas_status gas_server_poll(gas_server *s, uint64_t ticket, int32_t *done);
GAS_API gas_status gas_server_get_stats(gas_server *s, gas_server_stats *st);

/* ---------------- status / diagnostics ---------------------------------- */
GAS_API const char *gas_status_string(gas_status s);
GAS_API const char *gas_last_error(void);
/* 1 when a CUDA device with compute capability 10.3 is present. */
GAS_API int32_t gas_device_supported(int32_t device);
/* Failure path of a stalled round, without a fault (no reference
 * counterpart; the reference's waits are host-side): the grid barrier of
 * the persistent kernels and the look-back wait of the gather tiles each
 * wait on a partner that never arrives, give up at their spin limits
 * (seconds), and report GAS_ERR_TIMEOUT in *barrierStatus /
 * *lookbackStatus; the device stays usable.  *seconds (may be NULL)
 * receives the wall time of both. */
GAS_API gas_status gas_selftest_bounded_waits(int32_t device, gas_status *barrierStatus,
                                              gas_status *lookbackStatus, float *seconds);

/* ---------------- synthetic graph generators (host) --------------------- */
/* Edge lists are allocated by the library; release with gas_edge_list_free.
 * weights is NULL unless requested. Output is sorted by (src, dst). */
typedef struct {
  int32_t nVertices;
  int64_t nEdges;
  int32_t *srcs;
  int32_t *dsts;
  int32_t *weights;
} gas_edge_list;

/* R-MAT (Chakrabarti et al. 2004): 2^scale vertices, edgeFactor*2^scale
 * samples with quadrant probabilities a, b, c (d = 1-a-b-c), drawn from a
 * counter-based SplitMix64 stream keyed by `seed`; no vertex permutation.
 * Self-loops and duplicates are removed; symmetrize != 0 adds every
 * reverse edge.  When wHi >= wLo >= 1, integer weights uniform in
 * [wLo, wHi] are attached, equal in both directions of an edge. */
GAS_API gas_status gas_gen_rmat(int32_t scale, int32_t edgeFactor, double a, double b, double c,
                                uint64_t seed, int32_t symmetrize, int32_t wLo, int32_t wHi,
                                gas_edge_list *out);

/* rows x cols 4-neighbour lattice; each undirected edge deleted with
 * probability pDelete; the largest connected component is kept and
 * relabelled row-major to 0..V'-1; symmetric; weights as for R-MAT. */
GAS_API gas_status gas_gen_grid(int32_t rows, int32_t cols, double pDelete, uint64_t seed,
                                int32_t wLo, int32_t wHi, gas_edge_list *out);

GAS_API void gas_edge_list_free(gas_edge_list *l);

/* ---------------- graph files (graphio.cpp) ----------------------------- */
/* Replaces loadGraph (graphio.cpp:441-473): the format from the extension
 * (".edge" SNAP, ".mtx" MatrixMarket coordinate, ".gr" Lonestar binary CSR;
 * text formats may be gzip-compressed, ".gz", when the library was built
 * with zlib), the same edge list as the reference loaders: self-loops
 * dropped, symmetric/skew-symmetric/hermitian MatrixMarket files expanded
 * to both directions, ids 0-based, vertex count = largest id + 1.  With
 * wantValues, weights receives the edge values (MatrixMarket values
 * truncated to int; skew-symmetric reverse edges negated; NULL for
 * "pattern" files).  Errors return a status instead of exiting; hermitian
 * files with values are refused (the reference loads their values
 * misaligned); a .gr file without values loads when no values are asked
 * for (the reference's own writer produces those).  Release with
 * gas_edge_list_free. */
GAS_API gas_status gas_load_graph(const char *path, int32_t wantValues, gas_edge_list *out);
/* Replaces writeGraph_mtx (graphio.cpp:416-438): "%%MatrixMarket matrix
 * coordinate Integer general", 1-based ids; values may be NULL. */
GAS_API gas_status gas_write_graph_mtx(const char *path, int32_t nVertices, int64_t nEdges,
                                       const int32_t *srcs, const int32_t *dsts,
                                       const int32_t *values);
/* Replaces writeGraph_binaryCSR (graphio.cpp:365-413): CSR offsets
 * (nVertices + 1) and destinations; values may be NULL. */
GAS_API gas_status gas_write_graph_gr(const char *path, int32_t nVertices, int64_t nEdges,
                                      const int32_t *offsets, const int32_t *dsts,
                                      const int32_t *values);
/* The drivers' result files (bfs.cu:115-119, sssp.cu:85-89,
 * pagerank.cu:77-81): one "vid value" line per vertex, "%d %d" for int32
 * values or "%d %f" for float; element i at values + i * strideBytes
 * (0 = 4, e.g. 8 for PageRank's {rank, numOutEdges}). */
GAS_API gas_status gas_write_vertex_values(const char *path, int32_t nVertices,
                                           const void *values, int32_t isFloat,
                                           int32_t strideBytes);

#ifdef __cplusplus
}
#endif
#endif
