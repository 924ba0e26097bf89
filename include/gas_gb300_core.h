/*
 * gas_gb300_core.h -- core layer of the GB300 GAS engine's C ABI.
 *
 * The Program-independent half of the engine (the parts of gpugas.h that do
 * not call user code): device CSC/CSR construction (setGraph,
 * gpugas.h:212-322), the active frontier (setActive / countActive,
 * gpugas.h:342-356), scatter-activate and frontier rebuild
 * (gpugas.h:669-751) and the iteration loop (gpugas.h:754-772).
 *
 * The Program-dependent gather+apply kernel is compiled in the caller's
 * translation unit (gas_gb300/gpugas.cuh) and launched through the
 * callback given to gas_core_gather_apply / gas_core_run; its arguments are
 * the plain struct gas_gather_args below.
 */
#ifndef GAS_GB300_CORE_H
#define GAS_GB300_CORE_H

#include "gas_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Tile geometry shared by the core and header-instantiated kernels:
 * a gather tile covers GAS_GATHER_TILE merged items (active vertices plus
 * their in-edges), a scatter tile GAS_SCATTER_TILE items. */
#define GAS_GATHER_THREADS 256
#define GAS_GATHER_ITEMS 8
#define GAS_GATHER_TILE (GAS_GATHER_THREADS * GAS_GATHER_ITEMS)
#define GAS_SCATTER_THREADS 256
#define GAS_SCATTER_ITEMS 8
#define GAS_SCATTER_TILE (GAS_SCATTER_THREADS * GAS_SCATTER_ITEMS)

/* Device error bits (gas_gather_args.errWord). */
#define GAS_DEVERR_TIMEOUT 1u    /* bounded look-back wait gave up */
#define GAS_DEVERR_CAPACITY 2u   /* a queue would have overflowed  */

/* Low-degree mode: when every vertex of a list has degree <= this bound,
 * its phase runs one thread per vertex (edges folded left to right in CSC
 * order) instead of merge-path tiles. */
#define GAS_TPV_MAX_DEGREE 8
#define GAS_TPV_TILE GAS_GATHER_THREADS

/* Bytes of one vertex's cell in fused rounds: two value slots and a version
 * word, rounded up to 16 (one aligned vector load reads a whole cell). */
#define GAS_FUSED_CELL_BYTES(vertexBytes) ((((vertexBytes) * 2 + 4) + 15) / 16 * 16)

/* A vertex list on the device: ids, exclusive prefix of the degree that the
 * consumer walks (in-degree for the gather, out-degree for the scatter),
 * CSC/CSR begin offset of each vertex, merge-path tile splits, and a
 * control word pair (count << 32 | degree total, maximum degree). */
typedef struct {
  int32_t *vid;
  int32_t *pre;
  int32_t *beg;
  int32_t *split;
  unsigned long long *count;
  unsigned int *maxDeg;
} gas_vertex_list;

/* Arguments of one gather+apply launch (device pointers). */
typedef struct {
  /* graph: CSC for gather, CSR offsets for out-degrees */
  int32_t nVertices;
  int32_t nEdges;
  const int32_t *inOffsets;   /* [nVertices+1] */
  const int32_t *inSources;   /* [nEdges]      */
  const int32_t *outOffsets;  /* [nVertices+1] */
  const void *edgeData;       /* CSC order, NULL when EdgeData is empty */
  /* vertex data: gather reads vertexData; apply writes vertexNew[i] for
   * frontier position i (committed by scatter), or vertexData in place
   * when haveGather == 0 */
  void *vertexData;
  void *vertexNew;
  /* current frontier: range [rangeStart, rangeStart+n) or a list */
  int32_t rangeMode;
  int32_t rangeStart;
  int32_t rangeCount;
  int32_t rangeBase;          /* inOffsets[rangeStart]                      */
  int32_t rangeMaxDeg;        /* largest in-degree in the range (bound)     */
  const int32_t *rangeSplit;  /* gather-tile splits of the range            */
  gas_vertex_list front;      /* list mode                                  */
  /* scatter list appended by this launch (out-degree prefix) */
  gas_vertex_list scat;
  int32_t capacity;           /* capacity of every vertex list              */
  int32_t maxScatTiles;
  /* list this launch resets for the following scatter (list mode) */
  unsigned long long *resetCount;
  unsigned int *resetMaxDeg;
  unsigned int *resetTile;
  /* dynamic tile counter of this launch */
  unsigned int *tileCounter;
  /* cross-tile partial reductions (look-back) */
  void *carryVal;
  unsigned int *carryFlag;
  unsigned int epoch;
  /* misc */
  unsigned int *errWord;
  unsigned long long *statSlot; /* round statistics slot (may be NULL) */
  int32_t iteration;
  int32_t haveGather;
} gas_gather_args;

/* Arguments of one persistent run() launch: every round of gather/apply,
 * commit + scatter/activate and frontier swap in a single cooperative
 * kernel, the phases separated by bounded grid barriers. */
typedef struct {
  gas_gather_args g;          /* graph, vertex data, carry arrays, ...      */
  const int32_t *outDests;    /* CSR destinations [nEdges]                  */
  int32_t vertexBytes;
  int32_t maxGatherTiles;
  gas_vertex_list frontL[2];  /* frontier lists (in-degree prefix)          */
  gas_vertex_list scatL[2];   /* scatter lists (out-degree prefix)          */
  int32_t *mark;
  unsigned long long *stats;  /* 2 words per round, maxStatRounds rounds    */
  int32_t maxStatRounds;
  int32_t cur;                /* frontier buffer of round 0 (list mode)     */
  int32_t sidx;               /* scatter list of round 0                    */
  int32_t maxRounds;          /* 0 = until no vertex is active              */
  unsigned epochBase;         /* carry-flag epoch of round 0                */
  int32_t stampBase;          /* activation stamp of round 0                */
  unsigned *barrier;          /* [2]: [0] the grid barrier's arrival word (zero
                                 at launch), [1] unused                       */
  int32_t *roundsOut;         /* rounds executed                            */
  /* dense (pull) rounds */
  void *vertexAlt;            /* second vertex-data buffer (ping-pong)      */
  uint32_t *retBits[3];       /* frontier bitmaps, bitWords words each: bit v set when
                                 v's apply returned true; the round of stamp S sets
                                 bits in [S % 3], reads [(S-1) % 3] and clears
                                 [(S+1) % 3]; [stampBase % 3] is clear at launch */
  int32_t bitWords;           /* ceil(V / 32)                                */
  uint32_t *frontBits[3];     /* active-set bitmaps of the fused rounds (null when
                                 the graph has none), bitWords words each: the
                                 round of stamp S reads [S % 3] (when its frontier
                                 is a bitmap), sets the bits of the vertices it
                                 activates in [(S+1) % 3] and clears [(S+2) % 3];
                                 [(stampBase+1) % 3] is clear at launch */
  unsigned long long *denseCnt; /* [3][4] per-round counters: active/in-edges,
                                 ret/out-edges, dense work units taken, unused */
  int32_t denseAlpha;         /* next round dense when out-edges*alpha > E; 0 = never */
  int32_t allActive;          /* round 0 is every vertex (setActive(0, V)) */
  int32_t *vcurOut;           /* 1 when the final vertex data is in vertexAlt */
  /* degree bins of the dense pass (fixed per graph): warp work units are
   * [large-vertex chunks | warp-per-vertex | 8-lane groups | thread-per-vertex] */
  const int32_t *binMid;      /* in-degree 65..1024: one warp each          */
  const int32_t *binSmall;    /* in-degree 9..64: 8 lanes each              */
  const int32_t *binTiny;     /* in-degree 0..8: one thread each            */
  int32_t nMid, nSmall, nTiny;
  const int32_t *chunkVertex; /* in-degree > 1024: 1024-edge chunks          */
  const int32_t *chunkBegin;  /* first CSC position of each chunk            */
  const int32_t *chunkFirst;  /* index of the vertex's first chunk, per chunk */
  const int32_t *chunkCount;  /* chunks of the vertex, per chunk             */
  const int32_t *chunkSlot;   /* arrival-counter slot of the vertex, per chunk */
  int32_t nChunks;
  int32_t nChunkVertices;
  unsigned *chunkArrive;      /* [2][nChunkVertices] arrival counters        */
  void *chunkVal;             /* [nChunks] GatherResult partials             */
  unsigned *chunkFlags;       /* [nChunks] has | act << 1                    */
  /* Program::scatter over the out-edges of each round's ret vertices
   * (gas_core_enable_edge_scatter); dense rounds are off then */
  int32_t edgeScatter;
  const int32_t *csr2csc;     /* [E] CSC position of the edge at each CSR position */
  /* fused list rounds (every degree <= 8): gather, apply and activation in
   * one phase, vertex data versioned across the two buffers */
  int32_t fused;
  /* fixed-width adjacency rows of fused graphs (every degree <= 8): row v of
   * ellWidth entries (4 or 8) holds v's in-neighbours (ellIn, CSC order, -1
   * after the last), their edge data (ellEd, edgeBytes each) and v's
   * out-neighbours (ellOut, -1 after the last) */
  const int32_t *ellIn;
  const int32_t *ellOut;
  const void *ellEd;
  int32_t ellWidth;
  void *fusedCells;           /* [V] cells of GAS_FUSED_CELL_BYTES(vertexBytes) each:
                                 two value slots and (stamp << 1) | newest slot */
  /* the run starts with dense rounds (allActive): the caller may run them in
   * a leaner kernel first, which leaves the state the main kernel resumes
   * from in resume[4] = rounds done, vcur, dense -> list transition pending,
   * run ended; denseFirst tells the main kernel to resume */
  int32_t denseFirst;
  int32_t *resume;
  /* set to 1 when the run stopped at maxRounds before a dense round: the
   * next frontier is then the vertices whose bits its last round set
   * (retBits) instead of a list */
  int32_t *denseEndOut;
} gas_run_args;

/* The vertices whose apply returned true in the round just scattered, for
 * a Program's scatter over their out-edges (edge data in CSC order). */
typedef struct {
  const int32_t *vid;                 /* [count] vertex ids                   */
  const unsigned long long *count;    /* device: count << 32 | out-degree sum */
  const int32_t *outOffsets;          /* CSR                                  */
  const int32_t *outDests;
  const int32_t *csr2csc;             /* [E] CSC position of each CSR edge    */
  void *vertexData;
  void *edgeData;                     /* CSC order                            */
} gas_edge_scatter_args;

typedef struct gas_core_s gas_core;

/* Launches the caller's gather+apply kernel for `args` on `stream`. */
typedef gas_status (*gas_gather_launch_fn)(void *user, const gas_gather_args *args,
                                           void *stream);
/* Launches the caller's persistent run kernel (cooperative launch).
 * Returns GAS_ERR_UNSUPPORTED when it cannot be launched co-resident; the
 * core then falls back to one launch per phase. */
typedef gas_status (*gas_run_launch_fn)(void *user, const gas_run_args *args, void *stream);
/* Launches the caller's Program::scatter kernel. */
typedef gas_status (*gas_edge_scatter_fn)(void *user, const gas_edge_scatter_args *args,
                                          void *stream);

GAS_API gas_status gas_core_create(int32_t device, void *stream, gas_core **out);
GAS_API gas_status gas_core_destroy(gas_core *c);
GAS_API gas_status gas_core_stream(gas_core *c, void **stream);

/* setGraph: builds CSC+CSR on the device, sorts edge data (edgeBytes per
 * edge, may be 0) into CSC order and allocates per-vertex state for the
 * given VertexData / GatherResult sizes. */
GAS_API gas_status gas_core_set_graph(gas_core *c, int32_t nVertices, int32_t nEdges,
                                      const int32_t *srcs, const int32_t *dsts,
                                      const void *edgeData, int32_t edgeBytes,
                                      int32_t vertexBytes, int32_t gatherBytes);

GAS_API gas_status gas_core_upload_vertex_data(gas_core *c, const void *host);
GAS_API gas_status gas_core_download_vertex_data(gas_core *c, void *host);
/* Edge data in the caller's original edge-list order. */
GAS_API gas_status gas_core_download_edge_data(gas_core *c, void *host);
/* Device pointer of the vertex data array. */
GAS_API gas_status gas_core_vertex_data(gas_core *c, void **dev);

GAS_API gas_status gas_core_set_active(gas_core *c, int32_t start, int32_t end);
GAS_API gas_status gas_core_count_active(gas_core *c, int32_t *n);
GAS_API gas_status gas_core_set_iteration(gas_core *c, int32_t iteration);

/* One gatherApply: fills gas_gather_args and calls `launch`. */
GAS_API gas_status gas_core_gather_apply(gas_core *c, int32_t haveGather,
                                         gas_gather_launch_fn launch, void *user);
/* One scatterActivate (commits apply's vertex data, expands out-edges of
 * vertices whose apply returned true, builds the next frontier). */
GAS_API gas_status gas_core_scatter_activate(gas_core *c);
GAS_API gas_status gas_core_next_iter(gas_core *c);

/* run(): rounds of gatherApply/scatterActivate/nextIter until no vertex is
 * active (or maxIters rounds when maxIters > 0), without a host round trip
 * per round. */
GAS_API gas_status gas_core_run(gas_core *c, int32_t maxIters, int32_t haveGather,
                                gas_gather_launch_fn launch, void *user,
                                int32_t *iterations);

/* run() as one persistent cooperative launch (runLaunch); falls back to
 * gas_core_run's per-phase launches when runLaunch is NULL or reports
 * GAS_ERR_UNSUPPORTED. */
GAS_API gas_status gas_core_run_persistent(gas_core *c, int32_t maxIters, int32_t haveGather,
                                           gas_run_launch_fn runLaunch,
                                           gas_gather_launch_fn launch, void *user,
                                           int32_t *iterations);

GAS_API gas_status gas_core_round_stats(gas_core *c, int32_t capacity, int64_t *active,
                                        int64_t *gathered, int64_t *ret,
                                        int64_t *scattered, int32_t *rounds);
GAS_API gas_status gas_core_last_run_ms(gas_core *c, float *ms);
GAS_API gas_status gas_core_save_vertex_data(gas_core *c);
GAS_API gas_status gas_core_restore_vertex_data(gas_core *c);
GAS_API gas_status gas_core_set_profiling(gas_core *c, int32_t enabled);
/* run(): a round runs dense (pull over every vertex) when the previous
 * round's apply-returned-true vertices have more than nEdges/alpha
 * out-edges; 0 disables dense rounds.  Results do not depend on it. */
GAS_API gas_status gas_core_set_dense_policy(gas_core *c, int32_t alpha);
/* run(): on graphs whose in- and out-degrees are all <= 8, list rounds run
 * as one phase (gather, apply and activation together, one grid barrier)
 * with versioned vertex data; 0 keeps the two-phase rounds.  Default on.
 * Results, round counts and per-round counts do not depend on it. */
GAS_API gas_status gas_core_set_fused_rounds(gas_core *c, int32_t on);
GAS_API gas_status gas_core_kernel_times(gas_core *c, float *gatherMs, float *scatterMs,
                                         int32_t *gatherLaunches, int32_t *scatterLaunches);
/* Waits for queued work and reports device-side errors. */
GAS_API gas_status gas_core_sync(gas_core *c);

/* Program::scatter(src, dst, edge) for every out-edge of the vertices whose
 * apply returned true, after their activation, as the reference's CPU
 * engine does (refgas.h:171-197); its GPU engine never calls it
 * (gpugas.h:666-668).  Enable before gas_core_set_graph (the graph then
 * keeps the CSR -> CSC edge map; getResults returns the edge data in the
 * caller's order).  run() then uses list rounds only. */
GAS_API gas_status gas_core_enable_edge_scatter(gas_core *c, int32_t on);
/* After gas_core_scatter_activate and before gas_core_next_iter: hands
 * the round's vertices to the caller's scatter kernel. */
GAS_API gas_status gas_core_edge_scatter(gas_core *c, gas_edge_scatter_fn launch, void *user);

#ifdef __cplusplus
}
#endif
#endif
