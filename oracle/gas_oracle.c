/*
 * TEST INFRASTRUCTURE ONLY -- the oracle (see gas_oracle.h for what it
 * restates and how it is pinned).  Only tests/, __graft_entry__.smoke() and
 * the CPU-baseline leg of bench.py load this code.
 */
#define _POSIX_C_SOURCE 199309L
#include "gas_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ---------------------------------------------------------------------- */
/* util.h:79-110 edgeListToCSR.  offsets[v] = first sorted position whose
 * key is >= v; trailing offsets = nE.  Ties keep edge-list order. */
void ora_edge_list_to_csr(int32_t nV, int32_t nE, const int32_t *srcs,
                          const int32_t *dsts, int32_t *offsets,
                          int32_t *out_dsts, int32_t *sort_idx)
{
  memset(offsets, 0, sizeof(int32_t) * ((size_t)nV + 1));
  for (int32_t i = 0; i < nE; ++i) offsets[srcs[i] + 1]++;
  for (int32_t v = 0; v < nV; ++v) offsets[v + 1] += offsets[v];
  int32_t *cur = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nV + 1));
  memcpy(cur, offsets, sizeof(int32_t) * ((size_t)nV + 1));
  for (int32_t i = 0; i < nE; ++i) {
    int32_t p = cur[srcs[i]]++;
    if (sort_idx) sort_idx[p] = i;
    if (out_dsts) out_dsts[p] = dsts[i];
  }
  free(cur);
}

/* bfs.cu:148-166 */
int32_t ora_max_outdegree_vertex(int32_t nV, int32_t nE, const int32_t *srcs)
{
  int32_t *deg = (int32_t *)calloc((size_t)nV + 1, sizeof(int32_t));
  for (int32_t i = 0; i < nE; ++i) deg[srcs[i]]++;
  int32_t best = -1, maxDegree = -1;
  for (int32_t v = 0; v < nV; ++v)
    if (deg[v] > maxDegree) { maxDegree = deg[v]; best = v; }
  free(deg);
  return best;
}

/* ---------------------------------------------------------------------- */
/* Program-independent half of GASEngineRef (refgas.h:31-225). */
typedef struct {
  int32_t nV, nE;
  int32_t *srcOffsets, *srcs, *edgeIndexCSC; /* CSC for gather  (refgas.h:44-47) */
  int32_t *dstOffsets, *dsts, *edgeIndexCSR; /* CSR for scatter (refgas.h:49-52) */
  int32_t *active;                           /* refgas.h:56 */
  int32_t nActive;
  int32_t *applyRet;                         /* refgas.h:57 */
  uint64_t *activeFlags;                     /* refgas.h:58, bit-packed like vector<bool> */
  double param;                              /* program constant (PPR damping) */
} ora_engine;

static int ora_check_edges(int32_t nV, int32_t nE, const int32_t *srcs,
                           const int32_t *dsts)
{
  if (nV < 0 || nE < 0) return 1;
  if (nE > 0 && (!srcs || !dsts)) return 1;
  for (int32_t i = 0; i < nE; ++i)
    if (srcs[i] < 0 || srcs[i] >= nV || dsts[i] < 0 || dsts[i] >= nV) return 1;
  return 0;
}

/* refgas.h:81-113 setGraph */
static void ora_engine_init(ora_engine *e, int32_t nV, int32_t nE,
                            const int32_t *srcs, const int32_t *dsts)
{
  size_t v1 = (size_t)nV + 1, ne = (size_t)(nE > 0 ? nE : 1);
  e->nV = nV;
  e->nE = nE;
  e->dstOffsets = (int32_t *)malloc(sizeof(int32_t) * v1);
  e->dsts = (int32_t *)malloc(sizeof(int32_t) * ne);
  e->edgeIndexCSR = (int32_t *)malloc(sizeof(int32_t) * ne);
  ora_edge_list_to_csr(nV, nE, srcs, dsts, e->dstOffsets, e->dsts, e->edgeIndexCSR);
  /* util.h:114-121: CSC is CSR of the reversed edge list */
  e->srcOffsets = (int32_t *)malloc(sizeof(int32_t) * v1);
  e->srcs = (int32_t *)malloc(sizeof(int32_t) * ne);
  e->edgeIndexCSC = (int32_t *)malloc(sizeof(int32_t) * ne);
  ora_edge_list_to_csr(nV, nE, dsts, srcs, e->srcOffsets, e->srcs, e->edgeIndexCSC);
  e->active = (int32_t *)malloc(sizeof(int32_t) * v1);
  e->nActive = 0;
  e->applyRet = (int32_t *)malloc(sizeof(int32_t) * v1);
  e->activeFlags = (uint64_t *)calloc((size_t)nV / 64 + 1, sizeof(uint64_t));
  e->param = 0.0;
}

static void ora_engine_free(ora_engine *e)
{
  free(e->dstOffsets); free(e->dsts); free(e->edgeIndexCSR);
  free(e->srcOffsets); free(e->srcs); free(e->edgeIndexCSC);
  free(e->active); free(e->applyRet); free(e->activeFlags);
}

/* refgas.h:128-134 setActive */
static void ora_set_active(ora_engine *e, int32_t start, int32_t end)
{
  e->nActive = 0;
  for (int32_t i = start; i < end; ++i) e->active[e->nActive++] = i;
}

/* refgas.h:171-197 scatterActivate.  Program::scatter is empty in every
 * example program (bfs.cu:72-76, sssp.cu:58-62, pagerank.cu:66-70,
 * connected_component.cu:57-61) and is not called here. */
static void ora_scatter_activate(ora_engine *e)
{
  memset(e->activeFlags, 0, sizeof(uint64_t) * ((size_t)e->nV / 64 + 1));
  for (int32_t i = 0; i < e->nActive; ++i) {
    if (e->applyRet[i]) {
      int32_t sv = e->active[i];
      for (int32_t ie = e->dstOffsets[sv]; ie < e->dstOffsets[sv + 1]; ++ie) {
        int32_t dv = e->dsts[ie];
        e->activeFlags[dv >> 6] |= (uint64_t)1 << (dv & 63);
      }
    }
  }
}

/* refgas.h:201-210 nextIter: ascending list of flagged vertices */
static void ora_next_iter(ora_engine *e)
{
  e->nActive = 0;
  for (int32_t i = 0; i < e->nV; ++i)
    if ((e->activeFlags[i >> 6] >> (i & 63)) & 1) e->active[e->nActive++] = i;
}

static void ora_record_pre(ora_engine *e, ora_stats *st, int32_t it)
{
  int64_t eg = 0;
  for (int32_t i = 0; i < e->nActive; ++i) {
    int32_t v = e->active[i];
    eg += e->srcOffsets[v + 1] - e->srcOffsets[v];
  }
  st->active[it] = e->nActive;
  st->edges_gathered[it] = eg;
}

static void ora_record_post(ora_engine *e, ora_stats *st, int32_t it)
{
  int64_t r = 0, es = 0;
  for (int32_t i = 0; i < e->nActive; ++i) {
    if (e->applyRet[i]) {
      int32_t v = e->active[i];
      ++r;
      es += e->dstOffsets[v + 1] - e->dstOffsets[v];
    }
  }
  st->ret[it] = r;
  st->edges_scattered[it] = es;
}

/* ---------------------------------------------------------------------- */
/* BFS, bfs.cu:31-78.  The driver's g_iterationCount (bfs.cu:27,81-88) is
 * the iteration index handed to apply. */
typedef struct { int32_t depth; } bfs_vd;
typedef struct { char unused; } empty_ed;
static inline int bfs_apply(bfs_vd *v, int32_t g, int32_t iter)
{
  (void)g;
  if (v->depth == -1) { v->depth = iter; return 1; }
  return 0;
}
#define ORA_FN(x) bfs_##x
#define ORA_VD bfs_vd
#define ORA_ED empty_ed
#define ORA_GR int32_t
#define ORA_GZERO (INT_MAX - 1)
#define ORA_GATHER_MAP(d, s, e) ((void)(d), (void)(s), (void)(e), 0)
#define ORA_GATHER_REDUCE(a, b) ((void)(a), (void)(b), 0)
#define ORA_APPLY(v, g, it, e) ((void)(e), bfs_apply(v, g, it))
#define ORA_HAS_ED 0
#include "gas_oracle_engine.inc"
#undef ORA_FN
#undef ORA_VD
#undef ORA_ED
#undef ORA_GR
#undef ORA_GZERO
#undef ORA_GATHER_MAP
#undef ORA_GATHER_REDUCE
#undef ORA_APPLY
#undef ORA_HAS_ED

/* SSSP, sssp.cu:25-64.  gatherZero = INT_MAX - 100000 is also the initial
 * and "unreached" distance (sssp.cu:32-33, 141-144). */
#define SSSP_GZERO (INT_MAX - 100000)
static inline int32_t imin32(int32_t a, int32_t b) { return a < b ? a : b; }
static inline int sssp_apply(int32_t *cur, int32_t d)
{
  int changed = d < *cur;
  *cur = imin32(*cur, d);
  return changed;
}
#define ORA_FN(x) sssp_##x
#define ORA_VD int32_t
#define ORA_ED int32_t
#define ORA_GR int32_t
#define ORA_GZERO SSSP_GZERO
#define ORA_GATHER_MAP(d, s, e) ((void)(d), *(s) + *(e))
#define ORA_GATHER_REDUCE(a, b) imin32(a, b)
#define ORA_APPLY(v, g, it, e) ((void)(it), (void)(e), sssp_apply(v, g))
#define ORA_HAS_ED 1
#include "gas_oracle_engine.inc"
#undef ORA_FN
#undef ORA_VD
#undef ORA_ED
#undef ORA_GR
#undef ORA_GZERO
#undef ORA_GATHER_MAP
#undef ORA_GATHER_REDUCE
#undef ORA_APPLY
#undef ORA_HAS_ED

/* SSSP whose scatter writes its edge (not a reference program): a visit
 * count and the source's distance at the visit -- exercises the engine's
 * call of Program::scatter (refgas.h:171-197). */
typedef struct { int32_t w, visits, last; } visit_ed;
#define ORA_FN(x) sssp_visits_##x
#define ORA_VD int32_t
#define ORA_ED visit_ed
#define ORA_GR int32_t
#define ORA_GZERO SSSP_GZERO
#define ORA_GATHER_MAP(d, s, e) ((void)(d), *(s) + (e)->w)
#define ORA_GATHER_REDUCE(a, b) imin32(a, b)
#define ORA_APPLY(v, g, it, e) ((void)(it), (void)(e), sssp_apply(v, g))
#define ORA_HAS_ED 1
#define ORA_SCATTER(s, d, e) ((void)(d), (e)->visits += 1, (e)->last = *(s))
#include "gas_oracle_engine.inc"
#undef ORA_FN
#undef ORA_VD
#undef ORA_ED
#undef ORA_GR
#undef ORA_GZERO
#undef ORA_GATHER_MAP
#undef ORA_GATHER_REDUCE
#undef ORA_APPLY
#undef ORA_HAS_ED
#undef ORA_SCATTER

/* Connected components, connected_component.cu:25-63 */
#define ORA_FN(x) cc_##x
#define ORA_VD int32_t
#define ORA_ED empty_ed
#define ORA_GR int32_t
#define ORA_GZERO INT_MAX
#define ORA_GATHER_MAP(d, s, e) ((void)(d), (void)(e), *(s))
#define ORA_GATHER_REDUCE(a, b) imin32(a, b)
#define ORA_APPLY(v, g, it, e) ((void)(it), (void)(e), sssp_apply(v, g))
#define ORA_HAS_ED 0
#include "gas_oracle_engine.inc"
#undef ORA_FN
#undef ORA_VD
#undef ORA_ED
#undef ORA_GR
#undef ORA_GZERO
#undef ORA_GATHER_MAP
#undef ORA_GATHER_REDUCE
#undef ORA_APPLY
#undef ORA_HAS_ED

/* PageRank, pagerank.cu:27-73: pageConst 0.15f, tol 0.01f, unnormalised.
 * The FP64 twin is the same program with double rank and GatherResult and
 * the same constant values (the float constants widened exactly). */
typedef struct { float rank; int32_t numOutEdges; } pr32_vd;
typedef struct { double rank; int32_t numOutEdges; } pr64_vd;
static const float PR_PAGE_CONST = 0.15f;
static const float PR_TOL = 0.01f;
static inline int pr32_apply(pr32_vd *v, float g)
{
  float newRank = PR_PAGE_CONST + (1.0f - PR_PAGE_CONST) * g;
  int ret = fabsf(newRank - v->rank) >= PR_TOL;
  v->rank = newRank;
  return ret;
}
static inline int pr64_apply(pr64_vd *v, double g)
{
  double pc = (double)PR_PAGE_CONST;
  double newRank = pc + (1.0 - pc) * g;
  int ret = fabs(newRank - v->rank) >= (double)PR_TOL;
  v->rank = newRank;
  return ret;
}
#define ORA_FN(x) pr32_##x
#define ORA_VD pr32_vd
#define ORA_ED empty_ed
#define ORA_GR float
#define ORA_GZERO 0.0f
#define ORA_GATHER_MAP(d, s, e) ((void)(d), (void)(e), (s)->rank / (float)(s)->numOutEdges)
#define ORA_GATHER_REDUCE(a, b) ((a) + (b))
#define ORA_APPLY(v, g, it, e) ((void)(it), (void)(e), pr32_apply(v, g))
#define ORA_HAS_ED 0
#include "gas_oracle_engine.inc"
#undef ORA_FN
#undef ORA_VD
#undef ORA_GR
#undef ORA_GZERO
#undef ORA_GATHER_MAP
#undef ORA_APPLY
#define ORA_FN(x) pr64_##x
#define ORA_VD pr64_vd
#define ORA_GR double
#define ORA_GZERO 0.0
#define ORA_GATHER_MAP(d, s, e) ((void)(d), (void)(e), (s)->rank / (double)(s)->numOutEdges)
#define ORA_APPLY(v, g, it, e) ((void)(it), (void)(e), pr64_apply(v, g))
#include "gas_oracle_engine.inc"
#undef ORA_FN
#undef ORA_VD
#undef ORA_GR
#undef ORA_GZERO
#undef ORA_GATHER_MAP
#undef ORA_APPLY

/* Personalised PageRank (new program, same contract).  teleport holds
 * alpha for the source vertex and 0 elsewhere; every vertex stays active. */
typedef struct { float rank; int32_t numOutEdges; float teleport; } ppr32_vd;
typedef struct { double rank; int32_t numOutEdges; double teleport; } ppr64_vd;
static inline int ppr32_apply(ppr32_vd *v, float g, float damp)
{
  v->rank = v->teleport + damp * g;
  return 1;
}
static inline int ppr64_apply(ppr64_vd *v, double g, double damp)
{
  v->rank = v->teleport + damp * g;
  return 1;
}
#define ORA_FN(x) ppr32_##x
#define ORA_VD ppr32_vd
#define ORA_GR float
#define ORA_GZERO 0.0f
#define ORA_GATHER_MAP(d, s, e) ((void)(d), (void)(e), (s)->rank / (float)(s)->numOutEdges)
#define ORA_APPLY(v, g, it, e) ((void)(it), ppr32_apply(v, g, (float)(e)->param))
#include "gas_oracle_engine.inc"
#undef ORA_FN
#undef ORA_VD
#undef ORA_GR
#undef ORA_GZERO
#undef ORA_GATHER_MAP
#undef ORA_APPLY
#define ORA_FN(x) ppr64_##x
#define ORA_VD ppr64_vd
#define ORA_GR double
#define ORA_GZERO 0.0
#define ORA_GATHER_MAP(d, s, e) ((void)(d), (void)(e), (s)->rank / (double)(s)->numOutEdges)
#define ORA_APPLY(v, g, it, e) ((void)(it), ppr64_apply(v, g, (e)->param))
#include "gas_oracle_engine.inc"
#undef ORA_FN
#undef ORA_VD
#undef ORA_ED
#undef ORA_GR
#undef ORA_GZERO
#undef ORA_GATHER_MAP
#undef ORA_GATHER_REDUCE
#undef ORA_APPLY
#undef ORA_HAS_ED

/* ---------------------------------------------------------------------- */
/* Drivers, mirroring the example programs' run<Engine>() functions. */

/* bfs.cu:91-112 (depth = -1 initially, bfs.cu:143-145) */
int ora_run_bfs(int32_t nV, int32_t nE, const int32_t *srcs,
                const int32_t *dsts, int32_t source, int32_t *depth,
                ora_stats *st)
{
  if (ora_check_edges(nV, nE, srcs, dsts) || !depth) return 1;
  if (source < 0 || source >= nV) return 1;
  bfs_vd *vd = (bfs_vd *)malloc(sizeof(bfs_vd) * ((size_t)nV + 1));
  for (int32_t i = 0; i < nV; ++i) vd[i].depth = -1;
  ora_engine e;
  ora_engine_init(&e, nV, nE, srcs, dsts);
  ora_set_active(&e, source, source + 1);
  bfs_run(&e, vd, 0, 0, st);
  for (int32_t i = 0; i < nV; ++i) depth[i] = vd[i].depth;
  ora_engine_free(&e);
  free(vd);
  return 0;
}

/* sssp.cu:67-82, vertex data as sssp.cu:139-144 */
int ora_run_sssp(int32_t nV, int32_t nE, const int32_t *srcs,
                 const int32_t *dsts, const int32_t *weights, int32_t source,
                 int32_t *dist, ora_stats *st)
{
  if (ora_check_edges(nV, nE, srcs, dsts) || !dist) return 1;
  if (source < 0 || source >= nV || (nE > 0 && !weights)) return 1;
  for (int32_t i = 0; i < nV; ++i) dist[i] = SSSP_GZERO;
  dist[source] = 0;
  ora_engine e;
  ora_engine_init(&e, nV, nE, srcs, dsts);
  ora_set_active(&e, 0, nV);
  sssp_run(&e, dist, weights, 0, st);
  ora_engine_free(&e);
  return 0;
}

/* The scatter-writing SSSP, driven as sssp.cu:67-82: edge data {w,
 * visits, last} in edge-list order (visits/last start at 0). */
int ora_run_sssp_visits(int32_t nV, int32_t nE, const int32_t *srcs,
                        const int32_t *dsts, const int32_t *weights, int32_t source,
                        int32_t *dist, int32_t *visits, int32_t *last, ora_stats *st)
{
  if (ora_check_edges(nV, nE, srcs, dsts) || !dist || !visits || !last) return 1;
  if (source < 0 || source >= nV || (nE > 0 && !weights)) return 1;
  for (int32_t i = 0; i < nV; ++i) dist[i] = SSSP_GZERO;
  dist[source] = 0;
  visit_ed *ed = (visit_ed *)calloc((size_t)(nE > 0 ? nE : 1), sizeof(visit_ed));
  for (int32_t i = 0; i < nE; ++i) ed[i].w = weights[i];
  ora_engine e;
  ora_engine_init(&e, nV, nE, srcs, dsts);
  ora_set_active(&e, 0, nV);
  sssp_visits_run(&e, dist, ed, 0, st);
  ora_engine_free(&e);
  for (int32_t i = 0; i < nE; ++i) {
    visits[i] = ed[i].visits;
    last[i] = ed[i].last;
  }
  free(ed);
  return 0;
}

/* connected_component.cu:66-81, labels as :110-114 */
int ora_run_cc(int32_t nV, int32_t nE, const int32_t *srcs,
               const int32_t *dsts, int32_t *label, ora_stats *st)
{
  if (ora_check_edges(nV, nE, srcs, dsts) || !label) return 1;
  for (int32_t i = 0; i < nV; ++i) label[i] = i;
  ora_engine e;
  ora_engine_init(&e, nV, nE, srcs, dsts);
  ora_set_active(&e, 0, nV);
  cc_run(&e, label, 0, 0, st);
  ora_engine_free(&e);
  return 0;
}

/* pagerank.cu:76-101 and :120-132 (numOutEdges from CSR offsets) */
int ora_run_pagerank_f32(int32_t nV, int32_t nE, const int32_t *srcs,
                         const int32_t *dsts, int32_t max_iters, float *rank,
                         ora_stats *st)
{
  if (ora_check_edges(nV, nE, srcs, dsts) || !rank) return 1;
  ora_engine e;
  ora_engine_init(&e, nV, nE, srcs, dsts);
  pr32_vd *vd = (pr32_vd *)malloc(sizeof(pr32_vd) * ((size_t)nV + 1));
  for (int32_t i = 0; i < nV; ++i) {
    vd[i].numOutEdges = e.dstOffsets[i + 1] - e.dstOffsets[i];
    vd[i].rank = PR_PAGE_CONST;
  }
  ora_set_active(&e, 0, nV);
  pr32_run(&e, vd, 0, max_iters, st);
  for (int32_t i = 0; i < nV; ++i) rank[i] = vd[i].rank;
  ora_engine_free(&e);
  free(vd);
  return 0;
}

int ora_run_pagerank_f64(int32_t nV, int32_t nE, const int32_t *srcs,
                         const int32_t *dsts, int32_t max_iters,
                         double *rank, ora_stats *st)
{
  if (ora_check_edges(nV, nE, srcs, dsts) || !rank) return 1;
  ora_engine e;
  ora_engine_init(&e, nV, nE, srcs, dsts);
  pr64_vd *vd = (pr64_vd *)malloc(sizeof(pr64_vd) * ((size_t)nV + 1));
  for (int32_t i = 0; i < nV; ++i) {
    vd[i].numOutEdges = e.dstOffsets[i + 1] - e.dstOffsets[i];
    vd[i].rank = (double)PR_PAGE_CONST;
  }
  ora_set_active(&e, 0, nV);
  pr64_run(&e, vd, 0, max_iters, st);
  for (int32_t i = 0; i < nV; ++i) rank[i] = vd[i].rank;
  ora_engine_free(&e);
  free(vd);
  return 0;
}

int ora_run_ppr_f32(int32_t nV, int32_t nE, const int32_t *srcs,
                    const int32_t *dsts, int32_t source, float alpha,
                    int32_t iters, float *rank, ora_stats *st)
{
  if (ora_check_edges(nV, nE, srcs, dsts) || !rank) return 1;
  if (source < 0 || source >= nV || iters < 0) return 1;
  ora_engine e;
  ora_engine_init(&e, nV, nE, srcs, dsts);
  ppr32_vd *vd = (ppr32_vd *)malloc(sizeof(ppr32_vd) * ((size_t)nV + 1));
  for (int32_t i = 0; i < nV; ++i) {
    vd[i].numOutEdges = e.dstOffsets[i + 1] - e.dstOffsets[i];
    vd[i].rank = (i == source) ? 1.0f : 0.0f;
    vd[i].teleport = (i == source) ? alpha : 0.0f;
  }
  e.param = (double)(1.0f - alpha);
  ora_set_active(&e, 0, nV);
  if (iters > 0) ppr32_run(&e, vd, 0, iters, st);
  else if (st) { st->iterations = 0; st->run_ns = 0; }
  for (int32_t i = 0; i < nV; ++i) rank[i] = vd[i].rank;
  ora_engine_free(&e);
  free(vd);
  return 0;
}

int ora_run_ppr_f64(int32_t nV, int32_t nE, const int32_t *srcs,
                    const int32_t *dsts, int32_t source, double alpha,
                    int32_t iters, double *rank, ora_stats *st)
{
  if (ora_check_edges(nV, nE, srcs, dsts) || !rank) return 1;
  if (source < 0 || source >= nV || iters < 0) return 1;
  ora_engine e;
  ora_engine_init(&e, nV, nE, srcs, dsts);
  ppr64_vd *vd = (ppr64_vd *)malloc(sizeof(ppr64_vd) * ((size_t)nV + 1));
  for (int32_t i = 0; i < nV; ++i) {
    vd[i].numOutEdges = e.dstOffsets[i + 1] - e.dstOffsets[i];
    vd[i].rank = (i == source) ? 1.0 : 0.0;
    vd[i].teleport = (i == source) ? alpha : 0.0;
  }
  e.param = 1.0 - alpha;
  ora_set_active(&e, 0, nV);
  if (iters > 0) ppr64_run(&e, vd, 0, iters, st);
  else if (st) { st->iterations = 0; st->run_ns = 0; }
  for (int32_t i = 0; i < nV; ++i) rank[i] = vd[i].rank;
  ora_engine_free(&e);
  free(vd);
  return 0;
}
