/*
 * TEST INFRASTRUCTURE ONLY -- builds the reference's own CPU engine.
 *
 * This file is compiled by oracle/build.py together with the reference's
 * unmodified refgas.h / util.h (GASEngineRef, refgas.h:31-225; util.h:44-121)
 * and graphio.cpp (graph loaders), read in place from the reference tree,
 * into oracle/_ref/libgas_ref.so.  It never ships and is never copied into
 * this repository.  The reference's vertex programs live in .cu files that
 * also include the GPU engine (which cannot be built), so they are restated
 * here host-side, member for member:
 *   BFS      bfs.cu:31-78        SSSP     sssp.cu:25-64
 *   CC       connected_component.cu:25-63
 *   PageRank pagerank.cu:27-73   (FP64 twin: same struct with double)
 * Drivers mirror bfs.cu:91-112, sssp.cu:67-82, connected_component.cu:66-81
 * and pagerank.cu:76-101.  The exported functions have the same signatures
 * as the oracle restatement (oracle/gas_oracle.h) with a ref_ prefix.
 */
#define __host__
#define __device__
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

using std::min;

#include "refgas.h"
#include "graphio.h"

#include "gas_oracle.h"

namespace {

int g_iterationCount;  // bfs.cu:27

struct BFS {
  struct VertexData { int depth; };
  struct EdgeData {};
  typedef int GatherResult;
  static const int gatherZero = INT_MAX - 1;
  static int gatherReduce(const int &, const int &) { return 0; }
  static int gatherMap(const VertexData *, const VertexData *, const EdgeData *) { return 0; }
  static bool apply(VertexData *vert, int) {
    if (vert->depth == -1) { vert->depth = g_iterationCount; return true; }
    return false;
  }
  static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

struct SSSP {
  typedef int VertexData;
  typedef int EdgeData;
  typedef int GatherResult;
  static const int maxLength = 100000;
  static const int gatherZero = INT_MAX - maxLength;
  static int gatherReduce(const int &l, const int &r) { return min(l, r); }
  static int gatherMap(const VertexData *, const VertexData *s, const EdgeData *e) { return *s + *e; }
  static bool apply(VertexData *cur, GatherResult d) {
    bool changed = d < *cur;
    *cur = min(*cur, d);
    return changed;
  }
  static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

// An SSSP whose scatter writes its edge (not a reference program): a visit
// count and the source's distance, through refgas.h's own scatter call.
struct SSSPVisits {
  typedef int VertexData;
  struct EdgeData { int w, visits, last; };
  typedef int GatherResult;
  static const int gatherZero = INT_MAX - 100000;
  static int gatherReduce(const int &l, const int &r) { return min(l, r); }
  static int gatherMap(const VertexData *, const VertexData *s, const EdgeData *e) { return *s + e->w; }
  static bool apply(VertexData *cur, GatherResult d) {
    bool changed = d < *cur;
    *cur = min(*cur, d);
    return changed;
  }
  static void scatter(const VertexData *src, const VertexData *, EdgeData *e) {
    e->visits += 1;
    e->last = *src;
  }
};

struct CC {
  typedef int VertexData;
  struct EdgeData {};
  typedef int GatherResult;
  static const int gatherZero = INT_MAX;
  static int gatherReduce(const int &l, const int &r) { return min(l, r); }
  static int gatherMap(const VertexData *, const VertexData *s, const EdgeData *) { return *s; }
  static bool apply(VertexData *cur, GatherResult l) {
    bool changed = l < *cur;
    *cur = min(*cur, l);
    return changed;
  }
  static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

template <typename Real>
struct PageRankT {
  static constexpr Real pageConst = (Real)0.15f;
  static constexpr Real tol = (Real)0.01f;
  struct VertexData { Real rank; int numOutEdges; };
  struct EdgeData {};
  typedef Real GatherResult;
  static constexpr Real gatherZero = (Real)0;
  static Real gatherMap(const VertexData *, const VertexData *s, const EdgeData *) {
    return s->rank / s->numOutEdges;
  }
  static Real gatherReduce(const Real &l, const Real &r) { return l + r; }
  static bool apply(VertexData *v, const Real &g) {
    Real newRank = pageConst + ((Real)1 - pageConst) * g;
    bool ret = std::fabs(newRank - v->rank) >= tol;
    v->rank = newRank;
    return ret;
  }
  static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

bool bad_edges(int nV, int nE, const int32_t *s, const int32_t *d) {
  if (nV < 0 || nE < 0) return true;
  for (int i = 0; i < nE; ++i)
    if (s[i] < 0 || s[i] >= nV || d[i] < 0 || d[i] >= nV) return true;
  return false;
}

// per-iteration counts computed outside the engine from its own CSR/CSC
struct Counter {
  std::vector<int> inOff, outOff;
  Counter(int nV, int nE, const int32_t *s, const int32_t *d) : inOff(nV + 1), outOff(nV + 1) {
    edgeListToCSR<int>(nV, nE, s, d, &outOff[0], 0, 0);
    edgeListToCSC<int>(nV, nE, s, d, &inOff[0], 0, 0);
  }
};

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch()).count();
}

// GASEngineRef keeps its active list private, so this harness reports only
// the iteration count and the run()+getResults() time (bfs.cu:100-111); the
// per-iteration frontier counts come from the restatement.
template <typename Engine>
void drive(Engine &e, int max_iters, ora_stats *st, bool bfs) {
  int iter = 0;
  if (bfs) g_iterationCount = 0;
  int64_t t0 = now_ns();
  while (e.countActive() && (max_iters <= 0 || iter < max_iters)) {
    e.gatherApply(!bfs);
    e.scatterActivate(!bfs);
    e.nextIter();
    ++iter;
    if (bfs) g_iterationCount = iter;
  }
  e.getResults();
  int64_t t1 = now_ns();
  if (st) { st->iterations = iter; st->run_ns = t1 - t0; }
}

}  // namespace

template <typename Real>
int pr_run(int32_t nV, int32_t nE, const int32_t *srcs, const int32_t *dsts,
           int32_t max_iters, Real *rank, ora_stats *st) {
  typedef PageRankT<Real> P;
  if (bad_edges(nV, nE, srcs, dsts)) return 1;
  std::vector<int> off(nV + 1);
  edgeListToCSR<int>(nV, nE, srcs, dsts, &off[0], 0, 0);  // pagerank.cu:120-132
  std::vector<typename P::VertexData> vd(nV);
  for (int i = 0; i < nV; ++i) {
    vd[i].numOutEdges = off[i + 1] - off[i];
    vd[i].rank = P::pageConst;
  }
  GASEngineRef<P> e;
  e.setGraph(nV, vd.data(), nE, 0, srcs, dsts);
  e.setActive(0, nV);
  drive(e, max_iters, st, false);
  for (int i = 0; i < nV; ++i) rank[i] = vd[i].rank;
  return 0;
}

extern "C" {

int ref_run_bfs(int32_t nV, int32_t nE, const int32_t *srcs, const int32_t *dsts,
                int32_t source, int32_t *depth, ora_stats *st) {
  if (bad_edges(nV, nE, srcs, dsts) || source < 0 || source >= nV) return 1;
  std::vector<BFS::VertexData> vd(nV);
  for (int i = 0; i < nV; ++i) vd[i].depth = -1;
  GASEngineRef<BFS> e;
  e.setGraph(nV, vd.data(), nE, 0, srcs, dsts);
  e.setActive(source, source + 1);
  drive(e, 0, st, true);
  for (int i = 0; i < nV; ++i) depth[i] = vd[i].depth;
  return 0;
}

int ref_run_sssp(int32_t nV, int32_t nE, const int32_t *srcs, const int32_t *dsts,
                 const int32_t *w, int32_t source, int32_t *dist, ora_stats *st) {
  if (bad_edges(nV, nE, srcs, dsts) || source < 0 || source >= nV) return 1;
  for (int i = 0; i < nV; ++i) dist[i] = SSSP::gatherZero;
  dist[source] = 0;
  std::vector<int> ed(w, w + nE);
  GASEngineRef<SSSP> e;
  e.setGraph(nV, dist, nE, ed.data(), srcs, dsts);
  e.setActive(0, nV);
  drive(e, 0, st, false);
  return 0;
}

int ref_run_cc(int32_t nV, int32_t nE, const int32_t *srcs, const int32_t *dsts,
               int32_t *label, ora_stats *st) {
  if (bad_edges(nV, nE, srcs, dsts)) return 1;
  for (int i = 0; i < nV; ++i) label[i] = i;
  GASEngineRef<CC> e;
  e.setGraph(nV, label, nE, 0, srcs, dsts);
  e.setActive(0, nV);
  drive(e, 0, st, false);
  return 0;
}

int ref_run_pagerank_f32(int32_t nV, int32_t nE, const int32_t *s, const int32_t *d,
                         int32_t max_iters, float *rank, ora_stats *st) {
  return pr_run<float>(nV, nE, s, d, max_iters, rank, st);
}

int ref_run_pagerank_f64(int32_t nV, int32_t nE, const int32_t *s, const int32_t *d,
                         int32_t max_iters, double *rank, ora_stats *st) {
  return pr_run<double>(nV, nE, s, d, max_iters, rank, st);
}

int ref_run_sssp_visits(int32_t nV, int32_t nE, const int32_t *srcs, const int32_t *dsts,
                        const int32_t *w, int32_t source, int32_t *dist, int32_t *visits,
                        int32_t *last, ora_stats *st) {
  if (bad_edges(nV, nE, srcs, dsts) || source < 0 || source >= nV) return 1;
  std::vector<int> vd(nV, SSSPVisits::gatherZero);
  vd[source] = 0;
  std::vector<SSSPVisits::EdgeData> ed(nE > 0 ? nE : 1);
  for (int i = 0; i < nE; ++i) ed[i] = {w[i], 0, 0};
  GASEngineRef<SSSPVisits> e;
  e.setGraph(nV, vd.data(), nE, ed.data(), srcs, dsts);
  e.setActive(0, nV);
  drive(e, 0, st, false);
  for (int i = 0; i < nV; ++i) dist[i] = vd[i];
  for (int i = 0; i < nE; ++i) {
    visits[i] = ed[i].visits;
    last[i] = ed[i].last;
  }
  return 0;
}

// graphio.cpp:441-473 loadGraph; arrays are malloc'd, free with ref_free.
int ref_load_graph(const char *path, int32_t *nV, int32_t *nE, int32_t **srcs,
                   int32_t **dsts, int32_t **weights) {
  int n = 0;
  std::vector<int> s, d, w;
  loadGraph(path, n, s, d, weights ? &w : 0);
  *nV = n;
  *nE = (int32_t)s.size();
  *srcs = (int32_t *)malloc(sizeof(int32_t) * (s.size() + 1));
  *dsts = (int32_t *)malloc(sizeof(int32_t) * (d.size() + 1));
  std::copy(s.begin(), s.end(), *srcs);
  std::copy(d.begin(), d.end(), *dsts);
  if (weights) {
    *weights = (int32_t *)malloc(sizeof(int32_t) * (w.size() + 1));
    std::copy(w.begin(), w.end(), *weights);
  }
  return (int)w.size();
}

void ref_free(void *p) { free(p); }

}  // extern "C"
