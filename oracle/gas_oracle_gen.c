/*
 * TEST INFRASTRUCTURE ONLY -- the oracle's own synthetic graph generators.
 *
 * The CPU legs of the benchmark (the reference arm above all) must build
 * their input graphs without loading the product library, so the oracle
 * carries a second, independent implementation of the seeded R-MAT and
 * lattice generators that define the benchmark graphs.  The edge lists
 * must be identical to the product's (same SplitMix64 counter stream,
 * Steele, Lea & Flood 2014; same integer thresholds; same edge order);
 * tests/test_oracle.py compares the two and checks the edge-list hashes
 * recorded in tests/golden/index.json.
 *
 * Edge order of the outputs:
 *   R-MAT directed:   (src, dst) ascending, duplicates and self-loops removed;
 *   R-MAT symmetric:  both directions of every undirected pair, (src, dst)
 *                     ascending;
 *   lattice:          vertices row-major (relabelled over the largest
 *                     component), per vertex the neighbours up, left, right,
 *                     down.
 * Weights: lo + h % (hi - lo + 1) with h a hash of the unordered pair, so
 * both directions of an edge carry the same weight.
 */
#define _POSIX_C_SOURCE 200809L
#include "gas_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static uint64_t sm64(uint64_t x)
{
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

static int32_t pair_weight(uint64_t wseed, int32_t u, int32_t v, int32_t lo, int32_t hi)
{
  uint64_t a = (uint32_t)(u < v ? u : v), b = (uint32_t)(u < v ? v : u);
  uint64_t h = sm64(wseed ^ sm64((a << 32) | b));
  return (int32_t)((uint32_t)lo + (uint32_t)(h % (uint64_t)(hi - lo + 1)));
}

static uint64_t weight_seed(uint64_t seed) { return sm64(seed ^ 0x5745494748545321ull); }

void ora_graph_free(ora_graph *g)
{
  if (!g) return;
  free(g->srcs);
  free(g->dsts);
  free(g->weights);
  memset(g, 0, sizeof(*g));
}

/* LSD radix sort of n 64-bit keys on their low `bits` bits. */
static int radix_sort_u64(uint64_t *keys, size_t n, int bits)
{
  uint64_t *tmp = (uint64_t *)malloc(sizeof(uint64_t) * (n ? n : 1));
  size_t *cnt = (size_t *)malloc(sizeof(size_t) * (65536 + 1));
  if (!tmp || !cnt) { free(tmp); free(cnt); return 1; }
  uint64_t *a = keys, *b = tmp;
  for (int shift = 0; shift < bits; shift += 16) {
    memset(cnt, 0, sizeof(size_t) * (65536 + 1));
    for (size_t i = 0; i < n; ++i) cnt[((a[i] >> shift) & 0xffff) + 1]++;
    for (int d = 0; d < 65536; ++d) cnt[d + 1] += cnt[d];
    for (size_t i = 0; i < n; ++i) b[cnt[(a[i] >> shift) & 0xffff]++] = a[i];
    uint64_t *t = a; a = b; b = t;
  }
  if (a != keys) memcpy(keys, a, sizeof(uint64_t) * n);
  free(tmp);
  free(cnt);
  return 0;
}

typedef struct {
  uint64_t *keys;
  int64_t beg, end;
  uint64_t seed, tA, tAB, tABC;
  int scale, symmetrize;
} rmat_job;

#define ORA_SELF_LOOP (~0ull)

static void *rmat_worker(void *p)
{
  rmat_job *j = (rmat_job *)p;
  const int sh = j->scale;
  for (int64_t e = j->beg; e < j->end; ++e) {
    uint64_t h = sm64(j->seed + 0x632BE59BD9B4E019ull * (uint64_t)(e + 1));
    uint32_t s = 0, d = 0;
    for (int l = 0; l < sh; ++l) {
      if (l > 0 && (l & 1) == 0) h = sm64(h);
      uint64_t r = (l & 1) ? (h & 0xffffffffull) : (h >> 32);
      uint32_t sb = r >= j->tAB;
      uint32_t db = (r >= j->tA && r < j->tAB) || r >= j->tABC;
      s = (s << 1) | sb;
      d = (d << 1) | db;
    }
    if (s == d)
      j->keys[e] = ORA_SELF_LOOP;
    else if (j->symmetrize)
      j->keys[e] = ((uint64_t)(s < d ? s : d) << sh) | (s < d ? d : s);
    else
      j->keys[e] = ((uint64_t)s << sh) | d;
  }
  return NULL;
}

static int host_threads(void)
{
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  if (n < 1) n = 1;
  if (n > 32) n = 32;
  return (int)n;
}

static int fill_weights(ora_graph *g, uint64_t wseed, int32_t lo, int32_t hi)
{
  if (!(lo >= 1 && hi >= lo)) return 0;
  g->weights = (int32_t *)malloc(sizeof(int32_t) * (size_t)(g->nEdges ? g->nEdges : 1));
  if (!g->weights) return 1;
  for (int64_t i = 0; i < g->nEdges; ++i)
    g->weights[i] = pair_weight(wseed, g->srcs[i], g->dsts[i], lo, hi);
  return 0;
}

int ora_gen_rmat(int32_t scale, int32_t edgeFactor, double a, double b, double c,
                 uint64_t seed, int32_t symmetrize, int32_t wLo, int32_t wHi, ora_graph *out)
{
  if (!out) return 1;
  memset(out, 0, sizeof(*out));
  if (scale < 1 || scale > 30 || edgeFactor < 1) return 1;
  if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return 1;
  const int64_t samples = (int64_t)edgeFactor << scale;
  if (samples > ((int64_t)1 << 31)) return 1;
  uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)samples);
  if (!keys) return 1;
  int nt = host_threads();
  if (samples < (1 << 16)) nt = 1;
  rmat_job jobs[32];
  pthread_t th[32];
  for (int t = 0; t < nt; ++t) {
    jobs[t].keys = keys;
    jobs[t].beg = samples * t / nt;
    jobs[t].end = samples * (t + 1) / nt;
    jobs[t].seed = seed;
    jobs[t].tA = (uint64_t)(a * 4294967296.0);
    jobs[t].tAB = (uint64_t)((a + b) * 4294967296.0);
    jobs[t].tABC = (uint64_t)((a + b + c) * 4294967296.0);
    jobs[t].scale = scale;
    jobs[t].symmetrize = symmetrize;
  }
  for (int t = 1; t < nt; ++t) pthread_create(&th[t], NULL, rmat_worker, &jobs[t]);
  rmat_worker(&jobs[0]);
  for (int t = 1; t < nt; ++t) pthread_join(th[t], NULL);
  /* drop self-loops, sort, dedup */
  size_t m = 0;
  for (int64_t i = 0; i < samples; ++i)
    if (keys[i] != ORA_SELF_LOOP) keys[m++] = keys[i];
  if (radix_sort_u64(keys, m, 2 * scale)) { free(keys); return 1; }
  size_t u = 0;
  for (size_t i = 0; i < m; ++i)
    if (i == 0 || keys[i] != keys[i - 1]) keys[u++] = keys[i];
  const uint64_t low = (1ull << scale) - 1;
  if (symmetrize) {
    /* both directions of each canonical pair, re-sorted by (src, dst) */
    uint64_t *both = (uint64_t *)malloc(sizeof(uint64_t) * (2 * u ? 2 * u : 1));
    if (!both) { free(keys); return 1; }
    for (size_t i = 0; i < u; ++i) {
      both[2 * i] = keys[i];
      both[2 * i + 1] = ((keys[i] & low) << scale) | (keys[i] >> scale);
    }
    free(keys);
    keys = both;
    u *= 2;
    if (radix_sort_u64(keys, u, 2 * scale)) { free(keys); return 1; }
  }
  out->nVertices = (int32_t)(1u << scale);
  out->nEdges = (int64_t)u;
  out->srcs = (int32_t *)malloc(sizeof(int32_t) * (u ? u : 1));
  out->dsts = (int32_t *)malloc(sizeof(int32_t) * (u ? u : 1));
  if (!out->srcs || !out->dsts) { free(keys); ora_graph_free(out); return 1; }
  for (size_t i = 0; i < u; ++i) {
    out->srcs[i] = (int32_t)(keys[i] >> scale);
    out->dsts[i] = (int32_t)(keys[i] & low);
  }
  free(keys);
  if (fill_weights(out, weight_seed(seed), wLo, wHi)) { ora_graph_free(out); return 1; }
  return 0;
}

static int32_t uf_find(int32_t *parent, int32_t x)
{
  while (parent[x] != x) {
    parent[x] = parent[parent[x]];
    x = parent[x];
  }
  return x;
}

static void uf_union(int32_t *parent, int32_t x, int32_t y)
{
  x = uf_find(parent, x);
  y = uf_find(parent, y);
  if (x == y) return;
  if (x < y) parent[y] = x; else parent[x] = y;  /* the smaller id is the root */
}

int ora_gen_grid(int32_t rows, int32_t cols, double pDelete, uint64_t seed, int32_t wLo,
                 int32_t wHi, ora_graph *out)
{
  if (!out) return 1;
  memset(out, 0, sizeof(*out));
  if (rows < 1 || cols < 1 || (int64_t)rows * cols >= ((int64_t)1 << 30)) return 1;
  if (pDelete < 0 || pDelete > 1) return 1;
  const int64_t n = (int64_t)rows * cols;
  const int64_t H = (int64_t)rows * (cols - 1);  /* horizontal edges come first */
  const uint64_t thr = (uint64_t)(pDelete * 4294967296.0);
#define KEPT(eid) ((sm64(seed + 0x9E3779B97F4A7C15ull * (uint64_t)((eid) + 1)) >> 32) >= thr)
  int32_t *parent = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
  int32_t *label = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
  if (!parent || !label) { free(parent); free(label); return 1; }
  for (int64_t i = 0; i < n; ++i) parent[i] = (int32_t)i;
  for (int32_t r = 0; r < rows; ++r)
    for (int32_t c = 0; c + 1 < cols; ++c)
      if (KEPT((int64_t)r * (cols - 1) + c)) uf_union(parent, r * cols + c, r * cols + c + 1);
  for (int32_t r = 0; r + 1 < rows; ++r)
    for (int32_t c = 0; c < cols; ++c)
      if (KEPT(H + (int64_t)r * cols + c)) uf_union(parent, r * cols + c, (r + 1) * cols + c);
  /* component sizes (label[] as a counter), the largest with the smallest root */
  memset(label, 0, sizeof(int32_t) * (size_t)n);
  for (int64_t i = 0; i < n; ++i) label[uf_find(parent, (int32_t)i)]++;
  int32_t best = 0;
  for (int64_t i = 0; i < n; ++i)
    if (label[i] > label[best]) best = (int32_t)i;
  int32_t nV = 0;
  for (int64_t i = 0; i < n; ++i) label[i] = uf_find(parent, (int32_t)i) == best ? nV++ : -1;
  free(parent);
  size_t cap = (size_t)nV * 4 + 1;
  out->srcs = (int32_t *)malloc(sizeof(int32_t) * cap);
  out->dsts = (int32_t *)malloc(sizeof(int32_t) * cap);
  int32_t *osrc = (int32_t *)malloc(sizeof(int32_t) * cap);
  int32_t *odst = (int32_t *)malloc(sizeof(int32_t) * cap);
  if (!out->srcs || !out->dsts || !osrc || !odst) {
    free(label); free(osrc); free(odst); ora_graph_free(out); return 1;
  }
  int64_t m = 0;
  for (int32_t r = 0; r < rows; ++r)
    for (int32_t c = 0; c < cols; ++c) {
      const int32_t id = r * cols + c;
      if (label[id] < 0) continue;
      int ok[4] = {r > 0 && KEPT(H + (int64_t)(r - 1) * cols + c),
                   c > 0 && KEPT((int64_t)r * (cols - 1) + c - 1),
                   c + 1 < cols && KEPT((int64_t)r * (cols - 1) + c),
                   r + 1 < rows && KEPT(H + (int64_t)r * cols + c)};
      int32_t nb[4] = {id - cols, id - 1, id + 1, id + cols};
      for (int k = 0; k < 4; ++k)
        if (ok[k] && label[nb[k]] >= 0) {
          out->srcs[m] = label[id];
          out->dsts[m] = label[nb[k]];
          osrc[m] = id;
          odst[m] = nb[k];
          ++m;
        }
    }
#undef KEPT
  free(label);
  out->nVertices = nV;
  out->nEdges = m;
  int rc = 0;
  if (wLo >= 1 && wHi >= wLo) {
    out->weights = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m ? m : 1));
    if (!out->weights) {
      rc = 1;
    } else {
      const uint64_t wseed = weight_seed(seed);
      for (int64_t i = 0; i < m; ++i) out->weights[i] = pair_weight(wseed, osrc[i], odst[i], wLo, wHi);
    }
  }
  free(osrc);
  free(odst);
  if (rc) ora_graph_free(out);
  return rc;
}
