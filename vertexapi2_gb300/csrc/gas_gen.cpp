// Deterministic synthetic graph generators (gas_gen_rmat, gas_gen_grid).
//
// These stand in for the reference's downloaded regression graphs
// (regressions/Makefile:32; kron_g500-logn21 is an R-MAT-21 Kronecker
// graph), which are not available offline.  Pure integer arithmetic on a
// counter-based SplitMix64 stream (Steele, Lea & Flood 2014), so the same
// seed gives the same edge list on x86-64 and aarch64 and for any thread
// count.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "gas_gb300.h"
#include "gas_internal.h"

using gas::internal::fail;

namespace {

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

int worker_count() {
  unsigned h = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(h, 16u));
}

template <class F>
void parallel_for(int64_t n, F f) {
  const int nt = worker_count();
  if (nt <= 1 || n < (1 << 16)) {
    f(0, n);
    return;
  }
  std::vector<std::thread> ts;
  for (int t = 0; t < nt; ++t) {
    int64_t b = n * t / nt, e = n * (t + 1) / nt;
    ts.emplace_back([=] { f(b, e); });
  }
  for (auto &t : ts) t.join();
}

// LSD radix sort of keys using `bits` significant bits, 11 bits per pass.
void radix_sort(std::vector<uint64_t> &keys, int bits) {
  std::vector<uint64_t> tmp(keys.size());
  const int kDigit = 11;
  const uint64_t mask = (1u << kDigit) - 1;
  for (int shift = 0; shift < bits; shift += kDigit) {
    std::vector<size_t> cnt((size_t)mask + 2, 0);
    for (uint64_t k : keys) cnt[((k >> shift) & mask) + 1]++;
    for (size_t d = 1; d < cnt.size(); ++d) cnt[d] += cnt[d - 1];
    for (uint64_t k : keys) tmp[cnt[(k >> shift) & mask]++] = k;
    keys.swap(tmp);
  }
}

int bits_for(uint64_t maxv) {
  int b = 1;
  while (b < 64 && (maxv >> b)) ++b;
  return b;
}

uint32_t weight_of(uint64_t wseed, int32_t u, int32_t v, int32_t lo, int32_t hi) {
  const uint64_t a = (uint64_t)(uint32_t)std::min(u, v), b = (uint64_t)(uint32_t)std::max(u, v);
  const uint64_t h = splitmix64(wseed ^ splitmix64((a << 32) | b));
  return (uint32_t)lo + (uint32_t)(h % (uint64_t)(hi - lo + 1));
}

gas_status fill_output(int32_t nV, const std::vector<int32_t> &src, const std::vector<int32_t> &dst,
                       bool weighted, uint64_t wseed, int32_t wLo, int32_t wHi,
                       gas_edge_list *out) {
  const size_t m = src.size();
  out->nVertices = nV;
  out->nEdges = (int64_t)m;
  out->srcs = (int32_t *)malloc(sizeof(int32_t) * std::max<size_t>(m, 1));
  out->dsts = (int32_t *)malloc(sizeof(int32_t) * std::max<size_t>(m, 1));
  out->weights = weighted ? (int32_t *)malloc(sizeof(int32_t) * std::max<size_t>(m, 1)) : nullptr;
  if (!out->srcs || !out->dsts || (weighted && !out->weights)) {
    gas_edge_list_free(out);
    return fail(GAS_ERR_OOM, "edge list allocation");
  }
  if (m) {
    memcpy(out->srcs, src.data(), sizeof(int32_t) * m);
    memcpy(out->dsts, dst.data(), sizeof(int32_t) * m);
  }
  if (weighted) {
    int32_t *w = out->weights;
    parallel_for((int64_t)m, [&](int64_t b, int64_t e) {
      for (int64_t i = b; i < e; ++i) w[i] = (int32_t)weight_of(wseed, src[i], dst[i], wLo, wHi);
    });
  }
  return GAS_OK;
}

// Emits both directions of canonical (u < v) pairs sorted by (u, v), in
// (src, dst) order: stable counting sort by src of [reversed ; forward].
void symmetric_from_canonical(int32_t nV, const std::vector<uint64_t> &canon, int sh,
                              std::vector<int32_t> &src, std::vector<int32_t> &dst) {
  const size_t m = canon.size();
  const uint64_t lowMask = (sh >= 64) ? ~0ull : ((1ull << sh) - 1);
  std::vector<int64_t> off((size_t)nV + 1, 0);
  for (uint64_t k : canon) {
    off[(size_t)(k >> sh) + 1]++;
    off[(size_t)(k & lowMask) + 1]++;
  }
  for (int32_t v = 0; v < nV; ++v) off[(size_t)v + 1] += off[v];
  src.resize(2 * m);
  dst.resize(2 * m);
  std::vector<int64_t> cur(off.begin(), off.end() - 1);
  for (uint64_t k : canon) {  // reversed entries (v, u): u ascending per v
    const int32_t u = (int32_t)(k >> sh), v = (int32_t)(k & lowMask);
    const int64_t p = cur[v]++;
    src[p] = v;
    dst[p] = u;
  }
  for (uint64_t k : canon) {  // forward entries (u, v): v ascending per u
    const int32_t u = (int32_t)(k >> sh), v = (int32_t)(k & lowMask);
    const int64_t p = cur[u]++;
    src[p] = u;
    dst[p] = v;
  }
}

}  // namespace

extern "C" {

void gas_edge_list_free(gas_edge_list *l) {
  if (!l) return;
  free(l->srcs);
  free(l->dsts);
  free(l->weights);
  l->srcs = l->dsts = l->weights = nullptr;
  l->nEdges = 0;
  l->nVertices = 0;
}

gas_status gas_gen_rmat(int32_t scale, int32_t edgeFactor, double a, double b, double c,
                        uint64_t seed, int32_t symmetrize, int32_t wLo, int32_t wHi,
                        gas_edge_list *out) {
  if (!out) return fail(GAS_ERR_INVALID, "gas_gen_rmat: out is NULL");
  memset(out, 0, sizeof(*out));
  if (scale < 1 || scale > 30 || edgeFactor < 1)
    return fail(GAS_ERR_INVALID, "R-MAT scale must be in [1, 30], edge factor >= 1");
  if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
    return fail(GAS_ERR_INVALID, "R-MAT probabilities must be >= 0 with a+b+c <= 1");
  const bool weighted = wLo >= 1 && wHi >= wLo;
  const int32_t nV = (int32_t)(1u << scale);
  const int64_t samples = (int64_t)edgeFactor << scale;
  if (samples > (int64_t)1 << 31) return fail(GAS_ERR_UNSUPPORTED, "too many R-MAT samples");
  // quadrant thresholds on a 32-bit uniform draw
  const uint64_t tA = (uint64_t)(a * 4294967296.0);
  const uint64_t tAB = (uint64_t)((a + b) * 4294967296.0);
  const uint64_t tABC = (uint64_t)((a + b + c) * 4294967296.0);
  const int sh = scale;
  std::vector<uint64_t> keys;
  try {
    keys.resize((size_t)samples);
  } catch (const std::bad_alloc &) {
    return fail(GAS_ERR_OOM, "R-MAT sample buffer");
  }
  const uint64_t kSelf = ~0ull;
  parallel_for(samples, [&](int64_t beg, int64_t end) {
    for (int64_t e = beg; e < end; ++e) {
      uint64_t h = splitmix64(seed + 0x632BE59BD9B4E019ull * (uint64_t)(e + 1));
      uint32_t s = 0, d = 0;
      for (int l = 0; l < scale; ++l) {
        if (l > 0 && (l & 1) == 0) h = splitmix64(h);
        const uint64_t r = (l & 1) ? (h & 0xffffffffull) : (h >> 32);
        const uint32_t sb = r >= tAB ? 1u : 0u;
        const uint32_t db = (r >= tA && r < tAB) || r >= tABC ? 1u : 0u;
        s = (s << 1) | sb;
        d = (d << 1) | db;
      }
      if (s == d) {
        keys[e] = kSelf;
      } else if (symmetrize) {
        const uint32_t u = std::min(s, d), v = std::max(s, d);
        keys[e] = ((uint64_t)u << sh) | v;
      } else {
        keys[e] = ((uint64_t)s << sh) | d;
      }
    }
  });
  keys.erase(std::remove(keys.begin(), keys.end(), kSelf), keys.end());
  radix_sort(keys, 2 * sh);
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  std::vector<int32_t> src, dst;
  const uint64_t lowMask = (1ull << sh) - 1;
  if (symmetrize) {
    symmetric_from_canonical(nV, keys, sh, src, dst);
  } else {
    src.resize(keys.size());
    dst.resize(keys.size());
    for (size_t i = 0; i < keys.size(); ++i) {
      src[i] = (int32_t)(keys[i] >> sh);
      dst[i] = (int32_t)(keys[i] & lowMask);
    }
  }
  std::vector<uint64_t>().swap(keys);
  return fill_output(nV, src, dst, weighted, splitmix64(seed ^ 0x5745494748545321ull), wLo,
                     wHi, out);
}

gas_status gas_gen_grid(int32_t rows, int32_t cols, double pDelete, uint64_t seed, int32_t wLo,
                        int32_t wHi, gas_edge_list *out) {
  if (!out) return fail(GAS_ERR_INVALID, "gas_gen_grid: out is NULL");
  memset(out, 0, sizeof(*out));
  if (rows < 1 || cols < 1 || (int64_t)rows * cols >= (1ll << 30))
    return fail(GAS_ERR_INVALID, "grid dimensions out of range");
  if (pDelete < 0 || pDelete > 1) return fail(GAS_ERR_INVALID, "pDelete must be in [0, 1]");
  const bool weighted = wLo >= 1 && wHi >= wLo;
  const int64_t n = (int64_t)rows * cols;
  const int64_t H = (int64_t)rows * (cols - 1);
  const uint64_t thr = (uint64_t)(pDelete * 4294967296.0);
  auto kept = [&](int64_t eid) {
    return (splitmix64(seed + 0x9E3779B97F4A7C15ull * (uint64_t)(eid + 1)) >> 32) >= thr;
  };
  // union-find over kept edges
  std::vector<int32_t> parent((size_t)n);
  for (int64_t i = 0; i < n; ++i) parent[i] = (int32_t)i;
  auto find = [&](int32_t x) {
    while (parent[x] != x) {
      parent[x] = parent[parent[x]];
      x = parent[x];
    }
    return x;
  };
  auto unite = [&](int32_t x, int32_t y) {
    x = find(x);
    y = find(y);
    if (x == y) return;
    if (x < y) std::swap(x, y);
    parent[x] = y;  // smaller id becomes the root
  };
  for (int32_t r = 0; r < rows; ++r)
    for (int32_t c = 0; c + 1 < cols; ++c)
      if (kept((int64_t)r * (cols - 1) + c)) unite(r * cols + c, r * cols + c + 1);
  for (int32_t r = 0; r + 1 < rows; ++r)
    for (int32_t c = 0; c < cols; ++c)
      if (kept(H + (int64_t)r * cols + c)) unite(r * cols + c, (r + 1) * cols + c);
  std::vector<int32_t> size((size_t)n, 0);
  for (int64_t i = 0; i < n; ++i) size[find((int32_t)i)]++;
  int32_t best = 0;
  for (int64_t i = 0; i < n; ++i)
    if (size[i] > size[best]) best = (int32_t)i;  // first (smallest root) on ties
  std::vector<int32_t> label((size_t)n, -1);
  int32_t nV = 0;
  for (int64_t i = 0; i < n; ++i)
    if (find((int32_t)i) == best) label[i] = nV++;
  std::vector<int32_t> src, dst;
  src.reserve((size_t)nV * 4);
  dst.reserve((size_t)nV * 4);
  std::vector<int32_t> osrc, odst;  // original lattice ids, for weights
  osrc.reserve((size_t)nV * 4);
  odst.reserve((size_t)nV * 4);
  for (int32_t r = 0; r < rows; ++r)
    for (int32_t c = 0; c < cols; ++c) {
      const int32_t id = r * cols + c;
      if (label[id] < 0) continue;
      // neighbours in increasing new-id order: up, left, right, down
      struct Nb {
        bool ok;
        int32_t id;
      } nb[4] = {
          {r > 0 && kept(H + (int64_t)(r - 1) * cols + c), id - cols},
          {c > 0 && kept((int64_t)r * (cols - 1) + c - 1), id - 1},
          {c + 1 < cols && kept((int64_t)r * (cols - 1) + c), id + 1},
          {r + 1 < rows && kept(H + (int64_t)r * cols + c), id + cols},
      };
      for (auto &x : nb)
        if (x.ok && label[x.id] >= 0) {
          src.push_back(label[id]);
          dst.push_back(label[x.id]);
          osrc.push_back(id);
          odst.push_back(x.id);
        }
    }
  gas_status st = fill_output(nV, src, dst, false, 0, 0, 0, out);
  if (st) return st;
  if (weighted) {
    out->weights = (int32_t *)malloc(sizeof(int32_t) * std::max<size_t>(src.size(), 1));
    if (!out->weights) {
      gas_edge_list_free(out);
      return fail(GAS_ERR_OOM, "edge list allocation");
    }
    const uint64_t wseed = splitmix64(seed ^ 0x5745494748545321ull);
    for (size_t i = 0; i < src.size(); ++i)
      out->weights[i] = (int32_t)weight_of(wseed, osrc[i], odst[i], wLo, wHi);
  }
  return GAS_OK;
}

}  // extern "C"
