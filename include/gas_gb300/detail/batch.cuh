// Batched multi-source BFS and SSSP: Q queries with independent sources on
// one resident graph, all rounds in one persistent cooperative launch.
//
// State is laid out vertex-major so a warp touches one vertex's queries
// with coalesced accesses:
//   value[V][Q]      BFS depth (-1 unreached) or SSSP distance (int32)
//   mask[3][V][W]    W = Q/32 words per vertex: the queries whose value at
//                    this vertex changed in a round (rotating: round r
//                    reads mask[r%3], writes mask[(r+1)%3] and clears
//                    mask[(r+2)%3], so no stamps and no extra barrier)
//   seen[V][W]       BFS: queries that have reached the vertex
//
// A round runs in one of two modes, chosen from the previous round's
// changed vertices (list L, with their out-degree total E_out):
//   push  (E_out * alpha <= E): a warp per list entry -- a changed vertex
//         u and one kPushChunk-edge chunk of its out-edges (hubs span
//         several entries, so no warp walks a hub alone) -- updates the
//         destinations for u's changed queries with atomics, a lane per
//         edge (or, for SSSP when u has more changed queries than the
//         chunk has edges, a lane per query); destinations that change are
//         appended to the next list (one atomic per warp and step);
//   pull  otherwise: one pass over work units (a vertex's in-edges, split
//         into chunks of at most `chunk` edges for high in-degree vertices),
//         lanes mapped to queries (lane l owns queries l + 32k), followed
//         by a compaction of the changed vertices into the list.
// The updates:
//   BFS   next(v) = OR of mask[u] over in-neighbours u, minus seen(v);
//         newly seen queries get depth = round + 1           (bfs.cu:54-66)
//   SSSP  for queries whose distance at in-neighbour u changed, relax
//         dist[u][q] + w with atomicMin on dist[v][q]        (sssp.cu:36-55)
// Every query's result equals its single-source result bit for bit: BFS
// depths and shortest-path distances are unique.  Rounds end when a round
// changes nothing (bounded waits, as in the single-query persistent kernel).
#pragma once

#include "persistent.cuh"

namespace gas {
namespace detail {

enum BatchKind { kBatchBFS = 1, kBatchSSSP = 2 };

struct BatchArgs {
  int32_t nVertices;
  int32_t nEdges;
  const int32_t *outOffsets;  // CSR (push rounds)
  const int32_t *outDests;
  const int32_t *weightsOut;  // CSR order (SSSP push rounds)
  int32_t *list[3];           // [listCap] changed vertices (rotating), one
  int32_t *listC[3];          //   entry per kPushChunk out-edges: (vertex, chunk)
  unsigned long long *listCnt;  // [3] (entries << 32) | out-degree total
  int32_t *inList;            // [V] round stamp of list membership
  int32_t alpha;              // push when out-degree total * alpha <= nEdges
  int32_t nQueries;       // padded to 32 * W
  const int32_t *inSources;
  const int32_t *weights;  // CSC order (SSSP)
  const int32_t *unitV;
  const int32_t *unitBeg;
  const int32_t *unitEnd;
  int32_t nUnits;
  int32_t *value;          // [V][Q]
  unsigned *mask[3];       // [V][W] each
  unsigned *seen;          // [V][W] (BFS)
  unsigned long long *cnt; // [3] changed (vertex, query) pairs per round
  unsigned *barrier;       // [2]
  unsigned *errWord;
  int32_t *roundsOut;
  int32_t maxRounds;       // 0 = until nothing changes
  // SSSP bucket order (delta-stepping; persistent kernel only): a changed
  // (u, q) is relaxed once dist[u][q] < thresh[q]; others wait in the
  // changed set.  A query's bound grows by delta after a round in which it
  // produced no value below the bound.  0 = every changed pair every round.
  int32_t delta;
  int32_t *thresh[2];      // [Q] by round parity
  unsigned *nearFlag[3];   // [W] queries with a new value below the bound (rotating)
  // Pair frontier (graphs of small out-degree, V * Q < 2^31): the changed
  // set is a list of (vertex, query) entries u * Q + q, one lane each,
  // instead of vertex entries with query masks; every round pushes.
  uint32_t *pairs[3];      // [V * Q] each (rotating, counts in listCnt >> 32)
  int32_t pairMode;
};

// Shared-memory view of the bucket bounds for one round (null when off).
struct BatchBucket {
  const int32_t *bound;  // [Q] this round's thresh
  unsigned *near;        // [W] block-local near flags
};

constexpr int32_t kBatchInf = 0x7fffffff - 100000;  // SSSP gatherZero (sssp.cu:32-33)

// Out-edges per push-list entry; a list holds at most V + E / kPushChunk
// entries (each vertex once per round).
constexpr int kPushChunk = 512;

__host__ __device__ inline long long batch_list_capacity(long long nVertices, long long nEdges) {
  return nVertices + nEdges / kPushChunk + 32;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(kFullMask, x, o);
  return x;  // lane 0
}

// Appends, for each lane with `want`, vertex v of out-degree d to a list as
// ceil(d / kPushChunk) entries (at least one): one atomic per warp.
// Warp-uniform call.
__device__ __forceinline__ void warp_append(bool want, int v, int d, int32_t *list,
                                            int32_t *listC, unsigned long long *cnt) {
  const int lane = threadIdx.x & 31;
  const int ne = want ? max(1, (d + kPushChunk - 1) / kPushChunk) : 0;
  int incl = ne;
  unsigned dsum = want ? (unsigned)d : 0u;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFullMask, incl, o);
    const unsigned z = __shfl_up_sync(kFullMask, dsum, o);
    if (lane >= o) {
      incl += y;
      dsum += z;
    }
  }
  const int total = __shfl_sync(kFullMask, incl, 31);
  if (total == 0) return;
  const unsigned dtot = __shfl_sync(kFullMask, dsum, 31);
  unsigned long long base = 0ull;
  if (lane == 0) base = atomicAdd(cnt, ((unsigned long long)total << 32) | dtot);
  base = __shfl_sync(kFullMask, base, 0);
  const long long pos = (long long)(base >> 32) + incl - ne;
  for (int c = 0; c < ne; ++c) {
    list[pos + c] = v;
    listC[pos + c] = c;
  }
}

template <int W, int KIND>
__device__ __forceinline__ void batch_unit(const BatchArgs &a, int u, int round,
                                           const unsigned *cur, unsigned *nxt,
                                           unsigned long long &changed) {
  const int lane = threadIdx.x & 31;
  const int v = a.unitV[u];
  const int beg = a.unitBeg[u], end = a.unitEnd[u];
  const int Q = W * 32;
  if (KIND == kBatchBFS) {
    unsigned acc[W];
#pragma unroll
    for (int k = 0; k < W; ++k) acc[k] = 0u;
    for (int e0 = beg; e0 < end; e0 += 32) {
      const int e = e0 + lane;
      const int s = e < end ? __ldg(a.inSources + e) : -1;
      unsigned m[W];
#pragma unroll
      for (int k = 0; k < W; ++k) m[k] = s >= 0 ? __ldcg(cur + (size_t)s * W + k) : 0u;
#pragma unroll
      for (int k = 0; k < W; ++k) acc[k] |= __reduce_or_sync(kFullMask, m[k]);
    }
#pragma unroll
    for (int k = 0; k < W; ++k) {
      if (!acc[k]) continue;  // warp-uniform
      unsigned fresh = 0u;
      if (lane == 0) {
        const unsigned old = atomicOr(a.seen + (size_t)v * W + k, acc[k]);
        fresh = acc[k] & ~old;
        if (fresh) atomicOr(nxt + (size_t)v * W + k, fresh);
      }
      fresh = __shfl_sync(kFullMask, fresh, 0);
      if ((fresh >> lane) & 1u) a.value[(size_t)v * Q + k * 32 + lane] = round + 1;
      if (lane == 0) changed += __popc(fresh);
    }
  } else {
    int best[W];
#pragma unroll
    for (int k = 0; k < W; ++k) best[k] = kBatchInf;
    for (int e0 = beg; e0 < end; e0 += 32) {
      // lane j loads edge e0+j: source, weight and its changed-query mask
      const int e = e0 + lane;
      const bool ok = e < end;
      const int s = ok ? __ldg(a.inSources + e) : 0;
      const int w = ok ? __ldg(a.weights + e) : 0;
      unsigned m[W], any = 0u;
#pragma unroll
      for (int k = 0; k < W; ++k) {
        m[k] = ok ? __ldcg(cur + (size_t)s * W + k) : 0u;
        any |= m[k];
      }
      unsigned work = __ballot_sync(kFullMask, any != 0u);  // edges with a changed query
      while (work) {  // warp-uniform; four edges' loads in flight per pass
        int js[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          js[t] = work ? __ffs(work) - 1 : -1;
          if (work) work &= work - 1;
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          if (js[t] < 0) continue;
          const int sj = __shfl_sync(kFullMask, s, js[t]);
          const int wj = __shfl_sync(kFullMask, w, js[t]);
#pragma unroll
          for (int k = 0; k < W; ++k) {
            const unsigned mk = __shfl_sync(kFullMask, m[k], js[t]);
            if ((mk >> lane) & 1u) {
              const int d = __ldcg(a.value + (size_t)sj * Q + k * 32 + lane);
              best[k] = min(best[k], d + wj);
            }
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < W; ++k) {
      bool improved = false;
      if (best[k] < kBatchInf) {
        const int old = atomicMin(a.value + (size_t)v * Q + k * 32 + lane, best[k]);
        improved = best[k] < old;
      }
      const unsigned word = __ballot_sync(kFullMask, improved);
      if (lane == 0 && word) {
        atomicOr(nxt + (size_t)v * W + k, word);
        changed += __popc(word);
      }
    }
  }
}

// Push round: a warp per list entry (u, chunk), lanes over the chunk's
// out-edges (32 at a time).  Warp-uniform.
template <int W, int KIND>
__device__ __forceinline__ void batch_push_unit(const BatchArgs &a, int u, int chunk, int round,
                                                const unsigned *cur, unsigned *nxt,
                                                int32_t *listNext, int32_t *listNextC,
                                                unsigned long long *cntNext,
                                                unsigned long long &changed,
                                                const BatchBucket bk = BatchBucket{nullptr, nullptr}) {
  const int lane = threadIdx.x & 31;
  const int Q = W * 32;
  unsigned m[W];
#pragma unroll
  for (int k = 0; k < W; ++k) m[k] = __ldcg(cur + (size_t)u * W + k);
  int du[W];
  if (KIND == kBatchSSSP) {
#pragma unroll
    for (int k = 0; k < W; ++k)
      du[k] = ((m[k] >> lane) & 1u) ? __ldcg(a.value + (size_t)u * Q + k * 32 + lane) : kBatchInf;
  }
  bool deferred = false;
  if (KIND == kBatchSSSP && bk.bound) {  // relax below the bound now, keep the rest
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const unsigned nearM =
          __ballot_sync(kFullMask, ((m[k] >> lane) & 1u) && du[k] < bk.bound[k * 32 + lane]);
      const unsigned far = m[k] & ~nearM;
      m[k] = nearM;
      if (far) {
        deferred = true;
        if (lane == 0) {
          atomicOr(nxt + (size_t)u * W + k, far);
          changed += __popc(far);
        }
      }
    }
  }
  int nbits = 0, nwords = 0;
#pragma unroll
  for (int k = 0; k < W; ++k) {
    nbits += __popc(m[k]);
    nwords += m[k] != 0u;
  }
  unsigned nearW[W];
#pragma unroll
  for (int k = 0; k < W; ++k) nearW[k] = 0u;
  const int ub = a.outOffsets[u];
  const int eb = ub + chunk * kPushChunk;
  const int ee = min(eb + kPushChunk, a.outOffsets[u + 1]);
  // SSSP: a lane per edge costs ceil(deg/32) * nbits atomic steps, a lane
  // per query deg * nwords
  const bool perEdge =
      KIND == kBatchBFS || (long long)((ee - eb + 31) / 32) * nbits <= (long long)(ee - eb) * nwords;
  for (int e0 = eb; e0 < ee; e0 += 32) {
    const int e = e0 + lane;
    const bool ok = e < ee;
    const int v = ok ? __ldg(a.outDests + e) : 0;
    bool any = false;
    if (KIND == kBatchBFS) {
#pragma unroll
      for (int k = 0; k < W; ++k) {
        if (!m[k] || !ok) continue;
        const unsigned old = atomicOr(a.seen + (size_t)v * W + k, m[k]);
        unsigned fresh = m[k] & ~old;
        if (!fresh) continue;
        atomicOr(nxt + (size_t)v * W + k, fresh);
        any = true;
        changed += __popc(fresh);
        while (fresh) {
          const int b = __ffs(fresh) - 1;
          fresh &= fresh - 1u;
          a.value[(size_t)v * Q + k * 32 + b] = round + 1;
        }
      }
    } else if (perEdge) {
      const int w = ok ? __ldg(a.weightsOut + e) : 0;
#pragma unroll
      for (int k = 0; k < W; ++k) {
        unsigned bits = m[k], imp = 0u;
        while (bits) {  // warp-uniform; up to four relaxations in flight
          int bs[4], ds[4], olds[4];
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            bs[t] = bits ? __ffs(bits) - 1 : -1;
            if (bits) bits &= bits - 1u;
            ds[t] = __shfl_sync(kFullMask, du[k], bs[t] < 0 ? 0 : bs[t]);
          }
#pragma unroll
          for (int t = 0; t < 4; ++t)
            olds[t] = (ok && bs[t] >= 0)
                          ? atomicMin(a.value + (size_t)v * Q + k * 32 + bs[t], ds[t] + w)
                          : kBatchInf;
#pragma unroll
          for (int t = 0; t < 4; ++t)
            if (ok && bs[t] >= 0 && ds[t] + w < olds[t]) {
              imp |= 1u << bs[t];
              if (bk.bound && ds[t] + w < bk.bound[k * 32 + bs[t]]) nearW[k] |= 1u << bs[t];
            }
        }
        if (imp) {
          atomicOr(nxt + (size_t)v * W + k, imp);
          any = true;
          changed += __popc(imp);
        }
      }
    } else {  // lane per query, the 32 edges in turn
      const int w = ok ? __ldg(a.weightsOut + e) : 0;
      const int n = min(32, ee - e0);
      unsigned anyMask = 0u;
      for (int t = 0; t < n; ++t) {
        const int vt = __shfl_sync(kFullMask, v, t);
        const int wt = __shfl_sync(kFullMask, w, t);
#pragma unroll
        for (int k = 0; k < W; ++k) {
          bool imp = false;
          if ((m[k] >> lane) & 1u) {
            const int cand = du[k] + wt;
            const int old = atomicMin(a.value + (size_t)vt * Q + k * 32 + lane, cand);
            imp = cand < old;
            if (imp && bk.bound && cand < bk.bound[k * 32 + lane]) nearW[k] |= 1u << lane;
          }
          const unsigned word = __ballot_sync(kFullMask, imp);
          if (word) {
            if (lane == 0) {
              atomicOr(nxt + (size_t)vt * W + k, word);
              changed += __popc(word);
            }
            anyMask |= 1u << t;
          }
        }
      }
      any = (anyMask >> lane) & 1u;
    }
    bool want = false;
    if (any) want = atomicExch(a.inList + v, round + 1) != round + 1;
    warp_append(want, v, want ? a.outOffsets[v + 1] - a.outOffsets[v] : 0, listNext, listNextC,
                cntNext);
  }
  if (KIND == kBatchSSSP && bk.bound) {
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const unsigned nw = __reduce_or_sync(kFullMask, nearW[k]);
      if (lane == 0 && nw) atomicOr(bk.near + k, nw);
    }
    // u keeps its deferred queries: back on the next list (all its chunks)
    bool wantU = false;
    if (deferred && lane == 0) wantU = atomicExch(a.inList + u, round + 1) != round + 1;
    warp_append(wantU, u, wantU ? a.outOffsets[u + 1] - ub : 0, listNext, listNextC, cntNext);
  }
}

// Appends each lane's entry (when `want`) to a pair list: one atomic per
// warp.  Warp-uniform call.
__device__ __forceinline__ void warp_append_pair(bool want, uint32_t entry, uint32_t *list,
                                                 unsigned long long *cnt) {
  const int lane = threadIdx.x & 31;
  const unsigned who = __ballot_sync(kFullMask, want);
  if (!who) return;
  unsigned long long base = 0ull;
  if (lane == 0) base = atomicAdd(cnt, (unsigned long long)__popc(who) << 32);
  base = __shfl_sync(kFullMask, base, 0) >> 32;
  if (want) list[base + __popc(who & ((1u << lane) - 1u))] = entry;
}

// Appends each lane's entries out[k] with want[k] (k < K) to a pair list:
// one atomic per warp for all K.  Warp-uniform call.
template <int K>
__device__ __forceinline__ void warp_append_pairs(const bool (&want)[K], const uint32_t (&out)[K],
                                                  uint32_t *list, unsigned long long *cnt) {
  const int lane = threadIdx.x & 31;
  unsigned n = 0u;
#pragma unroll
  for (int k = 0; k < K; ++k) n += want[k] ? 1u : 0u;
  unsigned incl = n;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned o = __shfl_up_sync(kFullMask, incl, d);
    if (lane >= d) incl += o;
  }
  const unsigned total = __shfl_sync(kFullMask, incl, 31);
  if (total == 0u) return;
  unsigned long long base = 0ull;
  if (lane == 31) base = atomicAdd(cnt, (unsigned long long)total << 32);
  base = __shfl_sync(kFullMask, base, 31) >> 32;
  unsigned long long pos = base + (incl - n);
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (want[k]) list[pos++] = out[k];
}

// Pair-frontier push (state query-major: value[q][v], mask and seen words
// [w][v], so that the pairs of one query's wavefront, which relax
// neighbouring vertices, touch neighbouring words): lane i takes entry i of
// the current pair list (when
// `valid`), a changed (u, q), and relaxes u's out-edges for q alone; a
// destination whose value changes is appended as (v, q) the first time its
// query bit is set this round.  Warp-uniform (lanes step through their
// edges together, up to the warp's largest out-degree).
template <int W, int KIND>
__device__ __forceinline__ void batch_pair_unit(const BatchArgs &a, bool valid, uint32_t entry,
                                                int round, unsigned *cur, unsigned *nxt, uint32_t *listNext,
                                                unsigned long long *cntNext,
                                                unsigned long long &changed,
                                                const BatchBucket bk) {
  constexpr int Q = 32 * W;
  constexpr int LOGQ = W == 1 ? 5 : W == 2 ? 6 : W == 4 ? 7 : 8;
  const int u = valid ? (int)(entry >> LOGQ) : 0;
  const int q = (int)(entry & (Q - 1));
  const unsigned bit = 1u << (q & 31);
  const int wq = q >> 5;
  const size_t V = (size_t)a.nVertices;  // pair batches keep their state query-major
  int eb = valid ? a.outOffsets[u] : 0;
  int deg = valid ? a.outOffsets[u + 1] - eb : 0;
  int du = 0;
  bool keep = false;
  if (KIND == kBatchSSSP && valid) {
    // Every bit of this round's mask belongs to a pair of this round's
    // list, and nothing else touches the mask this round: each pair clears
    // its word (idempotent zeros), so the mask is clean when it next
    // collects pairs, without a pass over all vertices.
    cur[(size_t)wq * V + u] = 0u;
    du = __ldcg(a.value + (size_t)q * V + u);
    if (bk.bound && du >= bk.bound[q]) {  // not this bucket: keep (u, q) for later
      const unsigned old = atomicOr(nxt + (size_t)wq * V + u, bit);
      keep = !(old & bit);
      changed += 1;
      deg = 0;
    }
  }
  if (KIND == kBatchSSSP && bk.bound) warp_append_pair(keep, entry, listNext, cntNext);
  // four out-edges a step, their appends to the next list in one atomic per
  // warp (the list counter is one word every warp of the grid contends for)
  constexpr int J = 4;
  const int maxDeg = __reduce_max_sync(kFullMask, deg);
  for (int j0 = 0; j0 < maxDeg; j0 += J) {
    bool want[J];
    uint32_t out[J];
#pragma unroll
    for (int t = 0; t < J; ++t) {
      const int j = j0 + t;
      want[t] = false;
      out[t] = 0u;
      if (j < deg) {
        const int v = __ldg(a.outDests + eb + j);
        if (KIND == kBatchBFS) {
          const unsigned old = atomicOr(a.seen + (size_t)wq * V + v, bit);
          if (!(old & bit)) {
            a.value[(size_t)q * V + v] = round + 1;
            want[t] = true;
          }
        } else {
          const int cand = du + __ldg(a.weightsOut + eb + j);
          const int old = atomicMin(a.value + (size_t)q * V + v, cand);
          if (cand < old) {
            const unsigned o2 = atomicOr(nxt + (size_t)wq * V + v, bit);
            want[t] = !(o2 & bit);
            if (bk.bound && cand < bk.bound[q] && !(bk.near[wq] & bit)) atomicOr(bk.near + wq, bit);
          }
        }
        if (want[t]) {
          changed += 1;
          out[t] = ((uint32_t)v << LOGQ) | (uint32_t)q;
        }
      }
    }
    warp_append_pairs<J>(want, out, listNext, cntNext);
  }
}

// After a pull round: list the vertices with a changed query.
template <int W>
__device__ __forceinline__ void batch_compact(const BatchArgs &a, const unsigned *nxt,
                                              int32_t *listNext, int32_t *listNextC,
                                              unsigned long long *cntNext) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  const long long gw = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  for (long long base = gw * 32; base < a.nVertices; base += warps * 32) {
    const long long v = base + lane;
    unsigned any = 0u;
    if (v < a.nVertices) {
#pragma unroll
      for (int k = 0; k < W; ++k) any |= __ldcg(nxt + (size_t)v * W + k);
    }
    const bool want = any != 0u;
    warp_append(want, (int)v, want ? a.outOffsets[v + 1] - a.outOffsets[v] : 0, listNext,
                listNextC, cntNext);
  }
}

// PAIRS: the instantiation for pair-frontier batches (a.pairMode set),
// which holds only the pair rounds: its smaller register budget (at most 40
// a thread) keeps more warps, and so more of the latency-bound atomics, in
// flight.  The other instantiation serves vertex-mask batches, at most 64
// registers a thread so that 4 CTAs fit an SM: its pull and push rounds are
// latency-bound too (256 R-MAT-21 SSSP queries: 118 ms at 4 CTAs/SM, 170 ms
// at the 2 a 128-register build allows).
template <int W, int KIND, bool PAIRS = false>
__global__ void __launch_bounds__(256, PAIRS ? 6 : 4) batch_run_kernel(const BatchArgs a) {
  __shared__ int32_t sBound[32 * W];
  __shared__ unsigned sNear[W];
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  const long long gw = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  // list entries are dealt to warps block-first (warp k of every block, then
  // warp k+1), so a short list spreads over every SM
  const long long gwl = (long long)(threadIdx.x / 32) * gridDim.x + blockIdx.x;
  const size_t maskWords = (size_t)a.nVertices * W;
  const bool buckets = KIND == kBatchSSSP && a.delta > 0;
  const BatchBucket bk{buckets ? sBound : nullptr, buckets ? sNear : nullptr};
  int r = 0;
  for (;; ++r) {
    if (a.maxRounds > 0 && r >= a.maxRounds) break;
    if (buckets) {
      // this round's bounds: last round's, plus delta for the queries that
      // produced no value below theirs (every block computes the same)
      const int32_t *tPrev = (r & 1) ? a.thresh[1] : a.thresh[0];
      int32_t *tNext = (r & 1) ? a.thresh[0] : a.thresh[1];
      const unsigned *nPrev = a.nearFlag[(r + 2) % 3];  // written in round r - 1
      for (int q = threadIdx.x; q < 32 * W; q += blockDim.x) {
        int32_t t = __ldcg(tPrev + q);
        if (r > 0 && !((__ldcg(nPrev + q / 32) >> (q % 32)) & 1u)) t += a.delta;
        sBound[q] = t;
        if (blockIdx.x == 0) tNext[q] = t;
      }
      if (threadIdx.x < W) sNear[threadIdx.x] = 0u;
      if (blockIdx.x == 0 && threadIdx.x < W) a.nearFlag[(r + 1) % 3][threadIdx.x] = 0u;
      __syncthreads();
    }
    unsigned *cur = a.mask[r % 3];
    unsigned *nxt = a.mask[(r + 1) % 3];
    unsigned *clr = a.mask[(r + 2) % 3];
    const int rc = r % 3, rn = (r + 1) % 3;
    const int32_t *listCur = a.list[rc];
    const int32_t *listCurC = a.listC[rc];
    int32_t *listNext = a.list[rn];
    int32_t *listNextC = a.listC[rn];
    unsigned long long *cntNext = a.listCnt + rn;
    const unsigned long long lc = a.listCnt[rc];
    const long long nList = (long long)(lc >> 32);
    const long long eOut = (long long)(lc & 0xffffffffull);
    const bool push = a.pairMode || buckets || eOut * a.alpha <= (long long)a.nEdges;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.cnt[rn] = 0ull;
      a.listCnt[(r + 2) % 3] = 0ull;  // input of round r-1, appended in round r+1
    }
    if (!PAIRS)  // pair rounds clear their own mask words (batch_pair_unit)
      for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < maskWords;
           i += (size_t)gridDim.x * blockDim.x)
        clr[i] = 0u;
    unsigned long long changed = 0ull;
    if constexpr (PAIRS) {
      const uint32_t *pc = a.pairs[rc];
      uint32_t *pn = a.pairs[rn];
      const long long threads = (long long)gridDim.x * blockDim.x;
      for (long long base = gwl * 32; base < nList; base += threads) {
        const long long i = base + (threadIdx.x & 31);
        const bool valid = i < nList;
        batch_pair_unit<W, KIND>(a, valid, valid ? __ldcg(pc + i) : 0u, r, cur, nxt,
                                 pn, cntNext, changed, bk);
      }
    } else if (push) {
      for (long long i = gwl; i < nList; i += warps)
        batch_push_unit<W, KIND>(a, listCur[i], listCurC[i], r, cur, nxt, listNext, listNextC,
                                 cntNext, changed, bk);
    } else {
      for (long long u = gw; u < a.nUnits; u += warps)
        batch_unit<W, KIND>(a, (int)u, r, cur, nxt, changed);
    }
    (void)clr;
    changed = warp_sum_u64(changed);
    if ((threadIdx.x & 31) == 0 && changed) atomicAdd(a.cnt + rc, changed);
    if (buckets) {
      __syncthreads();
      if (threadIdx.x < W && sNear[threadIdx.x]) atomicOr(a.nearFlag[rc] + threadIdx.x, sNear[threadIdx.x]);
    }
    if (!grid_barrier(a.barrier, a.errWord)) break;
    if (a.cnt[rc] == 0ull) break;  // uniform: read after the barrier
    if (!PAIRS && !push) {
      batch_compact<W>(a, nxt, listNext, listNextC, cntNext);
      if (!grid_barrier(a.barrier, a.errWord)) break;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *a.roundsOut = r;
}

// value[V][Q] := BFS -1 / SSSP gatherZero; sources get 0 and their bit.
// thresh0 (may be null): every query's first bucket bound, delta.
static __global__ void batch_init_kernel(int kind, int32_t nVertices, int32_t Q, int32_t *value,
                                         int32_t *thresh0 = nullptr, int32_t delta = 0) {
  const size_t n = (size_t)nVertices * Q;
  const int32_t fill = kind == kBatchBFS ? -1 : kBatchInf;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    value[i] = fill;
  if (thresh0)
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < (size_t)Q;
         q += (size_t)gridDim.x * blockDim.x)
      thresh0[q] = delta;
}

// Sources: value 0, their query bit, and the first list (each source
// vertex once; inList was reset to -1).
// With a pair list (pairs0 non-null) the first list is (s_q, q) per query,
// and the state is query-major (value[q][v], mask and seen words [w][v]).
static __global__ void batch_sources_kernel(int kind, int32_t nQueries, int32_t Q, int32_t W,
                                            int32_t nVertices, const int32_t *sources, int32_t *value,
                                            unsigned *mask0, unsigned *seen,
                                            const int32_t *outOffsets, int32_t *inList,
                                            int32_t *list0, int32_t *list0C,
                                            unsigned long long *listCnt0,
                                            uint32_t *pairs0 = nullptr) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nQueries) return;
  const int s = sources[q];
  if (pairs0) {  // pair batches keep their state query-major
    value[(size_t)q * nVertices + s] = 0;
    atomicOr(mask0 + (size_t)(q / 32) * nVertices + s, 1u << (q % 32));
    if (kind == kBatchBFS) atomicOr(seen + (size_t)(q / 32) * nVertices + s, 1u << (q % 32));
  } else {
    value[(size_t)s * Q + q] = 0;
    atomicOr(mask0 + (size_t)s * W + q / 32, 1u << (q % 32));
    if (kind == kBatchBFS) atomicOr(seen + (size_t)s * W + q / 32, 1u << (q % 32));
  }
  if (pairs0) {
    const unsigned long long pos = atomicAdd(listCnt0, 1ull << 32) >> 32;
    pairs0[pos] = (uint32_t)s * (uint32_t)Q + (uint32_t)q;
    return;
  }
  if (atomicExch(inList + s, 0) != 0) {
    const unsigned d = (unsigned)(outOffsets[s + 1] - outOffsets[s]);
    const unsigned ne = d > 0u ? (d + kPushChunk - 1) / kPushChunk : 1u;
    const unsigned long long pos = atomicAdd(listCnt0, ((unsigned long long)ne << 32) | d) >> 32;
    for (unsigned c = 0; c < ne; ++c) {
      list0[pos + c] = s;
      list0C[pos + c] = (int32_t)c;
    }
  }
}

// out[q][v] = value[v][q] for q < nQueries (32x32 tiles through shared memory)
static __global__ void batch_transpose_kernel(const int32_t *value, int32_t nVertices, int32_t Q,
                                       int32_t nQueries, int32_t *out) {
  __shared__ int32_t tile[32][33];
  const int v0 = blockIdx.x * 32, q0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int v = v0 + j, q = q0 + threadIdx.x;
    tile[j][threadIdx.x] = (v < nVertices && q < Q) ? value[(size_t)v * Q + q] : 0;
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int q = q0 + j, v = v0 + threadIdx.x;
    if (q < nQueries && v < nVertices) out[(size_t)q * nVertices + v] = tile[threadIdx.x][j];
  }
}

}  // namespace detail
}  // namespace gas
