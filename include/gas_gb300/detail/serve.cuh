// Round-at-a-time kernels of the serving loop.
//
// A served batch (Q queries of one program on one resident graph) advances
// by ordinary launches, one or two per round, on the stream of its lane.
// No kernel here waits on another block, so batches on different lanes --
// different graphs, programs and sizes -- share the SMs freely and overlap;
// nothing depends on co-residency (unlike the persistent kernels, whose
// grid barriers need every block resident).
//
// BFS / SSSP reuse the batched units of batch.cuh (the (vertex, query) pair
// frontier and SSSP distance buckets included): round r is
//   batch_round_kernel(r)  bounds, resets, pair / push / pull pass, count
//   batch_tail_kernel(r)   end test (sets done, rounds) or compaction
// and both return at once when the batch is done, so the host may queue
// rounds ahead of the end test.
//
// Personalised PageRank (PPR, alpha 0.15, teleport to the source) runs
// every query of a batch in lock step, pulling over in-edges:
//   rank'[v][q] = tele(v,q) + (1-alpha) * (sum over in-edges u->v, in CSC
//                 order, of rank[u][q] / outdeg(u))      for active v
//   rank'[v][q] = rank[v][q]                              otherwise
// with the engine's active sets A0 = every vertex, A(k+1) = out-neighbours
// of A(k) (apply always returns true).  Sums use correctly rounded float
// operations without contraction; for vertices of in-degree <= kPprChunk
// each is the left fold from 0 in CSC order, so those ranks equal a
// single-source run of the reference engine's CPU loop (refgas.h:140-166
// with the program of pagerank.cu:27-73 and a teleport term) bit for bit.
// Every sum depends on the graph alone: a query's ranks are the same in
// every batch and mix.
#pragma once

#include "batch.cuh"

namespace gas {
namespace detail {

// ---------------------------------------------------------------- BFS/SSSP

template <int W, int KIND>
__global__ void __launch_bounds__(256) batch_round_kernel(const BatchArgs a, int r,
                                                          const unsigned *done) {
  if (ld_acquire(done)) return;
  __shared__ int32_t sBound[32 * W];
  __shared__ unsigned sNear[W];
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  const long long gw = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  // list entries are dealt to warps block-first (warp k of every block, then
  // warp k+1), so a short list spreads over every SM
  const long long gwl = (long long)(threadIdx.x / 32) * gridDim.x + blockIdx.x;
  const size_t maskWords = (size_t)a.nVertices * W;
  const int rc = r % 3, rn = (r + 1) % 3;
  const bool buckets = KIND == kBatchSSSP && a.delta > 0;
  const BatchBucket bk{buckets ? sBound : nullptr, buckets ? sNear : nullptr};
  if (buckets) {  // this round's bounds (as in batch_run_kernel)
    const int32_t *tPrev = (r & 1) ? a.thresh[1] : a.thresh[0];
    int32_t *tNext = (r & 1) ? a.thresh[0] : a.thresh[1];
    const unsigned *nPrev = a.nearFlag[(r + 2) % 3];
    for (int q = threadIdx.x; q < 32 * W; q += blockDim.x) {
      int32_t t = __ldcg(tPrev + q);
      if (r > 0 && !((__ldcg(nPrev + q / 32) >> (q % 32)) & 1u)) t += a.delta;
      sBound[q] = t;
      if (blockIdx.x == 0) tNext[q] = t;
    }
    if (threadIdx.x < W) sNear[threadIdx.x] = 0u;
    if (blockIdx.x == 0 && threadIdx.x < W) a.nearFlag[rn][threadIdx.x] = 0u;
    __syncthreads();
  }
  unsigned *cur = a.mask[rc];
  unsigned *nxt = a.mask[rn];
  unsigned *clr = a.mask[(r + 2) % 3];
  const unsigned long long lc = a.listCnt[rc];
  const long long nList = (long long)(lc >> 32);
  const long long eOut = (long long)(lc & 0xffffffffull);
  const bool push = a.pairMode || buckets || eOut * a.alpha <= (long long)a.nEdges;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.cnt[rn] = 0ull;
    a.listCnt[(r + 2) % 3] = 0ull;
  }
  if (!a.pairMode)  // pair rounds clear their own mask words (batch_pair_unit)
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < maskWords;
         i += (size_t)gridDim.x * blockDim.x)
      clr[i] = 0u;
  unsigned long long changed = 0ull;
  if (a.pairMode) {
    const uint32_t *pc = a.pairs[rc];
    uint32_t *pn = a.pairs[rn];
    const long long threads = (long long)gridDim.x * blockDim.x;
    for (long long base = gwl * 32; base < nList; base += threads) {
      const long long i = base + (threadIdx.x & 31);
      const bool valid = i < nList;
      batch_pair_unit<W, KIND>(a, valid, valid ? __ldcg(pc + i) : 0u, r, cur, nxt,
                               pn, a.listCnt + rn, changed, bk);
    }
  } else if (push) {
    for (long long i = gwl; i < nList; i += warps)
      batch_push_unit<W, KIND>(a, a.list[rc][i], a.listC[rc][i], r, cur, nxt, a.list[rn],
                               a.listC[rn], a.listCnt + rn, changed, bk);
  } else {
    for (long long u = gw; u < a.nUnits; u += warps)
      batch_unit<W, KIND>(a, (int)u, r, cur, nxt, changed);
  }
  changed = warp_sum_u64(changed);
  if ((threadIdx.x & 31) == 0 && changed) atomicAdd(a.cnt + rc, changed);
  if (buckets) {
    __syncthreads();
    if (threadIdx.x < W && sNear[threadIdx.x]) atomicOr(a.nearFlag[rc] + threadIdx.x, sNear[threadIdx.x]);
  }
}

// End of round r: no change -> done (rounds = r, as the persistent kernel
// reports); a pull round -> list its changed vertices for round r + 1.
template <int W>
__global__ void __launch_bounds__(256) batch_tail_kernel(const BatchArgs a, int r,
                                                         unsigned *done) {
  if (ld_acquire(done)) return;
  if (a.cnt[r % 3] == 0ull) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      *a.roundsOut = r;
      st_release(done, 1u);
    }
    return;
  }
  const unsigned long long lc = a.listCnt[r % 3];
  const bool push = a.pairMode || a.delta > 0 ||
                    (long long)(lc & 0xffffffffull) * a.alpha <= (long long)a.nEdges;
  if (push) return;
  const int rn = (r + 1) % 3;
  batch_compact<W>(a, a.mask[rn], a.list[rn], a.listC[rn], a.listCnt + rn);
}

// ---------------------------------------------------------------- PPR

// A vertex's in-edges form one work unit, or -- above kPprChunk edges --
// several units of kPprChunk edges whose partial sums the last unit to
// finish adds in chunk order.  Each (vertex, query) value is therefore a
// left fold in CSC order (bit for bit the reference loop's FP32 sum) for
// every vertex of in-degree <= kPprChunk, and a fixed-order sum of left-
// folded chunks above it: either way a function of the graph alone, the
// same in every batch.
constexpr int kPprChunk = 4096;

struct PprArgs {
  int32_t nVertices;
  int32_t nQueries;           // queries in the batch (<= the row width QP)
  const int32_t *inSources;   // CSC
  const int32_t *outDegree;   // [V]
  const uint8_t *lastActive;  // [V] last round in which the vertex is active
  int32_t nUnits;             // work units, longest first
  const int32_t *unitV;
  const int32_t *unitBeg;
  const int32_t *unitLen;
  const int32_t *unitSlot;    // -1, or the unit's partial-sum slot (hubs)
  const int32_t *slotFirst;   // [slots] first slot of the slot's vertex
  const int32_t *slotCount;   // [slots] chunks of that vertex
  const int32_t *slotHub;     // [slots] hub index (arrival counter)
  float *partial;             // [slots][QP] (per batch)
  unsigned *arrive;           // [hubs] arrivals, never reset within a batch
  const int32_t *sources;     // [nQueries]
  float *rank[2];             // [V][QP]
  float *contrib[2];          // [V][QP] rank / outdeg (0 where outdeg is 0)
  float damp;                 // 1 - alpha, as the program computes it in float
  float teleport;             // alpha
};

// The graph part of PprArgs, from a graph's PPR arrays (the work-unit block
// `mem` holds unitV | unitBeg | unitLen | unitSlot | slotFirst | slotCount |
// slotHub, `units` and `slots` entries long).
inline void ppr_args_graph(PprArgs &a, const int32_t *inSources, const int32_t *outDegree,
                           const uint8_t *lastActive, const int32_t *mem, int32_t units,
                           int32_t slots) {
  const size_t nu = (size_t)(units > 0 ? units : 1), ns = (size_t)(slots > 0 ? slots : 1);
  a.inSources = inSources;
  a.outDegree = outDegree;
  a.lastActive = lastActive;
  a.nUnits = units;
  a.unitV = mem;
  a.unitBeg = a.unitV + nu;
  a.unitLen = a.unitBeg + nu;
  a.unitSlot = a.unitLen + nu;
  a.slotFirst = a.unitSlot + nu;
  a.slotCount = a.slotFirst + ns;
  a.slotHub = a.slotCount + ns;
}

__device__ __forceinline__ float ppr_contrib(float rank, int deg) {
  return deg > 0 ? __fdiv_rn(rank, (float)deg) : 0.0f;
}

// The engine's active sets do not depend on the source: A0 = every vertex,
// A(k+1) = out-neighbours of A(k).  v is in A(k) iff a walk of length k
// ends at v, so membership only shrinks with k: lastActive[v] = the largest
// such k (capped).  One pull step per launch: nxt = out-neighbours of cur.
static __global__ void ppr_active_step_kernel(int32_t nVertices, const int32_t *inOffsets,
                                              const int32_t *inSources, const uint8_t *cur,
                                              uint8_t *nxt, uint8_t *lastActive, int k) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  for (long long v = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
       v < nVertices; v += warps) {
    const int beg = inOffsets[v], end = inOffsets[v + 1];
    bool any = false;
    for (int e = beg + lane; e < end && !any; e += 32) any = cur[inSources[e]] != 0;
    any = __any_sync(kFullMask, any);
    if (lane == 0) {
      nxt[v] = any;
      if (any) lastActive[v] = (uint8_t)k;
    }
  }
}

// Row width QP (queries per vertex row, a power of two 1..256) and how a
// warp covers it: L lanes per unit (L = min(QP, 32)), G = 32 / L units per
// warp, W = QP / L words of queries per lane (query of lane j, word k:
// k * L + j), D edges gathered per step (their loads all in flight), M
// source ids loaded per lane per step.
template <int QP>
struct PprShape {
  static constexpr int L = QP < 32 ? QP : 32;
  static constexpr int G = 32 / L;
  static constexpr int W = QP / L;
  static constexpr int D = W == 1 ? 32 : 32 / W;
  static constexpr int M = D > L ? D / L : 1;
};

// rank := 1 at each query's source, 0 elsewhere (pagerank-style init of a
// personalised run).
template <int QP>
__global__ void ppr_init_kernel(const PprArgs a) {
  const size_t n = (size_t)a.nVertices * QP;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    a.rank[0][i] = 0.0f;
    a.contrib[0][i] = 0.0f;
  }
}

template <int QP>
__global__ void ppr_sources_kernel(const PprArgs a) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.nQueries) return;
  const int s = a.sources[q];
  a.rank[0][(size_t)s * QP + q] = 1.0f;
  a.contrib[0][(size_t)s * QP + q] = ppr_contrib(1.0f, a.outDegree[s]);
}

// Round r: reads rank/contrib[r & 1], writes [(r + 1) & 1].  Groups of L
// lanes take units longest first (the G groups of a warp get neighbouring
// units, so similar lengths); a group loads D source ids per step (M per
// lane, coalesced), issues the D gathered rows' loads, then each lane folds
// its queries' D values in edge order.
template <int QP>
__device__ __forceinline__ void ppr_round(const PprArgs &a, int r) {
  using S = PprShape<QP>;
  constexpr int L = S::L, G = S::G, W = S::W, D = S::D, M = S::M;
  const int lane = threadIdx.x & 31;
  const int grp = lane / L, j = lane % L;
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  const long long gw = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const bool odd = (r & 1) != 0;  // selects, not indexes (keeps the params out of local memory)
  const float *rk = odd ? a.rank[1] : a.rank[0];
  const float *ct = odd ? a.contrib[1] : a.contrib[0];
  float *rk2 = odd ? a.rank[0] : a.rank[1];
  float *ct2 = odd ? a.contrib[0] : a.contrib[1];
  for (long long base = gw * G; base < a.nUnits; base += warps * G) {
    const long long u = base + grp;
    const bool valid = u < a.nUnits;
    const int v = valid ? a.unitV[u] : 0;
    const int beg = valid ? a.unitBeg[u] : 0;
    const int len = valid ? a.unitLen[u] : 0;
    const bool isAct = valid && (int)a.lastActive[v] >= r;
    const int maxLen = __reduce_max_sync(kFullMask, isAct ? len : 0);
    float acc[W];
#pragma unroll
    for (int k = 0; k < W; ++k) acc[k] = 0.0f;
    for (int o = 0; o < maxLen; o += D) {  // warp-uniform trip count
      int ids[M];
#pragma unroll
      for (int m = 0; m < M; ++m) {
        const int t = m * L + j;
        ids[m] = (t < D && o + t < len) ? __ldg(a.inSources + beg + o + t) : 0;
      }
      const int n = isAct ? min(D, len - o) : 0;  // this group's edges in the step
      float c[D][W];
#pragma unroll
      for (int t = 0; t < D; ++t) {
        const int sj = __shfl_sync(kFullMask, ids[t / L], t % L, L);
#pragma unroll
        for (int k = 0; k < W; ++k)
          c[t][k] = t < n ? __ldcg(ct + (size_t)sj * QP + k * L + j) : 0.0f;
      }
#pragma unroll
      for (int t = 0; t < D; ++t)
#pragma unroll
        for (int k = 0; k < W; ++k)
          if (t < n) acc[k] = __fadd_rn(acc[k], c[t][k]);
    }
    // hub chunks: publish the partial sums; the last chunk to arrive adds
    // them in chunk order and finishes the vertex
    const int slot = valid ? a.unitSlot[u] : -1;
    unsigned arrived = 0u;
    if (slot >= 0) {
#pragma unroll
      for (int k = 0; k < W; ++k) a.partial[(size_t)slot * QP + k * L + j] = acc[k];
      __threadfence();
      __syncwarp(L == 32 ? kFullMask : (((1u << L) - 1u) << (grp * L)));
      if (j == 0) {
        const unsigned old = atomicAdd(a.arrive + a.slotHub[slot], 1u);
        arrived = (old + 1u) % (unsigned)a.slotCount[slot] == 0u ? 1u : 0u;
      }
    }
    const unsigned last = __shfl_sync(kFullMask, arrived, grp * L);
    if (!valid || (slot >= 0 && !last)) continue;
    if (slot >= 0) {
      __threadfence();
      const int first = a.slotFirst[slot], cnt = a.slotCount[slot];
#pragma unroll
      for (int k = 0; k < W; ++k) {
        float sum = 0.0f;
        for (int c = 0; c < cnt; ++c)
          sum = __fadd_rn(sum, __ldcg(a.partial + (size_t)(first + c) * QP + k * L + j));
        acc[k] = sum;
      }
    }
    const int odeg = a.outDegree[v];
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const int q = k * L + j;
      const size_t idx = (size_t)v * QP + q;
      if (isAct) {
        const float tele = (q < a.nQueries && a.sources[q] == v) ? a.teleport : 0.0f;
        const float nr = __fadd_rn(tele, __fmul_rn(a.damp, acc[k]));
        rk2[idx] = nr;
        ct2[idx] = ppr_contrib(nr, odeg);
      } else {
        rk2[idx] = __ldcg(rk + idx);
        ct2[idx] = __ldcg(ct + idx);
      }
    }
  }
}

template <int QP>
__global__ void __launch_bounds__(256) ppr_round_kernel(const PprArgs a, int r) {
  ppr_round<QP>(a, r);
}

// Every round of a PPR batch in one cooperative launch (the batched engine,
// gas_batch_run): the served round body, rounds separated by bounded grid
// barriers.  *roundsOut receives the rounds completed.
template <int QP>
__global__ void __launch_bounds__(256) ppr_run_kernel(const PprArgs a, int rounds, unsigned *barrier,
                                                      unsigned *errWord, int32_t *roundsOut) {
  int r = 0;
  for (; r < rounds; ++r) {
    ppr_round<QP>(a, r);
    if (!grid_barrier(barrier, errWord)) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *roundsOut = r;
}

}  // namespace detail
}  // namespace gas
