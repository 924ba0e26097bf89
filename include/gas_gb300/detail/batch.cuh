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
//   push  (E_out * alpha <= E): one warp per listed vertex u walks its
//         out-edges and updates the destinations for u's changed queries
//         with atomics; destinations that change are appended to the next
//         list (per-warp shared-memory staging, one atomic per 32 entries);
//   pull  otherwise: one pass over work units (a vertex's in-edges, split
//         into chunks of at most `chunk` edges for high in-degree vertices)
//         followed by a compaction of the changed vertices into the list.
// In both, lanes map to queries (lane l owns queries l + 32k):
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
  int32_t *list[3];           // [V] vertices with a changed query (rotating)
  unsigned long long *listCnt;  // [3] (count << 32) | out-degree total
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
};

constexpr int32_t kBatchInf = 0x7fffffff - 100000;  // SSSP gatherZero (sssp.cu:32-33)

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

// Per-warp staging of list appends in shared memory (warp-uniform calls).
struct WarpStage {
  int32_t v[32];
  int32_t d[32];
};

__device__ __forceinline__ void stage_flush(WarpStage &st, int &n, int32_t *list,
                                            unsigned long long *cnt) {
  if (n == 0) return;
  const int lane = threadIdx.x & 31;
  __syncwarp();
  unsigned dsum = lane < n ? (unsigned)st.d[lane] : 0u;
  dsum = __reduce_add_sync(kFullMask, dsum);
  unsigned long long base = 0ull;
  if (lane == 0) base = atomicAdd(cnt, ((unsigned long long)n << 32) | dsum);
  base = __shfl_sync(kFullMask, base, 0);
  if (lane < n) list[(base >> 32) + lane] = st.v[lane];
  __syncwarp();
  n = 0;
}

__device__ __forceinline__ void stage_push(WarpStage &st, int &n, int v, int deg, int32_t *list,
                                           unsigned long long *cnt) {
  if ((threadIdx.x & 31) == 0) {
    st.v[n] = v;
    st.d[n] = deg;
  }
  if (++n == 32) stage_flush(st, n, list, cnt);
}

// Push round: warp per listed vertex u, over u's out-edges.
template <int W, int KIND>
__device__ __forceinline__ void batch_push_unit(const BatchArgs &a, int u, int round,
                                                const unsigned *cur, unsigned *nxt,
                                                int32_t *listNext, unsigned long long *cntNext,
                                                WarpStage &st, int &stn,
                                                unsigned long long &changed) {
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
  const int eb = a.outOffsets[u], ee = a.outOffsets[u + 1];
  for (int e = eb; e < ee; ++e) {
    const int v = __ldg(a.outDests + e);
    unsigned any = 0u;
    if (KIND == kBatchSSSP) {
      const int w = __ldg(a.weightsOut + e);
#pragma unroll
      for (int k = 0; k < W; ++k) {
        bool imp = false;
        if ((m[k] >> lane) & 1u) {
          const int cand = du[k] + w;
          const int old = atomicMin(a.value + (size_t)v * Q + k * 32 + lane, cand);
          imp = cand < old;
        }
        const unsigned word = __ballot_sync(kFullMask, imp);
        if (word) {
          if (lane == 0) atomicOr(nxt + (size_t)v * W + k, word);
          any |= word;
          if (lane == 0) changed += __popc(word);
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < W; ++k) {
        if (!m[k]) continue;  // warp-uniform
        unsigned fresh = 0u;
        if (lane == 0) {
          const unsigned old = atomicOr(a.seen + (size_t)v * W + k, m[k]);
          fresh = m[k] & ~old;
          if (fresh) atomicOr(nxt + (size_t)v * W + k, fresh);
        }
        fresh = __shfl_sync(kFullMask, fresh, 0);
        if ((fresh >> lane) & 1u) a.value[(size_t)v * Q + k * 32 + lane] = round + 1;
        if (lane == 0) changed += __popc(fresh);
        any |= fresh;
      }
    }
    if (any) {  // warp-uniform
      int first = 0;
      if (lane == 0) first = atomicExch(a.inList + v, round + 1) != round + 1;
      first = __shfl_sync(kFullMask, first, 0);
      if (first)
        stage_push(st, stn, v, a.outOffsets[v + 1] - a.outOffsets[v], listNext, cntNext);
    }
  }
}

// After a pull round: list the vertices with a changed query.
template <int W>
__device__ __forceinline__ void batch_compact(const BatchArgs &a, const unsigned *nxt,
                                              int32_t *listNext, unsigned long long *cntNext,
                                              WarpStage &st) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  const long long gw = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  int stn = 0;
  for (long long base = gw * 32; base < a.nVertices; base += warps * 32) {
    const long long v = base + lane;
    unsigned any = 0u;
    if (v < a.nVertices) {
#pragma unroll
      for (int k = 0; k < W; ++k) any |= __ldcg(nxt + (size_t)v * W + k);
    }
    const unsigned who = __ballot_sync(kFullMask, any != 0u);
    const int n = __popc(who);
    if (n == 0) continue;
    // stage this group's changed vertices (at most 32) in one flush
    stage_flush(st, stn, listNext, cntNext);
    const int pos = __popc(who & ((1u << lane) - 1u));
    if (any) {
      st.v[pos] = (int32_t)v;
      st.d[pos] = a.outOffsets[v + 1] - a.outOffsets[v];
    }
    stn = n;
    stage_flush(st, stn, listNext, cntNext);
  }
}

template <int W, int KIND>
__global__ void __launch_bounds__(256) batch_run_kernel(const BatchArgs a) {
  __shared__ WarpStage stage[8];
  WarpStage &st = stage[threadIdx.x / 32];
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  const long long gw = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const size_t maskWords = (size_t)a.nVertices * W;
  int r = 0;
  for (;; ++r) {
    if (a.maxRounds > 0 && r >= a.maxRounds) break;
    const unsigned *cur = a.mask[r % 3];
    unsigned *nxt = a.mask[(r + 1) % 3];
    unsigned *clr = a.mask[(r + 2) % 3];
    const int32_t *listCur = a.list[r % 3];
    int32_t *listNext = a.list[(r + 1) % 3];
    unsigned long long *cntNext = a.listCnt + (r + 1) % 3;
    const unsigned long long lc = a.listCnt[r % 3];
    const int nList = (int)(lc >> 32);
    const long long eOut = (long long)(lc & 0xffffffffull);
    const bool push = eOut * a.alpha <= (long long)a.nEdges;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.cnt[(r + 1) % 3] = 0ull;
      a.listCnt[(r + 2) % 3] = 0ull;  // input of round r-1, appended in round r+1
    }
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < maskWords;
         i += (size_t)gridDim.x * blockDim.x)
      clr[i] = 0u;
    unsigned long long changed = 0ull;
    if (push) {
      int stn = 0;
      for (long long i = gw; i < nList; i += warps)
        batch_push_unit<W, KIND>(a, listCur[i], r, cur, nxt, listNext, cntNext, st, stn, changed);
      stage_flush(st, stn, listNext, cntNext);
    } else {
      for (long long u = gw; u < a.nUnits; u += warps)
        batch_unit<W, KIND>(a, (int)u, r, cur, nxt, changed);
    }
    if ((threadIdx.x & 31) == 0 && changed) atomicAdd(a.cnt + (r % 3), changed);
    if (!grid_barrier(a.barrier, a.errWord)) break;
    if (a.cnt[r % 3] == 0ull) break;  // uniform: read after the barrier
    if (!push) {
      batch_compact<W>(a, nxt, listNext, cntNext, st);
      if (!grid_barrier(a.barrier, a.errWord)) break;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *a.roundsOut = r;
}

// value[V][Q] := BFS -1 / SSSP gatherZero; sources get 0 and their bit.
static __global__ void batch_init_kernel(int kind, int32_t nVertices, int32_t Q, int32_t *value) {
  const size_t n = (size_t)nVertices * Q;
  const int32_t fill = kind == kBatchBFS ? -1 : kBatchInf;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    value[i] = fill;
}

// Sources: value 0, their query bit, and the first list (each source
// vertex once; inList was reset to -1).
static __global__ void batch_sources_kernel(int kind, int32_t nQueries, int32_t Q, int32_t W,
                                            const int32_t *sources, int32_t *value,
                                            unsigned *mask0, unsigned *seen,
                                            const int32_t *outOffsets, int32_t *inList,
                                            int32_t *list0, unsigned long long *listCnt0) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nQueries) return;
  const int s = sources[q];
  value[(size_t)s * Q + q] = 0;
  atomicOr(mask0 + (size_t)s * W + q / 32, 1u << (q % 32));
  if (kind == kBatchBFS) atomicOr(seen + (size_t)s * W + q / 32, 1u << (q % 32));
  if (atomicExch(inList + s, 0) != 0) {
    const unsigned d = (unsigned)(outOffsets[s + 1] - outOffsets[s]);
    const unsigned long long pos = atomicAdd(listCnt0, (1ull << 32) | d);
    list0[pos >> 32] = s;
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
