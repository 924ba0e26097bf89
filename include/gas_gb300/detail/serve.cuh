// Round-at-a-time kernels of the serving loop.
//
// A served batch (Q queries of one program on one resident graph) advances
// by ordinary launches, one or two per round, on the stream of its lane.
// No kernel here waits on another block, so batches on different lanes --
// different graphs, programs and sizes -- share the SMs freely and overlap;
// nothing depends on co-residency (unlike the persistent kernels, whose
// grid barriers need every block resident).
//
// BFS / SSSP reuse the batched units of batch.cuh: round r is
//   batch_round_kernel(r)  resets, push or pull pass, changed count
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
// of A(k) (apply always returns true).  Each (v, q) sum is a left fold from
// 0 in CSC order with correctly rounded float operations and no
// contraction, so every query's ranks equal a single-source run of the
// reference engine's CPU loop (refgas.h:140-166 with the program of
// pagerank.cu:27-73 and a teleport term) bit for bit, alone or in any mix.
#pragma once

#include "batch.cuh"

namespace gas {
namespace detail {

// ---------------------------------------------------------------- BFS/SSSP

template <int W, int KIND>
__global__ void __launch_bounds__(256) batch_round_kernel(const BatchArgs a, int r,
                                                          const unsigned *done) {
  if (ld_acquire(done)) return;
  __shared__ WarpStage stage[8];
  WarpStage &st = stage[threadIdx.x / 32];
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  const long long gw = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const size_t maskWords = (size_t)a.nVertices * W;
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
    a.listCnt[(r + 2) % 3] = 0ull;
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
  const bool push = (long long)(lc & 0xffffffffull) * a.alpha <= (long long)a.nEdges;
  if (push) return;
  __shared__ WarpStage stage[8];
  batch_compact<W>(a, a.mask[(r + 1) % 3], a.list[(r + 1) % 3], a.listCnt + (r + 1) % 3,
                   stage[threadIdx.x / 32]);
}

// ---------------------------------------------------------------- PPR

struct PprArgs {
  int32_t nVertices;
  int32_t nQueries;           // queries in the batch (<= Q = 32 * W)
  const int32_t *inOffsets;   // CSC
  const int32_t *inSources;
  const int32_t *outDegree;   // [V]
  const int32_t *order;       // [V] vertices by in-degree, largest first
  const int32_t *sources;     // [nQueries]
  float *rank[2];             // [V][Q]
  float *contrib[2];          // [V][Q] rank / outdeg (0 where outdeg is 0)
  unsigned char *active[2];   // [V] active set of the round
  float damp;                 // 1 - alpha, as the program computes it in float
  float teleport;             // alpha
};

__device__ __forceinline__ float ppr_contrib(float rank, int deg) {
  return deg > 0 ? __fdiv_rn(rank, (float)deg) : 0.0f;
}

// rank := 1 at each query's source, 0 elsewhere (pagerank-style init of a
// personalised run); every vertex active in round 0.
template <int W>
__global__ void ppr_init_kernel(const PprArgs a) {
  const int Q = 32 * W;
  const size_t n = (size_t)a.nVertices * Q;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    a.rank[0][i] = 0.0f;
    a.contrib[0][i] = 0.0f;
  }
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < (size_t)a.nVertices;
       v += (size_t)gridDim.x * blockDim.x)
    a.active[0][v] = 1;
}

template <int W>
__global__ void ppr_sources_kernel(const PprArgs a) {
  const int Q = 32 * W;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.nQueries) return;
  const int s = a.sources[q];
  a.rank[0][(size_t)s * Q + q] = 1.0f;
  a.contrib[0][(size_t)s * Q + q] = ppr_contrib(1.0f, a.outDegree[s]);
}

// Round r: reads rank/contrib/active[r & 1], writes [(r + 1) & 1].  A warp
// per vertex (taken in decreasing in-degree order), lane l owning queries
// l + 32k; in-edges are walked in CSC order, 32 source ids per coalesced
// load, each gathered row of contributions one 128-byte load per word.
template <int W>
__global__ void __launch_bounds__(256) ppr_round_kernel(const PprArgs a, int r) {
  const int Q = 32 * W;
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  const long long gw = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const bool odd = (r & 1) != 0;  // selects, not indexes (keeps the params out of local memory)
  const float *rk = odd ? a.rank[1] : a.rank[0];
  const float *ct = odd ? a.contrib[1] : a.contrib[0];
  const unsigned char *act = odd ? a.active[1] : a.active[0];
  float *rk2 = odd ? a.rank[0] : a.rank[1];
  float *ct2 = odd ? a.contrib[0] : a.contrib[1];
  unsigned char *act2 = odd ? a.active[0] : a.active[1];
  for (long long i = gw; i < a.nVertices; i += warps) {
    const int v = a.order[i];
    const int beg = a.inOffsets[v], end = a.inOffsets[v + 1];
    const bool isAct = act[v] != 0;
    float acc[W];
#pragma unroll
    for (int k = 0; k < W; ++k) acc[k] = 0.0f;
    unsigned anyAct = 0u;
    for (int e0 = beg; e0 < end; e0 += 32) {
      const int e = e0 + lane;
      const int s = e < end ? __ldg(a.inSources + e) : 0;
      anyAct |= __ballot_sync(kFullMask, e < end && act[s] != 0);
      if (!isAct) continue;  // warp-uniform
      const int n = min(32, end - e0);
      int j = 0;
      for (; j + 4 <= n; j += 4) {  // four rows in flight, folded in order
        float c[4][W];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int sj = __shfl_sync(kFullMask, s, j + t);
#pragma unroll
          for (int k = 0; k < W; ++k) c[t][k] = __ldcg(ct + (size_t)sj * Q + k * 32 + lane);
        }
#pragma unroll
        for (int t = 0; t < 4; ++t)
#pragma unroll
          for (int k = 0; k < W; ++k) acc[k] = __fadd_rn(acc[k], c[t][k]);
      }
      for (; j < n; ++j) {
        const int sj = __shfl_sync(kFullMask, s, j);
#pragma unroll
        for (int k = 0; k < W; ++k)
          acc[k] = __fadd_rn(acc[k], __ldcg(ct + (size_t)sj * Q + k * 32 + lane));
      }
    }
    if (lane == 0) act2[v] = anyAct != 0u;
    const int deg = a.outDegree[v];
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const int q = k * 32 + lane;
      const size_t idx = (size_t)v * Q + q;
      if (isAct) {
        const float tele = (q < a.nQueries && a.sources[q] == v) ? a.teleport : 0.0f;
        const float nr = __fadd_rn(tele, __fmul_rn(a.damp, acc[k]));
        rk2[idx] = nr;
        ct2[idx] = ppr_contrib(nr, deg);
      } else {
        rk2[idx] = __ldcg(rk + idx);
        ct2[idx] = __ldcg(ct + idx);
      }
    }
  }
}

}  // namespace detail
}  // namespace gas
