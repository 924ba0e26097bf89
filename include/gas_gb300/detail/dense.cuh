// Dense (pull) rounds of the GB300 GAS engine.
//
// When the vertices whose apply returned true in round r have many
// out-edges, round r+1 runs as one pass over every vertex's in-edges
// instead of push + compaction (the reference's dense path builds byte
// flags with IntervalGather and compacts them with a scan,
// gpugas.h:690-717, primitives/scatter_if_mgpu.h:130-157):
//
//   vertex v is active in round r+1  <=>  some in-neighbour u of v returned
//   true in round r  (bit u of round r's frontier bitmap)
//
// which is exactly the set the reference's scatterActivate builds, so the
// active sets and round counts are unchanged.  The frontier of a dense
// round is a bitmap of V bits (R-MAT-22: 512 KB, the reference keeps a byte
// per vertex, gpugas.h:115): the round of stamp S sets the bits of its
// apply-returned-true vertices in bitmap S % 3 (atomicOr, no return value),
// reads bitmap (S - 1) % 3, and clears bitmap (S + 1) % 3, which no round
// touches between its last read in round S - 1 and its first write in round
// S + 1; so no round waits for a clear.  The pass gathers speculatively,
// applies to the active vertices and writes every vertex's data to the
// other buffer of a ping-pong pair: no commit, no scatter traversal, no
// frontier list, one grid barrier per round.  A list round with a large
// frontier can run the same pass in mark mode: the active vertices are
// those the previous scatter marked, and the others gather nothing.
//
// Work units follow in-degree bins fixed per graph, each vertex owned by
// one warp work unit, with no block barriers and no waits; warps take the
// units heaviest first (dense_pass):
//   in-degree 0..8      one thread, edges folded left to right from
//                       gatherZero (the order of refgas.h:147-158);
//   in-degree 9..64     8 lanes, ordered shuffle tree;
//   in-degree 65..1024  one warp, ordered shuffle tree;
//   in-degree > 1024    1024-edge chunks, one warp each; the warp that
//                       finishes a vertex's last chunk (arrival counter)
//                       combines the partials in chunk order.
// Source ids (and 4-byte edge data) are read as 16-byte words: the lanes of
// a group take aligned quads of CSC positions, the one to three unaligned
// edges at either end of a vertex's range one per lane; a one-thread vertex
// reads the quads that cover its range.  Each vertex's reduction order
// depends only on its degree and CSC position, so results are identical
// run to run.
#pragma once

#include <cstring>

#include "gather.cuh"

namespace gas {
namespace detail {

struct DenseCtx {
  int32_t nVertices;
  int32_t nEdges;
  const int32_t *inOffsets;
  const int32_t *inSources;
  const int32_t *outOffsets;
  const void *edgeData;
  const void *vdCur;
  void *vdNext;
  const uint32_t *prevBits;  // frontier bitmap of the previous round (read only here)
  uint32_t *curBits;         // this round's apply-returned-true bits
  int32_t allActive;       // every vertex active (setActive(0, V))
  // Mark mode (a list round run as a pull pass): v is active iff
  // actMark[v] == markStamp (the previous round's scatter marks); inactive
  // vertices gather nothing.  Null: activity from the in-neighbours' bits.
  const int32_t *actMark;
  int32_t markStamp;
  // Active-set mode (a dense round after a fused round): v is active iff its
  // bit is set in actBits, the bitmap the fused round activated; the others
  // gather nothing.
  const uint32_t *actBits;
  int32_t skipBits;        // allActive, mark or active-set mode: no per-edge bitmap reads
  int32_t haveGather;
  int32_t iteration;
  unsigned long long *cnt;  // [3]: (active << 32 | in-edges), (ret << 32 | out-edges),
                            // work units taken (zero at the start of the pass)
  // degree bins, fixed per graph
  const int32_t *binMid;
  const int32_t *binSmall;
  const int32_t *binTiny;
  int32_t nMid, nSmall, nTiny;
  const int32_t *chunkVertex;
  const int32_t *chunkBegin;
  const int32_t *chunkFirst;
  const int32_t *chunkCount;
  const int32_t *chunkSlot;
  int32_t nChunks;
  unsigned *chunkArrive;
  void *chunkVal;
  unsigned *chunkFlags;
};

constexpr int kChunkEdges = 1024;  // edges per chunk of a large vertex
constexpr int kDenseCntStride = 4;  // counters per round (DenseCtx::cnt)
constexpr int kDenseGrab = 4;  // work units a warp takes at a time
constexpr int kSmallLanes = 8;     // lanes per vertex of in-degree 9..64

// Frontier bitmaps: bit v of word v / 32.  Bits written by other SMs in the
// previous round are read with plain loads after the grid barrier.
__device__ __forceinline__ bool bit_test(const uint32_t *bits, int v) {
  return (bits[v >> 5] >> (v & 31)) & 1u;
}
__device__ __forceinline__ void bit_set(uint32_t *bits, int v) {
  atomicOr(bits + (v >> 5), 1u << (v & 31));  // result unused: a reduction, no round trip
}
// Clears nWords words of a bitmap, grid-stride.
__device__ __forceinline__ void clear_bits(uint32_t *bits, int nWords) {
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nWords; i += stride) bits[i] = 0u;
}

// Per-lane accumulators of one edge stream: reduction, "has an edge",
// "some edge activates the vertex".
template <typename GR>
struct EdgeAcc {
  unsigned has;
  unsigned act;
  GR val;
};

// Edge data read by quads: 4-byte EdgeData (SSSP weights) comes with the
// source ids as one 16-byte word; other sizes are read edge by edge.
template <class P>
struct QuadEdgeData {
  typedef typename P::EdgeData ED;
  static constexpr bool value = !std::is_empty<ED>::value && sizeof(ED) == 4;
};

// One in-edge (source id src, edge data *ep) of vertex v.  known: the
// vertex is already known active, its activity bit is not read.
template <class P>
__device__ __forceinline__ void edge_acc(const DenseCtx &a, int v, int src,
                                         const typename P::EdgeData *ep, bool known,
                                         EdgeAcc<typename P::GatherResult> &x) {
  typedef typename P::VertexData VD;
  const VD *vd = reinterpret_cast<const VD *>(a.vdCur);
  x.act |= (known || bit_test(a.prevBits, src)) ? 1u : 0u;
  if (a.haveGather) {
    const typename P::GatherResult m = P::gatherMap(vd + v, vd + src, ep);
    x.val = x.has ? P::gatherReduce(x.val, m) : m;
  }
  x.has = 1u;
}

// The four in-edges at CSC positions [4q, 4q + 4): source ids (and 4-byte
// edge data) as 16-byte loads, activity bits and source data in flight
// together.
template <class P>
__device__ __forceinline__ void quad_acc(const DenseCtx &a, int v, int q, bool known,
                                         EdgeAcc<typename P::GatherResult> &x) {
  typedef typename P::EdgeData ED;
  const int4 s4 = __ldg(reinterpret_cast<const int4 *>(a.inSources) + q);
  const int src[4] = {s4.x, s4.y, s4.z, s4.w};
  if constexpr (QuadEdgeData<P>::value) {
    const int4 w4 = __ldg(reinterpret_cast<const int4 *>(a.edgeData) + q);
    const int w[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      ED e;
      memcpy(&e, &w[k], sizeof(ED));
      edge_acc<P>(a, v, src[k], &e, known, x);
    }
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) edge_acc<P>(a, v, src[k], edge_ptr<P>(a.edgeData, 4 * q + k), known, x);
  }
}

// Ordered tree combine of lane accumulators within aligned groups of
// `width` lanes; lane 0 of each group ends with the group's combination.
template <class P, int W>
__device__ __forceinline__ void group_reduce(EdgeAcc<typename P::GatherResult> &x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < W; d <<= 1) {
    const unsigned oh = __shfl_down_sync(kFullMask, x.has, d, W);
    const unsigned oa = __shfl_down_sync(kFullMask, x.act, d, W);
    const typename P::GatherResult ov = shfl_down_any_w(x.val, d, W);
    if ((lane & (2 * d - 1)) == 0) {
      x.act |= oa;
      if (oh) {
        x.val = x.has ? P::gatherReduce(x.val, ov) : ov;
        x.has = 1u;
      }
    }
  }
}

// The edges [beg, end) of vertex v walked by the W lanes of a group (sl:
// lane in the group): lanes 0..2 take the unaligned head [beg, 4*ceil(beg/4)),
// lanes 4..6 the unaligned tail, and aligned quads go round the group, one
// 16-byte load of source ids per lane and step (W = 32: 128 edges a step;
// once some lane has seen an activating in-neighbour the vertex is known
// active and no more activity bits are read).  W = 8 groups cover at most
// 64 edges: two steps.
template <class P, int W>
__device__ __forceinline__ void group_edges(const DenseCtx &a, int v, int beg, int end, int sl,
                                            EdgeAcc<typename P::GatherResult> &x) {
  const int qb = (beg + 3) >> 2, qe = end >> 2;
  const int hEnd = min(end, qb << 2);
  const int tBeg = max(qe << 2, hEnd);
  bool known = a.skipBits != 0;  // group-uniform
  if (sl < 3 && beg + sl < hEnd) {
    const int e = beg + sl;
    edge_acc<P>(a, v, __ldg(a.inSources + e), edge_ptr<P>(a.edgeData, e), known, x);
  }
  if (sl >= 4 && sl < 7 && tBeg + sl - 4 < end) {
    const int e = tBeg + sl - 4;
    edge_acc<P>(a, v, __ldg(a.inSources + e), edge_ptr<P>(a.edgeData, e), known, x);
  }
  if constexpr (W == 32) {
    known = known || __any_sync(kFullMask, x.act != 0u);
    for (int q0 = qb; q0 < qe; q0 += 32) {
      if (q0 + sl < qe) quad_acc<P>(a, v, q0 + sl, known, x);
      known = known || __any_sync(kFullMask, x.act != 0u);
    }
  } else {
    static_assert(W * 8 >= 64, "a group walks at most 64 edges in two steps");
#pragma unroll
    for (int k = 0; k < 2; ++k)
      if (qb + sl + W * k < qe) quad_acc<P>(a, v, qb + sl + W * k, known, x);
  }
}

struct DenseCounts {
  unsigned active, inEdges, ret, outEdges;
};

// Final gather result of a vertex from its combined (tree-ordered) state.
template <class P>
__device__ __forceinline__ typename P::GatherResult
combined_result(const DenseCtx &a, const EdgeAcc<typename P::GatherResult> &x) {
  const typename P::GatherResult gz = P::gatherZero;
  return (a.haveGather && x.has) ? P::gatherReduce(gz, x.val) : gz;
}

// apply() for vertex v; every vertex is written to vdNext.
template <class P>
__device__ __forceinline__ void dense_finish(const DenseCtx &a, int v, unsigned act,
                                             const typename P::GatherResult &g, int inDeg,
                                             DenseCounts &c) {
  typedef typename P::VertexData VD;
  const VD *vd = reinterpret_cast<const VD *>(a.vdCur);
  VD tmp = vd[v];
  if (a.allActive || (a.actMark ? a.actMark[v] == a.markStamp
                                 : (a.actBits ? bit_test(a.actBits, v) : act != 0u))) {
    const bool r = do_apply<P>(&tmp, g, a.iteration);
    ++c.active;
    c.inEdges += (unsigned)inDeg;
    if (r) {
      bit_set(a.curBits, v);
      ++c.ret;
      c.outEdges += (unsigned)(a.outOffsets[v + 1] - a.outOffsets[v]);
    }
  }
  reinterpret_cast<VD *>(a.vdNext)[v] = tmp;
}

// Mark or active-set mode: v is not active this round (its edges are
// skipped).
__device__ __forceinline__ bool mark_inactive(const DenseCtx &a, int v) {
  if (a.actMark) return a.actMark[v] != a.markStamp;
  return a.actBits != nullptr && !bit_test(a.actBits, v);
}

// Warp work units of one dense pass: [large-vertex chunks | one vertex per
// warp | 8-lane groups | one vertex per thread].
__device__ __forceinline__ long long dense_units(const DenseCtx &a) {
  return (long long)a.nChunks + a.nMid + (a.nSmall + 3) / 4 + (a.nTiny + 31) / 32;
}

template <class P>
__device__ void dense_warp_unit(const DenseCtx &a, long long u, DenseCounts &c) {
  typedef typename P::GatherResult GR;
  const int lane = threadIdx.x & 31;
  const GR gz = P::gatherZero;
  EdgeAcc<GR> x;
  x.has = 0u;
  x.act = 0u;
  x.val = gz;
  if (u < a.nChunks) {
    // ---- one chunk of a large vertex; the last chunk to finish combines
    const int ch = (int)u;
    const int v = a.chunkVertex[ch];
    const int beg = a.chunkBegin[ch];
    const int end = mark_inactive(a, v) ? beg : min(beg + kChunkEdges, a.inOffsets[v + 1]);
    group_edges<P, 32>(a, v, beg, end, lane, x);
    group_reduce<P, 32>(x);
    unsigned last = 0u;
    if (lane == 0) {
      if (x.has) reinterpret_cast<GR *>(a.chunkVal)[ch] = x.val;
      a.chunkFlags[ch] = x.has | (x.act << 1);
      __threadfence();
      const unsigned prev = atomicAdd(a.chunkArrive + a.chunkSlot[ch], 1u);
      last = (prev + 1 == (unsigned)a.chunkCount[ch]) ? 1u : 0u;
      if (last) __threadfence();
    }
    last = __shfl_sync(kFullMask, last, 0);
    if (!last) return;
    const int first = a.chunkFirst[ch], count = a.chunkCount[ch];
    EdgeAcc<GR> tot;
    tot.has = 0u;
    tot.act = 0u;
    tot.val = gz;
    for (int c0 = 0; c0 < count; c0 += 32) {
      EdgeAcc<GR> y;
      y.has = 0u;
      y.act = 0u;
      y.val = gz;
      if (c0 + lane < count) {
        const unsigned f = __ldcg(a.chunkFlags + first + c0 + lane);
        y.has = f & 1u;
        y.act = (f >> 1) & 1u;
        if (y.has) y.val = load_cg(reinterpret_cast<const GR *>(a.chunkVal) + first + c0 + lane);
      }
      group_reduce<P, 32>(y);
      if (lane == 0) {
        tot.act |= y.act;
        if (y.has) {
          tot.val = tot.has ? P::gatherReduce(tot.val, y.val) : y.val;
          tot.has = 1u;
        }
      }
    }
    if (lane == 0) {
      a.chunkArrive[a.chunkSlot[ch]] = 0u;  // ready for the next dense round
      dense_finish<P>(a, v, tot.act, combined_result<P>(a, tot), a.inOffsets[v + 1] - a.inOffsets[v], c);
    }
    return;
  }
  u -= a.nChunks;
  if (u < a.nMid) {
    // ---- one vertex per warp (in-degree 65..1024)
    const int v = a.binMid[u];
    const int beg = a.inOffsets[v], end = mark_inactive(a, v) ? beg : a.inOffsets[v + 1];
    group_edges<P, 32>(a, v, beg, end, lane, x);
    group_reduce<P, 32>(x);
    if (lane == 0) dense_finish<P>(a, v, x.act, combined_result<P>(a, x), end - beg, c);
    return;
  }
  u -= a.nMid;
  const long long smallGroups = (a.nSmall + 3) / 4;
  if (u < smallGroups) {
    // ---- one vertex per 8 lanes (in-degree 9..64)
    const long long idx = u * 4 + lane / kSmallLanes;
    const int sl = lane % kSmallLanes;
    int v = -1, beg = 0, end = 0;
    if (idx < a.nSmall) {
      v = a.binSmall[idx];
      beg = a.inOffsets[v];
      end = mark_inactive(a, v) ? beg : a.inOffsets[v + 1];
    }
    group_edges<P, kSmallLanes>(a, v, beg, end, sl, x);
    group_reduce<P, kSmallLanes>(x);
    if (sl == 0 && v >= 0) dense_finish<P>(a, v, x.act, combined_result<P>(a, x), end - beg, c);
    return;
  }
  u -= smallGroups;
  {
    // ---- one vertex per thread (in-degree 0..8), folded left to right
    // from gatherZero exactly as refgas.h:147-158
    const long long idx = u * 32 + lane;
    if (idx >= a.nTiny) return;
    const int v = a.binTiny[idx];
    const int beg = a.inOffsets[v], end = mark_inactive(a, v) ? beg : a.inOffsets[v + 1];
    typedef typename P::VertexData VD;
    const VD *vd = reinterpret_cast<const VD *>(a.vdCur);
    int src[GAS_TPV_MAX_DEGREE];
    load_window8(a.inSources, beg, end, src);
    GR g = gz;
    unsigned act = 0u;
#pragma unroll
    for (int k = 0; k < GAS_TPV_MAX_DEGREE; ++k)
      if (beg + k < end) {
        act |= (a.skipBits || bit_test(a.prevBits, src[k])) ? 1u : 0u;
        if (a.haveGather)
          g = P::gatherReduce(g, P::gatherMap(vd + v, vd + src[k], edge_ptr<P>(a.edgeData, beg + k)));
      }
    dense_finish<P>(a, v, act, g, end - beg, c);
  }
}

// Flushes the block's counts: one pair of atomics per block and pass (the
// caller's grid barrier follows).
__device__ __forceinline__ void dense_flush(const DenseCtx &a, const DenseCounts &c) {
  __shared__ unsigned long long sA[32], sR[32];
  const unsigned wA = __reduce_add_sync(kFullMask, c.active);
  const unsigned wEin = __reduce_add_sync(kFullMask, c.inEdges);
  const unsigned wR = __reduce_add_sync(kFullMask, c.ret);
  const unsigned wEout = __reduce_add_sync(kFullMask, c.outEdges);
  if ((threadIdx.x & 31) == 0) sR[threadIdx.x >> 5] = ((unsigned long long)wR << 32) | wEout;
  block_add_u64(((unsigned long long)wA << 32) | wEin, a.cnt, sA);
  if (threadIdx.x == 0) {
    unsigned long long s = 0ull;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sR[k];
    if (s) atomicAdd(a.cnt + 1, s);
  }
}

// One dense pass over every vertex, heaviest work units first (chunks, then
// the bins in descending in-degree).  The first kDenseGrab units of every
// warp are dealt round-robin; past them warps take kDenseGrab consecutive
// units at a time from a counter, so the pass ends on small units.
template <class P>
__device__ void dense_pass(const DenseCtx &a) {
  DenseCounts c = {0u, 0u, 0u, 0u};
  const unsigned long long units = (unsigned long long)dense_units(a);
  const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x / 32);
  const unsigned long long w = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
#pragma unroll 1
  for (int k = 0; k < kDenseGrab; ++k) {
    const unsigned long long u = w + k * warps;
    if (u >= units) break;
    dense_warp_unit<P>(a, (long long)u, c);
  }
  if (warps * kDenseGrab < units) {
    for (;;) {
      unsigned long long u0 = 0ull;
      if ((threadIdx.x & 31) == 0) u0 = warps * kDenseGrab + atomicAdd(a.cnt + 2, (unsigned long long)kDenseGrab);
      u0 = __shfl_sync(kFullMask, u0, 0);
      if (u0 >= units) break;
      const unsigned long long u1 = min(u0 + kDenseGrab, units);
      for (unsigned long long u = u0; u < u1; ++u) dense_warp_unit<P>(a, (long long)u, c);
    }
  }
  dense_flush(a, c);
}

// Dense -> list transition: the vertices whose bits this round set become
// the scatter list (out-degree prefix, CSR begin), in vertex order per block.
template <int NT, int KS>
__device__ void compact_ret(const uint32_t *bits, const int32_t *outOffsets,
                            int32_t nVertices, const gas_vertex_list &out, int32_t maxSplit,
                            unsigned *errWord, AppendSmem<NT, KS> &sm) {
  for (int base = blockIdx.x * NT; base < nVertices; base += gridDim.x * NT) {
    const int v = base + threadIdx.x;
    bool ok[1] = {false};
    int32_t ov[1] = {v}, od[1] = {0}, ob[1] = {0};
    if (v < nVertices && bit_test(bits, v)) {
      ok[0] = true;
      ob[0] = outOffsets[v];
      od[0] = outOffsets[v + 1] - ob[0];
    }
    block_append<NT, 1, GAS_SCATTER_TILE>(ok, ov, od, ob, out, maxSplit, nVertices, errWord, sm);
  }
}

// compact_ret as a kernel of its own (a frontier left as a bitmap by a run
// that stopped before a dense round, turned into a list when needed).
static __global__ void __launch_bounds__(256) compact_ret_kernel(const uint32_t *bits,
                                                                 const int32_t *outOffsets, int32_t nVertices,
                                                                 gas_vertex_list out, int32_t maxSplit,
                                                                 unsigned *errWord) {
  __shared__ AppendSmem<256, 1> sm;
  compact_ret<256, 1>(bits, outOffsets, nVertices, out, maxSplit, errWord, sm);
}

// List -> dense transition: the vertices of a scatter list into a bitmap.
__device__ __forceinline__ void bits_from_list(const gas_vertex_list &l, int n, uint32_t *bits) {
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) bit_set(bits, l.vid[i]);
}

}  // namespace detail
}  // namespace gas
