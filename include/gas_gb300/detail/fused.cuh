// Fused list rounds for graphs whose in- and out-degrees are all <= 8
// (lattices, road networks): a thread per frontier vertex gathers, applies
// and activates its out-neighbours in one phase, so a round costs one grid
// barrier instead of two (gather -> barrier -> commit + scatter ->
// barrier).
//
// Bulk-synchronous reads without a commit step: for the fused rounds of a
// run, vertex data moves into cells, one per vertex,
//   { value slot 0, value slot 1, ver = (round stamp << 1) | newest slot },
// 16-byte aligned so that one vector load reads a whole cell.  A vertex
// applied in round S writes the slot it is not in and publishes (S, that
// slot).  Every read in round S wants the value as of the end of round S-1:
// when v's word already says S, that is the other slot (which the writer
// never touches in round S), otherwise the slot in the word -- so readers
// need no ordering against the writer.  Active sets, round counts and
// results are those of the two-phase rounds; the newest values go back to
// the vertex data array before a dense or two-phase round and at the end of
// the run.
#pragma once

#include "gather.cuh"
#include "scatter.cuh"

namespace gas {
namespace detail {

template <class VD>
struct alignas(16) FusedCell {
  VD s[2];
  uint32_t ver;
};


struct FusedCtx {
  void *cells;          // [V] FusedCell<VD> (Programs with a gather)
  void *vd;             // the run's vertex data (apply-only Programs update it in place)
  uint32_t stamp;       // this round's stamp
  int32_t *retStamp;    // [V] stamp of the round whose apply returned true
};

// One cell, read from L2 (written by other CTAs) with 16-byte loads.
template <class VD>
__device__ __forceinline__ FusedCell<VD> load_cell(const FusedCell<VD> *p) {
  static_assert(sizeof(FusedCell<VD>) % 16 == 0, "cells are whole 16-byte words");
  constexpr int N = (int)(sizeof(FusedCell<VD>) / 16);
  union {
    int4 w[N];
    FusedCell<VD> c;
  } u;
#pragma unroll
  for (int k = 0; k < N; ++k) u.w[k] = __ldcg(reinterpret_cast<const int4 *>(p) + k);
  return u.c;
}

// v's value as of the end of the previous round.
template <class VD>
__device__ __forceinline__ VD fused_read(const FusedCtx &f, int v) {
  const FusedCell<VD> c = load_cell(reinterpret_cast<const FusedCell<VD> *>(f.cells) + v);
  const uint32_t s = ((c.ver >> 1) == f.stamp) ? (1u - (c.ver & 1u)) : (c.ver & 1u);
  return s ? c.s[1] : c.s[0];
}

// Every vertex's value into slot 0 of its cell, version 0 (before the first
// fused round of a run; a grid barrier follows).
template <class P>
__device__ void fused_enter(const FusedCtx &f, const void *vd, int nVertices) {
  typedef typename P::VertexData VD;
  // the library allocates GAS_FUSED_CELL_BYTES(sizeof(VertexData)) per vertex
  static_assert(sizeof(FusedCell<VD>) == GAS_FUSED_CELL_BYTES(sizeof(VD)),
                "VertexData alignment above 16 bytes");
  FusedCell<VD> *cells = reinterpret_cast<FusedCell<VD> *>(f.cells);
  const int stride = gridDim.x * blockDim.x;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nVertices; v += stride) {
    cells[v].s[0] = reinterpret_cast<const VD *>(vd)[v];
    cells[v].ver = 0u;
  }
}

// Frontiers of at most this many vertices append per warp (one atomic per
// warp, no block barrier); larger ones per block (one atomic per block, two
// block barriers).
constexpr int kWarpAppendMax = 16384;

// Frontier entry i (none when i >= n) for this thread.  Counts this round's
// apply-returned-true vertices and their out-edges into cRet / cOut.
// warpAppend (block-uniform): append the activated vertices per warp.
// Every thread of the block calls it (the appends are collective).
template <class P>
__device__ __forceinline__ void fused_tpv_tile(const gas_gather_args &a, const ScatterArgs &sa, const FusedCtx &f,
                               int i, int n, int T, bool warpAppend, unsigned &cRet, unsigned &cOut) {
  typedef typename P::VertexData VD;
  typedef typename P::GatherResult GR;
  constexpr int D = GAS_TPV_MAX_DEGREE;
  bool isEdge[D];
  int32_t dst[D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    isEdge[k] = false;
    dst[k] = 0;
  }
  if (i < n) {
    int v, pre, end, beg;
    front_entry(a, i, n, T, v, pre, end, beg);
    const int deg = end - pre;
    const int obeg = a.outOffsets[v], oend = a.outOffsets[v + 1];
    FusedCell<VD> *cell = reinterpret_cast<FusedCell<VD> *>(f.cells) + v;
    int own = 0;
    VD tmp;
    if (a.haveGather) {
      const FusedCell<VD> c = load_cell(cell);
      own = (int)(c.ver & 1u);  // v is applied once per round: its word is still old
      tmp = own ? c.s[1] : c.s[0];
    } else {
      tmp = reinterpret_cast<const VD *>(f.vd)[v];
    }
    // out-neighbours loaded before apply decides whether they are activated
    const int odeg = oend - obeg;
    int32_t outd[D];
#pragma unroll
    for (int k = 0; k < D; ++k) outd[k] = k < odeg ? __ldg(sa.outDests + obeg + k) : 0;
    bool r;
    if (a.haveGather) {
      int src[D];
#pragma unroll
      for (int k = 0; k < D; ++k) src[k] = k < deg ? __ldg(a.inSources + beg + k) : 0;
      VD sv[D];
#pragma unroll
      for (int k = 0; k < D; ++k)
        if (k < deg) sv[k] = fused_read<VD>(f, src[k]);
      GR acc = P::gatherZero;
#pragma unroll
      for (int k = 0; k < D; ++k)
        if (k < deg)
          acc = P::gatherReduce(acc, P::gatherMap(&tmp, &sv[k], edge_ptr<P>(a.edgeData, beg + k)));
      r = do_apply<P>(&tmp, acc, a.iteration);
      cell->s[own ^ 1] = tmp;
      cell->ver = (f.stamp << 1) | (uint32_t)(own ^ 1);
    } else {  // apply only: nothing reads other vertices, update in place
      const GR gz = P::gatherZero;
      r = do_apply<P>(&tmp, gz, a.iteration);
      reinterpret_cast<VD *>(f.vd)[v] = tmp;
    }
    if (r) {
      f.retStamp[v] = (int32_t)f.stamp;
      ++cRet;
      cOut += (unsigned)(oend - obeg);
#pragma unroll
      for (int k = 0; k < D; ++k) {
        isEdge[k] = k < odeg;
        dst[k] = outd[k];
      }
    }
  }
  // activation: in-degree, CSC begin and the stamp exchange in one round trip
  bool ok[D];
  int32_t dg[D], bg[D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    ok[k] = false;
    dg[k] = 0;
    bg[k] = 0;
    if (isEdge[k]) {
      bg[k] = sa.inOffsets[dst[k]];
      dg[k] = sa.inOffsets[dst[k] + 1];
      ok[k] = atomicExch(sa.mark + dst[k], sa.stamp) != sa.stamp;
    }
  }
#pragma unroll
  for (int k = 0; k < D; ++k) dg[k] -= bg[k];
  // the next round is fused again: one thread per entry, every degree <= 8
  // (no split hints, no maximum degree)
  if (warpAppend)
    warp_append_list<D, false>(ok, dst, dg, bg, sa.next, a.capacity, a.errWord);
  else
    block_append_list<D, false>(ok, dst, dg, bg, sa.next, a.capacity, a.errWord);
}

// Every vertex's newest value back into the run's vertex data (f.vd).
template <class P>
__device__ void fused_fold(const FusedCtx &f, int nVertices) {
  typedef typename P::VertexData VD;
  const FusedCell<VD> *cells = reinterpret_cast<const FusedCell<VD> *>(f.cells);
  const int stride = gridDim.x * blockDim.x;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nVertices; v += stride) {
    const FusedCell<VD> c = load_cell(cells + v);
    reinterpret_cast<VD *>(f.vd)[v] = (c.ver & 1u) ? c.s[1] : c.s[0];
  }
}

}  // namespace detail
}  // namespace gas
