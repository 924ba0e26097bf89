// Fused list rounds for graphs whose in- and out-degrees are all <= 8
// (lattices, road networks): a thread per frontier vertex gathers, applies
// and activates its out-neighbours in one phase, so a round costs one grid
// barrier instead of two (gather -> barrier -> commit + scatter ->
// barrier).
//
// Bulk-synchronous reads without a commit step: vertex data has two slots
// per vertex (the engine's two buffers) and a version word per vertex,
//   ver[v] = (round stamp << 1) | slot holding v's newest value.
// A vertex applied in round S writes the slot it is not in and publishes
// (S, that slot).  Every read in round S wants the value as of the end of
// round S-1: when v's word already says S, that is the other slot (which
// the writer never touches in round S), otherwise the slot in the word --
// so readers need no ordering against the writer.  Active sets, round
// counts and results are those of the two-phase rounds; versioned data is
// folded back into the first slot before a dense round and at the end of
// the run.
#pragma once

#include "gather.cuh"
#include "scatter.cuh"

namespace gas {
namespace detail {

struct FusedCtx {
  void *slot[2];        // vertex data: slot 0 = the run's current buffer
  uint32_t *ver;        // [V] (stamp << 1) | slot
  uint32_t stamp;       // this round's stamp
  int32_t *retStamp;    // [V] stamp of the round whose apply returned true
};

// v's value as of the end of the previous round.  The word and both slots
// are loaded together (one round trip), then the right slot is kept.
template <class VD>
__device__ __forceinline__ VD fused_read(const FusedCtx &f, int v) {
  const uint32_t w = __ldcg(f.ver + v);
  const VD x0 = load_cg(reinterpret_cast<const VD *>(f.slot[0]) + v);
  const VD x1 = load_cg(reinterpret_cast<const VD *>(f.slot[1]) + v);
  const uint32_t s = ((w >> 1) == f.stamp) ? (1u - (w & 1u)) : (w & 1u);
  return s ? x1 : x0;
}

// Frontiers of at most this many vertices append per warp (one atomic per
// warp, no block barrier); larger ones per block (one atomic per block).
constexpr int kWarpAppendMax = 4096;

// Frontier entry i (none when i >= n) for this thread.  Counts this round's
// apply-returned-true vertices and their out-edges into cRet / cOut.
// warpAppend (block-uniform): append the activated vertices per warp.
// Every thread of the block calls it (the appends are collective).
template <class P>
__device__ __forceinline__ void fused_tpv_tile(const gas_gather_args &a, const ScatterArgs &sa, const FusedCtx &f,
                               int i, int n, int T, bool warpAppend, ScatterSmem &sm, unsigned &cRet,
                               unsigned &cOut) {
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
    const uint32_t wv = __ldcg(f.ver + v);
    const VD own0 = load_cg(reinterpret_cast<const VD *>(f.slot[0]) + v);
    const VD own1 = load_cg(reinterpret_cast<const VD *>(f.slot[1]) + v);
    const int own = (int)(wv & 1u);  // v is applied once per round: its word is still old
    VD tmp = own ? own1 : own0;
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
      reinterpret_cast<VD *>(f.slot[own ^ 1])[v] = tmp;
      f.ver[v] = (f.stamp << 1) | (uint32_t)(own ^ 1);
    } else {  // apply only: nothing reads other vertices, update in place
      const GR gz = P::gatherZero;
      r = do_apply<P>(&tmp, gz, a.iteration);
      reinterpret_cast<VD *>(f.slot[own])[v] = tmp;
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
  if (warpAppend)  // the next round is fused again: one thread per entry, degrees <= 8
    warp_append_list<D, false>(ok, dst, dg, bg, sa.next, a.capacity, a.errWord);
  else
    block_append<kSNT, D, GAS_GATHER_TILE>(ok, dst, dg, bg, sa.next, sa.maxGatherTiles, a.capacity,
                                           a.errWord, sm.app);
}

// Every vertex's newest value into slot 0 (the run's current buffer).
template <class P>
__device__ void fused_fold(const FusedCtx &f, int nVertices) {
  typedef typename P::VertexData VD;
  const int stride = gridDim.x * blockDim.x;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nVertices; v += stride) {
    const uint32_t w = __ldcg(f.ver + v);
    if (w & 1u) {
      reinterpret_cast<VD *>(f.slot[0])[v] = load_cg(reinterpret_cast<const VD *>(f.slot[1]) + v);
      f.ver[v] = w & ~1u;
    }
  }
}

}  // namespace detail
}  // namespace gas
