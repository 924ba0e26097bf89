// Dense (pull) rounds of the GB300 GAS engine.
//
// When the vertices whose apply returned true in round r have many
// out-edges, round r+1 runs as one pass over every vertex's in-edges
// instead of push + compaction (the reference's dense path builds byte
// flags with IntervalGather and compacts them with a scan,
// gpugas.h:690-717, primitives/scatter_if_mgpu.h:130-157):
//
//   vertex v is active in round r+1  <=>  some in-neighbour u of v returned
//   true in round r  (retStamp[r & 1][u] == stamp of round r)
//
// The stamps of consecutive rounds live in two arrays, so a round reads the
// previous round's set while it records its own.
//
// which is exactly the set the reference's scatterActivate builds, so the
// active sets and round counts are unchanged.  The pass walks the whole CSC
// in merge-path tiles whose splits are fixed per graph (so FP reductions
// are associated the same way every run), gathers speculatively, applies
// to the active vertices and writes every vertex's data to the other
// buffer of a ping-pong pair: no commit, no scatter traversal, no frontier
// list, one grid barrier per round.
#pragma once

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
  const int32_t *split;  // gather-tile splits of [0, nVertices)
  const void *vdCur;
  void *vdNext;
  const int32_t *prevRet;  // stamps written by the previous round (read only here)
  int32_t *curRet;         // stamps of this round (the other array of the pair)
  int32_t prevStamp;       // stamp of the previous round's apply-returned-true set
  int32_t curStamp;
  int32_t allActive;     // every vertex active (setActive(0, V))
  int32_t haveGather;
  void *carryVal;
  unsigned *carryFlag;
  unsigned epoch;
  unsigned *errWord;
  int32_t iteration;
  unsigned long long *cnt;  // [2]: (active << 32 | in-edges), (ret << 32 | out-edges)
};

template <class P>
struct DenseSmem {
  int32_t end[kGTILE];
  SegScanSmem<typename P::GatherResult, kGNT> seg;
  int32_t headPre;
  unsigned lookHas;
  unsigned lookAct;
  typename P::GatherResult lookVal;
};

template <class P>
__device__ void dense_tile(const DenseCtx &a, int t, DenseSmem<P> &sm) {
  typedef typename P::VertexData VD;
  typedef typename P::GatherResult GR;
  const int tid = threadIdx.x;
  const long long total = (long long)a.nVertices + a.nEdges;
  const int d0 = t * kGTILE;
  const int d1 = (int)min((long long)d0 + kGTILE, total);
  const int i0 = a.split[t];
  const int i1 = (d1 == total) ? a.nVertices : a.split[t + 1];
  const int j0 = d0 - i0, j1 = d1 - i1;
  const int nb = i1 - i0, na = j1 - j0;
  const VD *vd = reinterpret_cast<const VD *>(a.vdCur);
  for (int m = tid; m < nb; m += kGNT) sm.end[m] = a.inOffsets[i0 + m + 1] - j0;
  if (tid == 0) sm.headPre = i0 < a.nVertices ? a.inOffsets[i0] : a.nEdges;
  __syncthreads();

  const int tileItems = d1 - d0;
  const int dl = tid * kGVT;
  int bi = 0;
  if (dl < tileItems) {
    int lo = max(0, dl - na), hi = min(dl, nb);
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (sm.end[mid - 1] <= dl - mid)
        lo = mid;
      else
        hi = mid - 1;
    }
    bi = lo;
  }
  int aj = dl - bi;
  int kind[kGVT], vloc[kGVT], phys[kGVT];
#pragma unroll
  for (int v = 0; v < kGVT; ++v) {
    kind[v] = 0;
    vloc[v] = 0;
    phys[v] = 0;
    if (dl + v < tileItems) {
      if (bi < nb && (aj >= na || sm.end[bi] <= aj)) {
        kind[v] = 2;
        vloc[v] = bi;
        ++bi;
      } else {
        kind[v] = 1;
        vloc[v] = bi;
        phys[v] = j0 + aj;
        ++aj;
      }
    }
  }
  int src[kGVT];
#pragma unroll
  for (int v = 0; v < kGVT; ++v) src[v] = (kind[v] == 1) ? __ldg(a.inSources + phys[v]) : 0;
  unsigned eact[kGVT];
#pragma unroll
  for (int v = 0; v < kGVT; ++v)
    eact[v] = (kind[v] == 1) && (a.allActive || a.prevRet[src[v]] == a.prevStamp) ? 1u : 0u;
  const GR gz = P::gatherZero;
  GR val[kGVT];
#pragma unroll
  for (int v = 0; v < kGVT; ++v) {
    val[v] = gz;
    if (kind[v] == 1 && a.haveGather)
      val[v] = P::gatherMap(vd + (i0 + vloc[v]), vd + src[v], edge_ptr<P>(a.edgeData, phys[v]));
  }

  // ---- fold: per segment (vertex) the reduction and the activation OR
  unsigned has = 0u, act = 0u;
  GR acc = gz;
  bool segHas[kGVT];
  unsigned segAct[kGVT];
  GR segVal[kGVT];
  unsigned anyEnd = 0u;
#pragma unroll
  for (int v = 0; v < kGVT; ++v) {
    segHas[v] = false;
    segAct[v] = 0u;
    if (kind[v] == 1) {
      acc = has ? P::gatherReduce(acc, val[v]) : val[v];
      has = 1u;
      act |= eact[v];
    } else if (kind[v] == 2) {
      segHas[v] = has != 0u;
      segAct[v] = act;
      segVal[v] = acc;
      has = 0u;
      act = 0u;
      anyEnd = 1u;
    }
  }
  SegVal<GR> mine;
  mine.end = anyEnd;
  mine.has = has;
  mine.act = act;
  mine.val = acc;
  SegVal<GR> excl, tot;
  block_seg_scan<P, GR, kGNT>(mine, excl, tot, sm.seg);

  if (tid == kGNT - 1 && tot.has) {
    reinterpret_cast<GR *>(a.carryVal)[t] = tot.val;
    __threadfence();
    publish_flag(a.carryFlag + t, a.epoch, tot.act);
  }
  const bool headSplit = nb > 0 && sm.headPre < j0;
  if (tid < 32) {
    if (headSplit) {
      const int ts = (int)(((long long)sm.headPre + i0) / kGTILE);
      unsigned lh = 0u, la = 0u;
      GR lv = gz;
      for (int c0 = ts; c0 < t; c0 += 32) {
        const int ti = c0 + tid;
        const int cnt = min(32, t - c0);
        unsigned h = 0u, xa = 0u;
        GR x = gz;
        if (ti < t) {
          unsigned fa;
          if (wait_epoch(a.carryFlag + ti, a.epoch, a.errWord, &fa)) {
            x = load_cg(reinterpret_cast<const GR *>(a.carryVal) + ti);
            h = 1u;
            xa = fa;
          }
        }
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          unsigned oh = __shfl_down_sync(kFullMask, h, d);
          unsigned oa = __shfl_down_sync(kFullMask, xa, d);
          GR ox = shfl_down_any(x, d);
          if ((tid & (2 * d - 1)) == 0 && tid + d < cnt) {
            xa |= oa;
            if (oh) {
              x = h ? P::gatherReduce(x, ox) : ox;
              h = 1u;
            }
          }
        }
        if (tid == 0) {
          la |= xa;
          if (h) {
            lv = lh ? P::gatherReduce(lv, x) : x;
            lh = 1u;
          }
        }
      }
      if (tid == 0) {
        sm.lookHas = lh;
        sm.lookAct = la;
        sm.lookVal = lv;
      }
    } else if (tid == 0) {
      sm.lookHas = 0u;
      sm.lookAct = 0u;
    }
  }
  __syncthreads();

  unsigned preHas = 0u, preAct = 0u;
  GR preVal = gz;
  if (!excl.end && headSplit) {
    preAct = sm.lookAct;
    if (sm.lookHas) {
      preVal = sm.lookVal;
      preHas = 1u;
    }
  }
  preAct |= excl.act;
  if (excl.has) {
    preVal = preHas ? P::gatherReduce(preVal, excl.val) : excl.val;
    preHas = 1u;
  }
  bool firstDone = false;
#pragma unroll
  for (int v = 0; v < kGVT; ++v) {
    if (kind[v] == 2 && !firstDone) {
      firstDone = true;
      segAct[v] |= preAct;
      if (preHas) {
        segVal[v] = segHas[v] ? P::gatherReduce(preVal, segVal[v]) : preVal;
        segHas[v] = true;
      }
    }
  }

  // ---- apply to active vertices; every vertex is written to vdNext
  VD *vnext = reinterpret_cast<VD *>(a.vdNext);
  unsigned nA = 0, nEin = 0, nR = 0, nEout = 0;
#pragma unroll
  for (int v = 0; v < kGVT; ++v) {
    if (kind[v] == 2) {
      const int m = vloc[v];
      const int vx = i0 + m;
      VD tmp = vd[vx];
      if (a.allActive || segAct[v]) {  // with every vertex active, in-degree 0 too
        GR g = gz;
        if (a.haveGather && segHas[v]) g = P::gatherReduce(gz, segVal[v]);
        const bool r = do_apply<P>(&tmp, g, a.iteration);
        const int start = (m == 0) ? sm.headPre - j0 : sm.end[m - 1];
        ++nA;
        nEin += (unsigned)(sm.end[m] - start);
        if (r) {
          a.curRet[vx] = a.curStamp;
          ++nR;
          nEout += (unsigned)(a.outOffsets[vx + 1] - a.outOffsets[vx]);
        }
      }
      vnext[vx] = tmp;
    }
  }
  const unsigned wA = __reduce_add_sync(kFullMask, nA);
  const unsigned wEin = __reduce_add_sync(kFullMask, nEin);
  const unsigned wR = __reduce_add_sync(kFullMask, nR);
  const unsigned wEout = __reduce_add_sync(kFullMask, nEout);
  if ((tid & 31) == 0) {
    if (wA) atomicAdd(a.cnt, ((unsigned long long)wA << 32) | wEin);
    if (wR) atomicAdd(a.cnt + 1, ((unsigned long long)wR << 32) | wEout);
  }
}

// Dense -> list transition: the vertices stamped in this round become the
// scatter list (out-degree prefix, CSR begin), in vertex order per block.
template <int NT, int KS>
__device__ void compact_ret(const int32_t *retStamp, int32_t stamp, const int32_t *outOffsets,
                            int32_t nVertices, const gas_vertex_list &out, int32_t maxSplit,
                            unsigned *errWord, AppendSmem<NT, KS> &sm) {
  for (int base = blockIdx.x * NT; base < nVertices; base += gridDim.x * NT) {
    const int v = base + threadIdx.x;
    bool ok[1] = {false};
    int32_t ov[1] = {v}, od[1] = {0}, ob[1] = {0};
    if (v < nVertices && retStamp[v] == stamp) {
      ok[0] = true;
      ob[0] = outOffsets[v];
      od[0] = outOffsets[v + 1] - ob[0];
    }
    block_append<NT, 1, GAS_SCATTER_TILE>(ok, ov, od, ob, out, maxSplit, nVertices, errWord, sm);
  }
}

// List -> dense transition: stamp the vertices of a scatter list.
__device__ __forceinline__ void stamp_list(const gas_vertex_list &l, int n, int32_t *retStamp,
                                           int32_t stamp) {
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    retStamp[l.vid[i]] = stamp;
}

}  // namespace detail
}  // namespace gas
