// Program-templated gather+apply kernel of the GB300 GAS engine.
//
// Replaces the reference's gather pipeline -- edge-count scan, merge-path
// partitions, kGatherMap writing one (key, value) pair per edge to global
// memory, ReduceByKey and kApply (gpugas.h:421-513,
// gpugas_kernels.cuh:53-151) -- by one kernel:
//
//   * tiles of GAS_GATHER_TILE merged items (active vertices + their
//     in-edges) whose merge-path splits were written by whoever built the
//     frontier (block_append) -- no partition pass;
//   * per thread GAS_GATHER_ITEMS consecutive items: all in-edge source
//     loads, then all gatherMap loads, issued before any reduction (ILP);
//   * thread-sequential fold + block-wide segmented scan for vertices that
//     straddle threads, and a decoupled look-back over published tile
//     aggregates for vertices that straddle tiles;
//   * apply() on a register copy of the vertex, written to vertexNew[i]
//     (committed by the scatter kernel, so every gather of this round reads
//     the previous round's values: the bulk-synchronous semantics of
//     refgas.h:143-167);
//   * vertices whose apply returned true are appended to the scatter list
//     with their out-degree prefix and the scatter kernel's tile splits.
//
// Rounds whose frontier has no vertex of in-degree above
// GAS_TPV_MAX_DEGREE (lattices, road networks) run one thread per vertex
// instead: no merge path, block scan or look-back, and the edges of a
// vertex are folded left to right in CSC order, exactly as
// refgas.h:147-158 folds them.
#pragma once

#include <type_traits>

#include "primitives.cuh"

namespace gas {
namespace detail {

constexpr int kGNT = GAS_GATHER_THREADS;
constexpr int kGVT = GAS_GATHER_ITEMS;
constexpr int kGTILE = GAS_GATHER_TILE;
constexpr int kSTILE = GAS_SCATTER_TILE;

// apply() with or without the iteration number.  The reference BFS reads
// the iteration from a __constant__ set by the driver (bfs.cu:28,63,85);
// programs may instead take it as a third argument.
template <class P>
struct ApplyTakesIteration {
  template <class Q>
  static auto test(int) -> decltype(Q::apply((typename Q::VertexData *)0,
                                             typename Q::GatherResult(), 0),
                                    std::true_type());
  template <class Q>
  static std::false_type test(...);
  static constexpr bool value = decltype(test<P>(0))::value;
};

template <class P>
__device__ __forceinline__ bool call_apply(typename P::VertexData *v,
                                           const typename P::GatherResult &g, int iteration,
                                           std::true_type) {
  return P::apply(v, g, iteration);
}
template <class P>
__device__ __forceinline__ bool call_apply(typename P::VertexData *v,
                                           const typename P::GatherResult &g, int,
                                           std::false_type) {
  return P::apply(v, g);
}
template <class P>
__device__ __forceinline__ bool do_apply(typename P::VertexData *v,
                                         const typename P::GatherResult &g, int iteration) {
  return call_apply<P>(v, g, iteration,
                       std::integral_constant<bool, ApplyTakesIteration<P>::value>());
}

template <class P>
__device__ __forceinline__ const typename P::EdgeData *edge_ptr(const void *ed, int32_t e) {
  if (std::is_empty<typename P::EdgeData>::value) return nullptr;
  return reinterpret_cast<const typename P::EdgeData *>(ed) + e;
}

// The merge-path arrays are dead once block_append stages its output (its
// first internal barrier follows the last read of vid), so they share
// storage with the staging area.
template <class P>
struct GatherSmem {
  union {
    struct {
      int32_t end[kGTILE];       // tile-local edge index at which vertex i0+m ends
      int32_t vid[kGTILE + 1];   // vertex id of frontier entry i0+m
      int32_t base[kGTILE + 1];  // CSC position = frontier edge index + base
    };
    AppendSmem<kGNT, kGVT> app;
  };
  SegScanSmem<typename P::GatherResult, kGNT> seg;
  int32_t headPre;
  unsigned lookHas;
  typename P::GatherResult lookVal;
  int32_t tile;
};

// Current frontier size: (n, total in-edges).
__device__ __forceinline__ void frontier_size(const gas_gather_args &a, int &n, int &T) {
  if (a.rangeMode) {
    n = a.rangeCount;
    T = a.inOffsets[a.rangeStart + a.rangeCount] - a.rangeBase;
  } else {
    unsigned long long c = *a.front.count;
    n = (int)(c >> 32);
    T = (int)(c & 0xffffffffull);
    if (n > a.capacity) n = a.capacity;  // only after a reported overflow
  }
}

__device__ __forceinline__ unsigned frontier_max_degree(const gas_gather_args &a) {
  return a.rangeMode ? (unsigned)a.rangeMaxDeg : *a.front.maxDeg;
}

// Entry i of the current frontier: vertex, in-edge prefix and end, CSC begin.
__device__ __forceinline__ void front_entry(const gas_gather_args &a, int i, int n, int T,
                                            int &v, int &pre, int &end, int &beg) {
  if (a.rangeMode) {
    v = a.rangeStart + i;
    beg = a.inOffsets[v];
    pre = beg - a.rangeBase;
    end = a.inOffsets[v + 1] - a.rangeBase;
  } else {
    v = a.front.vid[i];
    pre = a.front.pre[i];
    end = (i + 1 < n) ? a.front.pre[i + 1] : T;
    beg = a.front.beg[i];
  }
}

// Gather tiles of the current round: mode and count (maxDeg: the
// frontier's largest in-degree, frontier_max_degree).
__device__ __forceinline__ int gather_tiles(const gas_gather_args &a, int n, int T, unsigned maxDeg,
                                            bool &tpv) {
  tpv = a.haveGather && maxDeg <= GAS_TPV_MAX_DEGREE;
  long long items;
  int tile;
  if (!a.haveGather) {
    items = n;
    tile = kGTILE;
  } else if (tpv) {
    items = n;
    tile = GAS_TPV_TILE;
  } else {
    items = (long long)n + T;
    tile = kGTILE;
  }
  return (int)((items + tile - 1) / tile);
}

template <class P>
__device__ void gather_tile(const gas_gather_args &a, int t, int n, int T, GatherSmem<P> &sm) {
  typedef typename P::VertexData VD;
  typedef typename P::GatherResult GR;
  const int tid = threadIdx.x;
  const long long total = (long long)n + T;
  const int d0 = t * kGTILE;
  const int d1 = (int)min((long long)d0 + kGTILE, total);
  const int32_t *split = a.rangeMode ? a.rangeSplit : a.front.split;
  const int i0 = split[t];
  const int i1 = (d1 == total) ? n : split[t + 1];
  const int j0 = d0 - i0, j1 = d1 - i1;
  const int nb = i1 - i0;  // vertices ending in this tile
  const int na = j1 - j0;  // edges in this tile
  const int nload = nb + (i1 < n ? 1 : 0);
  const VD *vd = reinterpret_cast<const VD *>(a.vertexData);

  for (int m = tid; m < nload; m += kGNT) {
    int v, pre, end, beg;
    front_entry(a, i0 + m, n, T, v, pre, end, beg);
    sm.vid[m] = v;
    sm.base[m] = beg - pre;
    if (m < nb) sm.end[m] = end - j0;
    if (m == 0) sm.headPre = pre;
  }
  __syncthreads();

  // ---- merge-path walk of this thread's items
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
        phys[v] = j0 + aj + sm.base[bi];
        ++aj;
      }
    }
  }

  // ---- independent loads first: in-edge sources, and for vertex ends the
  // vertex data and CSR range that apply / the scatter list need
  int src[kGVT], obeg[kGVT], oend[kGVT];
#pragma unroll
  for (int v = 0; v < kGVT; ++v) {
    src[v] = 0;
    obeg[v] = oend[v] = 0;
    if (kind[v] == 1) src[v] = __ldg(a.inSources + phys[v]);
    if (kind[v] == 2) {
      const int vx = sm.vid[vloc[v]];
      obeg[v] = a.outOffsets[vx];
      oend[v] = a.outOffsets[vx + 1];
    }
  }
  GR val[kGVT];
#pragma unroll
  for (int v = 0; v < kGVT; ++v)
    if (kind[v] == 1)
      val[v] = P::gatherMap(vd + sm.vid[vloc[v]], vd + src[v], edge_ptr<P>(a.edgeData, phys[v]));

  // ---- thread-sequential fold; seg*[v] holds the segment ending at item v
  unsigned has = 0u;
  GR acc;
  bool segHas[kGVT];
  GR segVal[kGVT];
  unsigned anyEnd = 0u;
#pragma unroll
  for (int v = 0; v < kGVT; ++v) {
    segHas[v] = false;
    if (kind[v] == 1) {
      acc = has ? P::gatherReduce(acc, val[v]) : val[v];
      has = 1u;
    } else if (kind[v] == 2) {
      segHas[v] = has != 0u;
      segVal[v] = acc;
      has = 0u;
      anyEnd = 1u;
    }
  }
  SegVal<GR> mine;
  mine.end = anyEnd;
  mine.has = has;
  mine.act = 0u;
  mine.val = acc;
  SegVal<GR> excl, tot;
  block_seg_scan<P, GR, kGNT>(mine, excl, tot, sm.seg);

  // ---- publish this tile's tail aggregate for the tiles after it
  if (tid == kGNT - 1 && tot.has) {
    reinterpret_cast<GR *>(a.carryVal)[t] = tot.val;
    __threadfence();
    publish_flag(a.carryFlag + t, a.epoch, 0u);
  }
  // ---- look-back for a first vertex that started in an earlier tile
  const bool headSplit = nb > 0 && sm.headPre < j0;
  if (tid < 32) {
    if (headSplit) {
      const int ts = (int)(((long long)sm.headPre + i0) / kGTILE);
      unsigned lh = 0u;
      GR lv;
      for (int c0 = ts; c0 < t; c0 += 32) {
        const int ti = c0 + tid;
        const int cnt = min(32, t - c0);
        unsigned h = 0u;
        GR x;
        unsigned act;
        if (ti < t) {
          if (wait_epoch(a.carryFlag + ti, a.epoch, a.errWord, &act)) {
            x = load_cg(reinterpret_cast<const GR *>(a.carryVal) + ti);
            h = 1u;
          }
        }
        // ordered tree reduction over lanes 0..cnt-1
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          unsigned oh = __shfl_down_sync(kFullMask, h, d);
          GR ox = shfl_down_any(x, d);
          if ((tid & (2 * d - 1)) == 0 && tid + d < cnt) {
            if (oh) {
              x = h ? P::gatherReduce(x, ox) : ox;
              h = 1u;
            }
          }
        }
        if (tid == 0 && h) {
          lv = lh ? P::gatherReduce(lv, x) : x;
          lh = 1u;
        }
      }
      if (tid == 0) {
        sm.lookHas = lh;
        if (lh) sm.lookVal = lv;
      }
    } else if (tid == 0) {
      sm.lookHas = 0u;
    }
  }
  __syncthreads();

  // ---- prefix for this thread's first vertex end
  unsigned preHas = 0u;
  GR preVal;
  if (!excl.end && headSplit && sm.lookHas) {
    preVal = sm.lookVal;
    preHas = 1u;
  }
  if (excl.has) {
    preVal = preHas ? P::gatherReduce(preVal, excl.val) : excl.val;
    preHas = 1u;
  }
  bool firstDone = false;
#pragma unroll
  for (int v = 0; v < kGVT; ++v) {
    if (kind[v] == 2 && !firstDone) {
      firstDone = true;
      if (preHas) {
        segVal[v] = segHas[v] ? P::gatherReduce(preVal, segVal[v]) : preVal;
        segHas[v] = true;
      }
    }
  }

  // ---- apply and collect vertices that activate their out-neighbours
  const GR gz = P::gatherZero;
  bool ok[kGVT];
  int32_t ovid[kGVT], odeg[kGVT];
  VD *vnew = reinterpret_cast<VD *>(a.vertexNew);
#pragma unroll
  for (int v = 0; v < kGVT; ++v) {
    ok[v] = false;
    ovid[v] = 0;
    odeg[v] = 0;
    if (kind[v] == 2) {
      const int m = vloc[v];
      const int32_t vx = sm.vid[m];
      GR g = gz;
      if (segHas[v]) g = P::gatherReduce(gz, segVal[v]);
      VD tmp = vd[vx];
      const bool r = do_apply<P>(&tmp, g, a.iteration);
      vnew[i0 + m] = tmp;
      if (r) {
        ok[v] = true;
        ovid[v] = vx;
        odeg[v] = oend[v] - obeg[v];
      }
    }
  }
  block_append<kGNT, kGVT, kSTILE>(ok, ovid, odeg, obeg, a.scat, a.maxScatTiles, a.capacity,
                                   a.errWord, sm.app);
}

// Low-degree rounds: one thread per active vertex, its (<= GAS_TPV_MAX_DEGREE)
// in-edges folded left to right from gatherZero, as refgas.h:147-158.
template <class P>
__device__ void tpv_gather_tile(const gas_gather_args &a, int t, int n, int T,
                                GatherSmem<P> &sm) {
  typedef typename P::VertexData VD;
  typedef typename P::GatherResult GR;
  constexpr int D = GAS_TPV_MAX_DEGREE;
  const VD *vd = reinterpret_cast<const VD *>(a.vertexData);
  VD *vnew = reinterpret_cast<VD *>(a.vertexNew);
  const int i = t * GAS_TPV_TILE + threadIdx.x;
  bool ok[1] = {false};
  int32_t ov[1] = {0}, od[1] = {0}, ob[1] = {0};
  if (i < n) {
    int v, pre, end, beg;
    front_entry(a, i, n, T, v, pre, end, beg);
    const int deg = end - pre;
    const int obeg = a.outOffsets[v], oend = a.outOffsets[v + 1];
    // source ids (and 4-byte edge data) as 16-byte quads: at most three
    // each for the <= 8 in-edges at any alignment (the arrays are padded)
    typedef typename P::EdgeData ED;
    constexpr bool kQuadEd = !std::is_empty<ED>::value && sizeof(ED) == 4;
    int src[D], edw[kQuadEd ? D : 1];
    load_window8(a.inSources, beg, beg + deg, src);
    if constexpr (kQuadEd) load_window8(static_cast<const int32_t *>(a.edgeData), beg, beg + deg, edw);
    GR acc = P::gatherZero;
#pragma unroll
    for (int k = 0; k < D; ++k)
      if (k < deg) {
        const ED *ep;
        ED e;
        if constexpr (kQuadEd) {
          memcpy(&e, &edw[k], sizeof(ED));
          ep = &e;
        } else {
          ep = edge_ptr<P>(a.edgeData, beg + k);
        }
        acc = P::gatherReduce(acc, P::gatherMap(vd + v, vd + src[k], ep));
      }
    VD tmp = vd[v];
    const bool r = do_apply<P>(&tmp, acc, a.iteration);
    vnew[i] = tmp;
    if (r) {
      ok[0] = true;
      ov[0] = v;
      od[0] = oend - obeg;
      ob[0] = obeg;
    }
  }
  block_append<kGNT, 1, kSTILE>(ok, ov, od, ob, a.scat, a.maxScatTiles, a.capacity, a.errWord,
                                sm.app);
}

// apply only (gatherApply(false), gpugas.h:503-512): one thread per active
// vertex, vertex data updated in place.
template <class P>
__device__ void apply_tile(const gas_gather_args &a, int t, int n, GatherSmem<P> &sm) {
  typedef typename P::VertexData VD;
  typedef typename P::GatherResult GR;
  VD *vd = reinterpret_cast<VD *>(a.vertexData);
  const GR gz = P::gatherZero;
  bool ok[kGVT];
  int32_t ovid[kGVT], odeg[kGVT], obeg[kGVT];
#pragma unroll
  for (int v = 0; v < kGVT; ++v) {
    ok[v] = false;
    ovid[v] = 0;
    odeg[v] = 0;
    obeg[v] = 0;
    const int i = t * kGTILE + v * kGNT + threadIdx.x;
    if (i < n) {
      const int32_t vx = a.rangeMode ? a.rangeStart + i : a.front.vid[i];
      const int ob = a.outOffsets[vx], oe = a.outOffsets[vx + 1];
      VD tmp = vd[vx];
      const bool r = do_apply<P>(&tmp, gz, a.iteration);
      vd[vx] = tmp;
      if (r) {
        ok[v] = true;
        ovid[v] = vx;
        odeg[v] = oe - ob;
        obeg[v] = ob;
      }
    }
  }
  block_append<kGNT, kGVT, kSTILE>(ok, ovid, odeg, obeg, a.scat, a.maxScatTiles, a.capacity,
                                   a.errWord, sm.app);
}

template <class P>
__device__ __forceinline__ void gather_dispatch(const gas_gather_args &a, int t, int n, int T,
                                                bool tpv, GatherSmem<P> &sm) {
  if (!a.haveGather)
    apply_tile<P>(a, t, n, sm);
  else if (tpv)
    tpv_gather_tile<P>(a, t, n, T, sm);
  else
    gather_tile<P>(a, t, n, T, sm);
}

// One launch per phase: blocks take tiles in order from a counter, so a
// tile whose look-back waits on earlier tiles only waits on running CTAs.
template <class P>
__global__ void __launch_bounds__(kGNT) gather_apply_kernel(const gas_gather_args a) {
  __shared__ GatherSmem<P> sm;
  int n, T;
  frontier_size(a, n, T);
  bool tpv;
  const int ntiles = gather_tiles(a, n, T, frontier_max_degree(a), tpv);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *a.resetCount = 0ull;
    *a.resetMaxDeg = 0u;
    *a.resetTile = 0u;
    if (a.statSlot) a.statSlot[0] = ((unsigned long long)n << 32) | (unsigned)T;
  }
  for (;;) {
    if (threadIdx.x == 0) sm.tile = (int)atomicAdd(a.tileCounter, 1u);
    __syncthreads();
    const int t = sm.tile;
    __syncthreads();
    if (t >= ntiles) break;
    gather_dispatch<P>(a, t, n, T, tpv, sm);
    __syncthreads();
  }
}

}  // namespace detail
}  // namespace gas
