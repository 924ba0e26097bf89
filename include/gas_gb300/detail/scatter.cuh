// Program-independent scatter/activate kernel of the GB300 GAS engine.
//
// Replaces scatterActivate (gpugas.h:669-751): the predicated out-degree
// scan, the dense flag path (memset + IntervalGather + scan compaction,
// primitives/scatter_if_mgpu.h) and the sparse path (atomic list append +
// MergesortKeys + unique scan).  One kernel:
//
//   * commits vertexNew -> vertexData for every active vertex (the second
//     half of the bulk-synchronous apply, refgas.h:160-166);
//   * walks the out-edges of vertices whose apply returned true in merge
//     -path tiles (splits written by the gather kernel);
//   * deduplicates destinations with a per-vertex round stamp
//     (one atomicExch per first visit, none afterwards) instead of sorting;
//   * appends newly active vertices to the next frontier with their
//     in-degree prefix, CSC begin and the next gather's tile splits
//     (block_append);
//   * lists whose out-degrees are all <= GAS_TPV_MAX_DEGREE are walked one
//     thread per vertex instead of in merge-path tiles.
#pragma once

#include "primitives.cuh"

namespace gas {
namespace detail {

constexpr int kSNT = GAS_SCATTER_THREADS;
constexpr int kSVT = GAS_SCATTER_ITEMS;

struct ScatterArgs {
  const int32_t *outOffsets;
  const int32_t *outDests;
  const int32_t *inOffsets;
  gas_vertex_list scat;  // built by the gather kernel (out-degree prefix)
  // commit of vertexNew for the current frontier
  int32_t commit;
  int32_t vertexBytes;
  void *vertexData;
  const void *vertexNew;
  int32_t rangeMode;
  int32_t rangeStart;
  int32_t rangeCount;
  const int32_t *frontVid;
  const unsigned long long *frontCount;
  gas_vertex_list next;  // next frontier (in-degree prefix)
  int32_t maxGatherTiles;
  int32_t capacity;
  // destination dedup
  int32_t *mark;
  int32_t stamp;
  // counters
  unsigned *tileCounter;
  unsigned *resetTile;
  unsigned long long *resetScatCount;
  unsigned *resetScatMaxDeg;
  unsigned *errWord;
  unsigned long long *statSlot;  // round statistics (may be null)
};

struct ScatterSmem {
  union {
    struct {
      int32_t end[GAS_SCATTER_TILE];
      int32_t base[GAS_SCATTER_TILE + 1];
    };
    AppendSmem<kSNT, kSVT> app;  // staging reuses the merge-path arrays
  };
  int32_t tile;
};

__device__ __forceinline__ void commit_vertex(void *dst, const void *src, int bytes) {
  if ((bytes & 3) == 0) {
    unsigned *d = reinterpret_cast<unsigned *>(dst);
    const unsigned *s = reinterpret_cast<const unsigned *>(src);
    for (int k = 0; k < (bytes >> 2); ++k) d[k] = s[k];
  } else {
    char *d = reinterpret_cast<char *>(dst);
    const char *s = reinterpret_cast<const char *>(src);
    for (int k = 0; k < bytes; ++k) d[k] = s[k];
  }
}

// vertexData[frontier vertex i] = vertexNew[i] for the nf active vertices
// (grid-stride over the whole launch).
__device__ __forceinline__ void commit_frontier(const ScatterArgs &a, int nf) {
  const int stride = gridDim.x * blockDim.x;
  char *vd = reinterpret_cast<char *>(a.vertexData);
  const char *vn = reinterpret_cast<const char *>(a.vertexNew);
  const int vb = a.vertexBytes;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += stride) {
    const int v = a.rangeMode ? a.rangeStart + i : a.frontVid[i];
    commit_vertex(vd + (size_t)v * vb, vn + (size_t)i * vb, vb);
  }
}

// Activation of destination u: the in-degree and CSC begin are loaded
// before the stamp test so both round trips overlap.
template <int K>
__device__ __forceinline__ void activate(const ScatterArgs &a, const bool (&isEdge)[K],
                                         const int32_t (&dst)[K], bool (&ok)[K],
                                         int32_t (&deg)[K], int32_t (&beg)[K]) {
#pragma unroll
  for (int v = 0; v < K; ++v) {
    ok[v] = false;
    deg[v] = 0;
    beg[v] = 0;
    if (isEdge[v]) {
      beg[v] = a.inOffsets[dst[v]];
      deg[v] = a.inOffsets[dst[v] + 1];
    }
  }
#pragma unroll
  for (int v = 0; v < K; ++v) {
    if (isEdge[v]) {
      deg[v] -= beg[v];
      int32_t *mk = a.mark + dst[v];
      if (__ldcg(mk) != a.stamp && atomicExch(mk, a.stamp) != a.stamp) ok[v] = true;
    }
  }
}

__device__ inline void scatter_tile(const ScatterArgs &a, int t, int n, int T, ScatterSmem &sm) {
  const int tid = threadIdx.x;
  const long long total = (long long)n + T;
  const int d0 = t * GAS_SCATTER_TILE;
  const int d1 = (int)min((long long)d0 + GAS_SCATTER_TILE, total);
  const int i0 = a.scat.split[t];
  const int i1 = (d1 == total) ? n : a.scat.split[t + 1];
  const int j0 = d0 - i0, j1 = d1 - i1;
  const int nb = i1 - i0, na = j1 - j0;
  const int nload = nb + (i1 < n ? 1 : 0);
  for (int m = tid; m < nload; m += kSNT) {
    const int i = i0 + m;
    const int pre = a.scat.pre[i];
    const int end = (i + 1 < n) ? a.scat.pre[i + 1] : T;
    sm.base[m] = a.scat.beg[i] - pre;
    if (m < nb) sm.end[m] = end - j0;
  }
  __syncthreads();

  const int tileItems = d1 - d0;
  const int dl = tid * kSVT;
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
  int phys[kSVT];
  bool isEdge[kSVT];
#pragma unroll
  for (int v = 0; v < kSVT; ++v) {
    isEdge[v] = false;
    phys[v] = 0;
    if (dl + v < tileItems) {
      if (bi < nb && (aj >= na || sm.end[bi] <= aj)) {
        ++bi;
      } else {
        isEdge[v] = true;
        phys[v] = j0 + aj + sm.base[bi];
        ++aj;
      }
    }
  }
  int32_t dst[kSVT];
#pragma unroll
  for (int v = 0; v < kSVT; ++v) dst[v] = isEdge[v] ? __ldg(a.outDests + phys[v]) : 0;
  bool ok[kSVT];
  int32_t deg[kSVT], beg[kSVT];
  activate<kSVT>(a, isEdge, dst, ok, deg, beg);
  block_append<kSNT, kSVT, GAS_GATHER_TILE>(ok, dst, deg, beg, a.next, a.maxGatherTiles,
                                            a.capacity, a.errWord, sm.app);
}

// Low-degree rounds: one thread per vertex of the scatter list.
__device__ inline void tpv_scatter_tile(const ScatterArgs &a, int t, int n, int T,
                                        ScatterSmem &sm) {
  constexpr int D = GAS_TPV_MAX_DEGREE;
  const int i = t * GAS_TPV_TILE + threadIdx.x;
  bool isEdge[D];
  int32_t dst[D];
  if (i < n) {
    const int pre = a.scat.pre[i];
    const int end = (i + 1 < n) ? a.scat.pre[i + 1] : T;
    const int b = a.scat.beg[i];
    const int d = end - pre;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      isEdge[k] = k < d;
      dst[k] = k < d ? __ldg(a.outDests + b + k) : 0;
    }
  } else {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      isEdge[k] = false;
      dst[k] = 0;
    }
  }
  bool ok[D];
  int32_t deg[D], beg[D];
  activate<D>(a, isEdge, dst, ok, deg, beg);
  block_append<kSNT, D, GAS_GATHER_TILE>(ok, dst, deg, beg, a.next, a.maxGatherTiles,
                                         a.capacity, a.errWord, sm.app);
}

// Scatter tiles of a scatter list: mode and count.
__device__ __forceinline__ int scatter_tiles(const gas_vertex_list &l, int n, int T, bool &tpv) {
  tpv = *l.maxDeg <= GAS_TPV_MAX_DEGREE;
  if (tpv) return (n + GAS_TPV_TILE - 1) / GAS_TPV_TILE;
  return (int)(((long long)n + T + GAS_SCATTER_TILE - 1) / GAS_SCATTER_TILE);
}

static __global__ void __launch_bounds__(kSNT) scatter_activate_kernel(const ScatterArgs a) {
  __shared__ ScatterSmem sm;
  const unsigned long long sc = *a.scat.count;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *a.resetTile = 0u;
    *a.resetScatCount = 0ull;
    *a.resetScatMaxDeg = 0u;
    if (a.statSlot) a.statSlot[1] = sc;
  }
  if (a.commit) {
    int nf;
    if (a.rangeMode) {
      nf = a.rangeCount;
    } else {
      nf = (int)(*a.frontCount >> 32);
      if (nf > a.capacity) nf = a.capacity;
    }
    commit_frontier(a, nf);
  }
  int n = (int)(sc >> 32);
  if (n > a.capacity) n = a.capacity;
  const int T = (int)(sc & 0xffffffffull);
  bool tpv;
  const int ntiles = scatter_tiles(a.scat, n, T, tpv);
  for (;;) {
    if (threadIdx.x == 0) sm.tile = (int)atomicAdd(a.tileCounter, 1u);
    __syncthreads();
    const int t = sm.tile;
    __syncthreads();
    if (t >= ntiles) break;
    if (tpv)
      tpv_scatter_tile(a, t, n, T, sm);
    else
      scatter_tile(a, t, n, T, sm);
    __syncthreads();
  }
}

// Merge-path splits of a vertex range [rangeStart, rangeStart+n) against
// its in-edges, for gather tiles of GAS_GATHER_TILE items.
static __global__ void range_split_kernel(const int32_t *inOffsets, int rangeStart, int n, int T,
                                   int32_t *split, int nsplit) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nsplit) return;
  const long long total = (long long)n + T;
  const long long d = min((long long)t * GAS_GATHER_TILE, total);
  const int base = inOffsets[rangeStart];
  long long lo = max(0ll, d - T), hi = min(d, (long long)n);
  while (lo < hi) {
    long long mid = (lo + hi + 1) >> 1;
    const long long endPrev = (long long)inOffsets[rangeStart + mid] - base;
    if (endPrev <= d - mid)
      lo = mid;
    else
      hi = mid - 1;
  }
  split[t] = (int32_t)lo;
}

}  // namespace detail
}  // namespace gas
