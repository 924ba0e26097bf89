// Device primitives shared by the gather, apply and scatter kernels.
//
// - word-wise warp shuffles for any trivially copyable type;
// - block-wide scans (u64 sums; segmented pairs for partial reductions);
// - bounded acquire/release flag helpers for cross-tile look-back;
// - block_append: reserves space in a frontier list with one packed 64-bit
//   atomic per tile and writes merge-path split hints for the consumer's
//   tiles, so the next kernel needs no partition search.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../gas_gb300_core.h"

namespace gas {
namespace detail {

constexpr unsigned kFullMask = 0xffffffffu;
// ~0.5 s of polling before a look-back wait reports GAS_DEVERR_TIMEOUT
constexpr unsigned kSpinLimit = 1u << 22;

template <typename T>
__device__ __forceinline__ T shfl_up_any(const T &v, int delta) {
  constexpr int W = (int)((sizeof(T) + 3) / 4);
  uint32_t w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int k = 0; k < W; ++k) w[k] = __shfl_up_sync(kFullMask, w[k], delta);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

template <typename T>
__device__ __forceinline__ T shfl_down_any(const T &v, int delta) {
  constexpr int W = (int)((sizeof(T) + 3) / 4);
  uint32_t w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int k = 0; k < W; ++k) w[k] = __shfl_down_sync(kFullMask, w[k], delta);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

template <typename T>
__device__ __forceinline__ T shfl_down_any_w(const T &v, int delta, int width) {
  constexpr int W = (int)((sizeof(T) + 3) / 4);
  uint32_t w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int k = 0; k < W; ++k) w[k] = __shfl_down_sync(kFullMask, w[k], delta, width);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

template <typename T>
__device__ __forceinline__ T shfl_any(const T &v, int lane) {
  constexpr int W = (int)((sizeof(T) + 3) / 4);
  uint32_t w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int k = 0; k < W; ++k) w[k] = __shfl_sync(kFullMask, w[k], lane);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

// L1-bypassing load of any type (values published by other CTAs).
template <typename T>
__device__ __forceinline__ T load_cg(const T *p) {
  constexpr int W = (int)((sizeof(T) + 3) / 4);
  uint32_t w[W];
  if (sizeof(T) % 4 == 0) {
#pragma unroll
    for (int k = 0; k < W; ++k) w[k] = __ldcg(reinterpret_cast<const unsigned *>(p) + k);
  } else {
    memcpy(w, (const void *)p, sizeof(T));
  }
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

// Entries [beg, end) (end - beg <= 8) of an int32 array padded to whole
// 16-byte quads, as out[0..end-beg): the at most three quads covering them,
// then a shift by beg % 4 (selects, no local-memory indexing).
__device__ __forceinline__ void load_window8(const int32_t *arr, int beg, int end, int (&out)[8]) {
  static_assert(GAS_TPV_MAX_DEGREE == 8, "three quads cover 8 entries at any alignment");
  int w[12];
  const int q0 = beg >> 2, nq = end > beg ? ((end - 1) >> 2) - q0 + 1 : 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    int4 t = make_int4(0, 0, 0, 0);
    if (k < nq) t = __ldg(reinterpret_cast<const int4 *>(arr) + q0 + k);
    w[4 * k] = t.x;
    w[4 * k + 1] = t.y;
    w[4 * k + 2] = t.z;
    w[4 * k + 3] = t.w;
  }
  const int off = beg & 3;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    int x0 = w[k];
    x0 = off == 1 ? w[k + 1] : x0;
    x0 = off == 2 ? w[k + 2] : x0;
    x0 = off == 3 ? w[k + 3] : x0;
    out[k] = x0;
  }
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned *p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Tile aggregates are published with flag = (epoch << 1) | act.
__device__ __forceinline__ void publish_flag(unsigned *flag, unsigned epoch, unsigned act) {
  st_release(flag, (epoch << 1) | (act & 1u));
}

// Waits (bounded) until *flag carries `epoch`; returns false and sets
// GAS_DEVERR_TIMEOUT in *err when the limit is reached.  *act receives the
// published activation bit.
__device__ __forceinline__ bool wait_epoch(const unsigned *flag, unsigned epoch, unsigned *err,
                                           unsigned *act) {
  unsigned spins = 0;
  unsigned f;
  while (((f = ld_acquire(flag)) >> 1) != epoch) {
    if (++spins > kSpinLimit) {
      atomicOr(err, GAS_DEVERR_TIMEOUT);
      *act = 0u;
      return false;
    }
    __nanosleep(64);
  }
  *act = f & 1u;
  return true;
}

// ---------------------------------------------------------------------------
// Block-wide exclusive scan of unsigned 64-bit sums.
template <int NT>
struct ScanU64Smem {
  unsigned long long warp[NT / 32];
  unsigned long long total;
};

template <int NT>
__device__ __forceinline__ void block_exclusive_scan_u64(unsigned long long x,
                                                         unsigned long long &excl,
                                                         unsigned long long &total,
                                                         ScanU64Smem<NT> &sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    unsigned long long o = __shfl_up_sync(kFullMask, incl, d);
    if (lane >= d) incl += o;
  }
  if (lane == 31) sm.warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = lane < NT / 32 ? sm.warp[lane] : 0ull;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      unsigned long long o = __shfl_up_sync(kFullMask, w, d);
      if (lane >= d) w += o;
    }
    if (lane < NT / 32) sm.warp[lane] = w;
    if (lane == NT / 32 - 1) sm.total = w;
  }
  __syncthreads();
  unsigned long long wpre = warp > 0 ? sm.warp[warp - 1] : 0ull;
  excl = wpre + incl - x;
  total = sm.total;
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Segmented partial reductions.  A SegVal is the state flowing between
// consecutive items: `end` = a vertex boundary occurred inside, `has` = val
// holds a reduction of at least one gathered edge value, `act` = one of
// those edges activates its destination (dense rounds).
template <typename T>
struct SegVal {
  unsigned end;
  unsigned has;
  unsigned act;
  T val;
};

template <class P, typename T>
__device__ __forceinline__ SegVal<T> seg_combine(const SegVal<T> &a, const SegVal<T> &b) {
  if (b.end) return b;
  SegVal<T> r;
  r.end = a.end;
  r.act = a.act | b.act;
  if (!a.has) {
    r.has = b.has;
    r.val = b.val;
  } else if (!b.has) {
    r.has = 1u;
    r.val = a.val;
  } else {
    r.has = 1u;
    r.val = P::gatherReduce(a.val, b.val);
  }
  return r;
}

template <typename T, int NT>
struct SegScanSmem {
  SegVal<T> warp[NT / 32];
};

// Inclusive block scan with seg_combine; returns the exclusive prefix of
// this thread in `excl` and the block aggregate in `total`.
template <class P, typename T, int NT>
__device__ __forceinline__ void block_seg_scan(const SegVal<T> &x, SegVal<T> &excl,
                                               SegVal<T> &total, SegScanSmem<T, NT> &sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  SegVal<T> incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    SegVal<T> o;
    o.end = __shfl_up_sync(kFullMask, incl.end, d);
    o.has = __shfl_up_sync(kFullMask, incl.has, d);
    o.act = __shfl_up_sync(kFullMask, incl.act, d);
    o.val = shfl_up_any(incl.val, d);
    if (lane >= d) incl = seg_combine<P>(o, incl);
  }
  if (lane == 31) sm.warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    SegVal<T> w;
    if (lane < NT / 32) {
      w = sm.warp[lane];
    } else {
      w.end = 0u;
      w.has = 0u;
      w.act = 0u;
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      SegVal<T> o;
      o.end = __shfl_up_sync(kFullMask, w.end, d);
      o.has = __shfl_up_sync(kFullMask, w.has, d);
      o.act = __shfl_up_sync(kFullMask, w.act, d);
      o.val = shfl_up_any(w.val, d);
      if (lane >= d) w = seg_combine<P>(o, w);
    }
    if (lane < NT / 32) sm.warp[lane] = w;
  }
  __syncthreads();
  SegVal<T> wpre;
  if (warp > 0) {
    wpre = sm.warp[warp - 1];
  } else {
    wpre.end = 0u;
    wpre.has = 0u;
    wpre.act = 0u;
  }
  SegVal<T> prev;
  prev.end = __shfl_up_sync(kFullMask, incl.end, 1);
  prev.has = __shfl_up_sync(kFullMask, incl.has, 1);
  prev.act = __shfl_up_sync(kFullMask, incl.act, 1);
  prev.val = shfl_up_any(incl.val, 1);
  if (lane == 0) {
    excl = wpre;
  } else {
    excl = (warp > 0) ? seg_combine<P>(wpre, prev) : prev;
  }
  total = sm.warp[NT / 32 - 1];
  __syncthreads();
}

// ---------------------------------------------------------------------------
// block_append: every thread offers up to K vertices in static slots
// ok[k] / vid[k] / deg[k] / beg[k] (deg = the degree the list's consumer
// walks, beg = that vertex's CSC/CSR begin offset).  The block reserves
// (count, degree sum) with one atomicAdd on the list's packed counter
// (count << 32 | degree sum), so positions and exclusive degree prefixes
// of all batches agree, raises the list's maximum degree with one
// atomicMax, and writes, for every consumer tile boundary b = t*TILE
// inside this batch's merged (entries + degrees) range, the number of
// entries whose end precedes b -- the merge-path split of tile t.
template <int NT, int K>
struct AppendSmem {
  int32_t vid[NT * K + 1];
  int32_t pre[NT * K + 1];
  int32_t beg[NT * K + 1];
  ScanU64Smem<NT> scan;
  unsigned long long base;
  unsigned maxd;
};

template <int NT, int K, int TILE, int KS>
__device__ __forceinline__ void block_append(const bool (&ok)[K], const int32_t (&vid)[K],
                                             const int32_t (&deg)[K], const int32_t (&beg)[K],
                                             const gas_vertex_list &out, int32_t maxSplit,
                                             int32_t capacity, unsigned *errWord,
                                             AppendSmem<NT, KS> &sm) {
  static_assert(K <= KS, "staging area too small");
  unsigned cnt = 0, esum = 0, dmax = 0;
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (ok[k]) {
      ++cnt;
      esum += (unsigned)deg[k];
      dmax = max(dmax, (unsigned)deg[k]);
    }
  if (threadIdx.x == 0) sm.maxd = 0u;
  unsigned long long mine = ((unsigned long long)cnt << 32) | esum;
  unsigned long long excl, total;
  block_exclusive_scan_u64<NT>(mine, excl, total, sm.scan);
  if (total == 0ull) return;  // block-uniform
  const unsigned wmax = __reduce_max_sync(kFullMask, dmax);
  if ((threadIdx.x & 31) == 0 && wmax) atomicMax(&sm.maxd, wmax);
  if (threadIdx.x == 0) sm.base = atomicAdd(out.count, total);
  int off = (int)(excl >> 32);
  int eoff = (int)(excl & 0xffffffffull);
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (ok[k]) {
      sm.vid[off] = vid[k];
      sm.pre[off] = eoff;
      sm.beg[off] = beg[k];
      ++off;
      eoff += deg[k];
    }
  const int R = (int)(total >> 32);
  const int Esum = (int)(total & 0xffffffffull);
  if (threadIdx.x == 0) sm.pre[R] = Esum;
  __syncthreads();
  if (threadIdx.x == 0 && sm.maxd) atomicMax(out.maxDeg, sm.maxd);
  const unsigned long long base = sm.base;
  const long long qpos = (long long)(base >> 32);
  const long long epos = (long long)(base & 0xffffffffull);
  if (qpos + R > capacity) {
    if (threadIdx.x == 0) atomicOr(errWord, GAS_DEVERR_CAPACITY);
    __syncthreads();
    return;
  }
  for (int m = threadIdx.x; m < R; m += NT) {
    out.vid[qpos + m] = sm.vid[m];
    out.pre[qpos + m] = (int32_t)(epos + sm.pre[m]);
    out.beg[qpos + m] = sm.beg[m];
  }
  // split hints for boundaries b in [D, D + R + Esum)
  const long long D = qpos + epos;
  const long long Dend = D + R + Esum;
  const long long tFirst = (D + TILE - 1) / TILE;
  const long long tLast = (Dend - 1) / TILE;
  for (long long tb = tFirst + threadIdx.x; tb <= tLast; tb += NT) {
    const long long b = tb * TILE - D;  // local diagonal of the boundary
    // count entries m whose end (local diagonal pre[m+1] + m) is < b
    int lo = 0, hi = R;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if ((long long)sm.pre[mid + 1] + mid < b)
        lo = mid + 1;
      else
        hi = mid;
    }
    if (tb < maxSplit) out.split[tb] = (int32_t)(qpos + lo);
  }
  __syncthreads();
}

// Adds a per-warp 64-bit value (lane 0's v) into *target with one atomic per
// block (per-warp atomics on one address serialise at its L2 slice).  Every
// thread of the block calls it; sm holds one word per warp and is free again
// after the block's next barrier.
__device__ __forceinline__ void block_add_u64(unsigned long long v, unsigned long long *target,
                                              unsigned long long *sm) {
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long s = 0ull;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sm[k];
    if (s) atomicAdd(target, s);
  }
}

// warp_append: block_append for one warp, without split hints (for lists
// whose consumer walks one thread per entry): the warp reserves its
// (count, degree sum) with one atomicAdd on the packed counter and every
// lane writes its own entries.  No shared memory, no block barrier.
// kMaxDeg false leaves the list's maximum degree alone (a consumer that
// knows every degree is small does not read it).
template <int K, bool kMaxDeg = true>
__device__ __forceinline__ void warp_append_list(const bool (&ok)[K], const int32_t (&vid)[K],
                                                 const int32_t (&deg)[K], const int32_t (&beg)[K],
                                                 const gas_vertex_list &out, int32_t capacity,
                                                 unsigned *errWord) {
  const int lane = threadIdx.x & 31;
  unsigned cnt = 0, esum = 0, dmax = 0;
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (ok[k]) {
      ++cnt;
      esum += (unsigned)deg[k];
      dmax = max(dmax, (unsigned)deg[k]);
    }
  const unsigned long long mine = ((unsigned long long)cnt << 32) | esum;
  unsigned long long incl = mine;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long o = __shfl_up_sync(kFullMask, incl, d);
    if (lane >= d) incl += o;
  }
  const unsigned long long total = __shfl_sync(kFullMask, incl, 31);
  if (total == 0ull) return;  // warp-uniform
  const unsigned wmax = __reduce_max_sync(kFullMask, dmax);
  unsigned long long base = 0ull;
  if (lane == 0) {
    base = atomicAdd(out.count, total);
    if (kMaxDeg) atomicMax(out.maxDeg, wmax);
  }
  base = __shfl_sync(kFullMask, base, 0);
  const unsigned long long excl = incl - mine;
  long long q = (long long)(base >> 32) + (long long)(excl >> 32);
  long long e = (long long)(base & 0xffffffffull) + (long long)(excl & 0xffffffffull);
  if ((long long)(base >> 32) + (long long)(total >> 32) > capacity) {
    if (lane == 0) atomicOr(errWord, GAS_DEVERR_CAPACITY);
    return;
  }
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (ok[k]) {
      out.vid[q] = vid[k];
      out.pre[q] = (int32_t)e;
      out.beg[q] = beg[k];
      ++q;
      e += deg[k];
    }
}

// block_append_list: warp_append_list with one atomic per block instead of
// one per warp (a large frontier's appends would otherwise serialise on the
// list counter): the warps' totals meet in shared memory, thread 0 reserves
// the block's range, and every lane writes its own entries.  No split
// hints, no staging of the entries.  Every thread of the block calls it.
template <int K, bool kMaxDeg = true>
__device__ __forceinline__ void block_append_list(const bool (&ok)[K], const int32_t (&vid)[K],
                                                  const int32_t (&deg)[K], const int32_t (&beg)[K],
                                                  const gas_vertex_list &out, int32_t capacity,
                                                  unsigned *errWord) {
  __shared__ unsigned long long sTot[32];
  __shared__ unsigned long long sBase[32];
  __shared__ unsigned sMax;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned cnt = 0, esum = 0, dmax = 0;
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (ok[k]) {
      ++cnt;
      esum += (unsigned)deg[k];
      dmax = max(dmax, (unsigned)deg[k]);
    }
  const unsigned long long mine = ((unsigned long long)cnt << 32) | esum;
  unsigned long long incl = mine;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long o = __shfl_up_sync(kFullMask, incl, d);
    if (lane >= d) incl += o;
  }
  const unsigned wmax = kMaxDeg ? __reduce_max_sync(kFullMask, dmax) : 0u;
  if (lane == 31) sTot[warp] = incl;
  if (kMaxDeg && threadIdx.x == 0) sMax = 0u;
  __syncthreads();
  if (kMaxDeg && lane == 0 && wmax) atomicMax(&sMax, wmax);
  if (threadIdx.x == 0) {
    unsigned long long run = 0ull;
    for (int w = 0; w < nw; ++w) {
      const unsigned long long t = sTot[w];
      sTot[w] = run;  // exclusive prefix of the warps' totals
      run += t;
    }
    unsigned long long base = 0ull;
    if (run) base = atomicAdd(out.count, run);
    sBase[0] = base;
    sBase[1] = run;
  }
  __syncthreads();
  const unsigned long long base = sBase[0], total = sBase[1];
  if (total == 0ull) return;  // block-uniform
  if (kMaxDeg && threadIdx.x == 0 && sMax) atomicMax(out.maxDeg, sMax);
  if ((long long)(base >> 32) + (long long)(total >> 32) > capacity) {
    if (threadIdx.x == 0) atomicOr(errWord, GAS_DEVERR_CAPACITY);
    return;
  }
  const unsigned long long off = sTot[warp] + (incl - mine);
  long long q = (long long)(base >> 32) + (long long)(off >> 32);
  long long e = (long long)(base & 0xffffffffull) + (long long)(off & 0xffffffffull);
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (ok[k]) {
      out.vid[q] = vid[k];
      out.pre[q] = (int32_t)e;
      out.beg[q] = beg[k];
      ++q;
      e += deg[k];
    }
}

}  // namespace detail
}  // namespace gas
