// Persistent run() kernel: every round of the GAS loop in one cooperative
// launch.
//
// The reference drives each round from the host with two or three device
// synchronisations (gpugas.h:435-437, 682-683, 717, 747-748) and 8-10
// launches; on a high-diameter graph (the 1024^2 lattice runs 2173 rounds)
// that latency dominates.  Here one kernel loops over rounds:
//
//   gather/apply tiles  -> grid barrier -> commit + scatter/activate tiles
//   -> grid barrier -> swap frontier, next round
//
// Tiles are assigned statically (tile t to block t mod grid, in increasing
// order per block); all blocks are co-resident (cooperative launch), so a
// tile's look-back only waits on tiles that are being processed.  Every
// wait is bounded: a barrier or look-back that gives up sets
// GAS_DEVERR_TIMEOUT and the kernel returns.
#pragma once

#include "gather.cuh"
#include "scatter.cuh"

namespace gas {
namespace detail {

// ~2-4 s of polling before a grid barrier reports a timeout
constexpr unsigned kBarrierSpinLimit = 1u << 25;

// Grid-wide barrier of a cooperative launch (bar[0] arrivals, bar[1]
// generation).  Returns false on timeout or when another block reported one.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned *errWord) {
  __shared__ unsigned s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned ok = 1u;
    __threadfence();
    const unsigned gen = ld_acquire(bar + 1);
    const unsigned arrived = atomicAdd(bar, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      st_release(bar + 1, gen + 1);
    } else {
      unsigned spins = 0;
      while (ld_acquire(bar + 1) == gen) {
        ++spins;
        if (spins > kBarrierSpinLimit ||
            ((spins & 4095u) == 0 && (ld_acquire(errWord) & GAS_DEVERR_TIMEOUT))) {
          atomicOr(errWord, GAS_DEVERR_TIMEOUT);
          ok = 0u;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0u;
}

template <class P>
union PersistentSmem {
  GatherSmem<P> g;
  ScatterSmem s;
};

template <class P>
__global__ void __launch_bounds__(kGNT) run_persistent_kernel(const gas_run_args ra) {
  __shared__ PersistentSmem<P> sm;
  gas_gather_args a = ra.g;
  ScatterArgs sa;
  sa.outOffsets = a.outOffsets;
  sa.outDests = ra.outDests;
  sa.inOffsets = a.inOffsets;
  sa.commit = a.haveGather;
  sa.vertexBytes = ra.vertexBytes;
  sa.vertexData = a.vertexData;
  sa.vertexNew = a.vertexNew;
  sa.rangeStart = a.rangeStart;
  sa.rangeCount = a.rangeCount;
  sa.maxGatherTiles = ra.maxGatherTiles;
  sa.capacity = a.capacity;
  sa.mark = ra.mark;
  sa.tileCounter = nullptr;
  sa.resetTile = nullptr;
  sa.resetScatCount = nullptr;
  sa.resetScatMaxDeg = nullptr;
  sa.errWord = a.errWord;
  sa.statSlot = nullptr;

  int cur = ra.cur, sidx = ra.sidx;
  bool rangeMode = a.rangeMode != 0;
  int r = 0;
  for (;; ++r) {
    if (ra.maxRounds > 0 && r >= ra.maxRounds) break;
    // ---- this round's frontier (final since the previous barrier)
    a.rangeMode = rangeMode ? 1 : 0;
    a.front = ra.frontL[cur];
    a.scat = ra.scatL[sidx];
    a.epoch = ra.epochBase + (unsigned)r;
    a.iteration = ra.g.iteration + r;
    int n, T;
    frontier_size(a, n, T);
    if (n == 0) break;  // uniform: every block read the same count
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      *ra.frontL[cur ^ 1].count = 0ull;  // appended by this round's scatter
      *ra.frontL[cur ^ 1].maxDeg = 0u;
      *ra.scatL[sidx ^ 1].count = 0ull;  // appended by the next round's gather
      *ra.scatL[sidx ^ 1].maxDeg = 0u;
    }
    // ---- gather/apply
    bool tpvG;
    const int ntG = gather_tiles(a, n, T, tpvG);
    for (int t = blockIdx.x; t < ntG; t += gridDim.x) {
      gather_dispatch<P>(a, t, n, T, tpvG, sm.g);
      __syncthreads();
    }
    if (!grid_barrier(ra.barrier, a.errWord)) break;
    // ---- commit + scatter/activate
    sa.scat = a.scat;
    sa.rangeMode = a.rangeMode;
    sa.frontVid = a.front.vid;
    sa.frontCount = a.front.count;
    sa.next = ra.frontL[cur ^ 1];
    sa.stamp = ra.stampBase + r;
    const unsigned long long sc = *a.scat.count;
    if (blockIdx.x == 0 && threadIdx.x == 0 && r < ra.maxStatRounds) {
      ra.stats[2 * (size_t)r] = ((unsigned long long)n << 32) | (unsigned)T;
      ra.stats[2 * (size_t)r + 1] = sc;
    }
    if (a.haveGather) commit_frontier(sa, n);
    int ns = (int)(sc >> 32);
    if (ns > a.capacity) ns = a.capacity;
    const int Ts = (int)(sc & 0xffffffffull);
    bool tpvS;
    const int ntS = scatter_tiles(sa.scat, ns, Ts, tpvS);
    for (int t = blockIdx.x; t < ntS; t += gridDim.x) {
      if (tpvS)
        tpv_scatter_tile(sa, t, ns, Ts, sm.s);
      else
        scatter_tile(sa, t, ns, Ts, sm.s);
      __syncthreads();
    }
    if (!grid_barrier(ra.barrier, a.errWord)) break;
    cur ^= 1;
    sidx ^= 1;
    rangeMode = false;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *ra.roundsOut = r;
}

}  // namespace detail
}  // namespace gas
