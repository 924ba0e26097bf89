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
// On graphs whose degrees are all <= 8 a round is one phase (fused.cuh):
// a thread per frontier vertex gathers, applies and activates, then one
// grid barrier.  Rounds whose predecessor activated many out-edges run dense (pull, see
// dense.cuh): one pass of degree-binned warp units and one barrier.
// Transitions build the other representation: list -> dense sets the
// scatter list's bits in the frontier bitmap, dense -> list compacts the
// bitmap into a scatter list and pushes it.  A list round whose frontier has many in-edges runs
// as a pull pass too, over the vertices the previous scatter marked.  A run
// that starts with every vertex active may run its leading dense rounds in
// run_dense_kernel, a kernel with a smaller register budget, first.
//
// Tiles are assigned statically (tile t to block t mod grid, in increasing
// order per block); all blocks are co-resident (cooperative launch), so a
// tile's look-back only waits on tiles that are being processed.  Every
// wait is bounded: a barrier or look-back that gives up sets
// GAS_DEVERR_TIMEOUT and the kernel returns.
#pragma once

#include "dense.cuh"
#include "edge_scatter.cuh"
#include "fused.cuh"
#include "gather.cuh"
#include "scatter.cuh"

namespace gas {
namespace detail {

// ~2-4 s of polling before a grid barrier reports a timeout
constexpr unsigned kBarrierSpinLimit = 1u << 25;

// Grid-wide barrier of a cooperative launch on one 32-bit word (bar[0],
// zero at launch; bar[1] unused).  Each block arrives with one atomic:
// block 0 adds 2^31 - (gridDim.x - 1), every other block adds 1, so the
// word's top bit flips exactly when the last block arrives, whichever that
// is, and the low bits return to their value before the barrier.  A block
// waits until the top bit differs from the one its own atomic returned: no
// second atomic on the release path.  The block whose atomic flips the bit
// (the last to arrive) sees that in the value its atomic returned and does
// not poll.  The arrival is an acquire-release atomic at GPU scope and the
// polling load an acquire: with the block barriers around them they order
// every thread's writes before the barrier ahead of every thread's reads
// after it, without a sequentially consistent fence on either side.
// Returns false on timeout or when another block reported one.
//
// barrier_thread0 is thread 0's part, between the block barriers.
__device__ __forceinline__ bool barrier_thread0(unsigned *bar, unsigned *errWord) {
  const unsigned add = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1u) : 1u;
  const unsigned old = atom_add_acq_rel(bar, add);
  if ((((old + add) ^ old) & 0x80000000u) != 0u) return true;  // the last arrival
  unsigned spins = 0;
  while (((ld_acquire(bar) ^ old) & 0x80000000u) == 0u) {
    ++spins;
    if (spins > kBarrierSpinLimit ||
        ((spins & 4095u) == 0 && (ld_acquire(errWord) & GAS_DEVERR_TIMEOUT))) {
      atomicOr(errWord, GAS_DEVERR_TIMEOUT);
      return false;
    }
    __nanosleep(32);
  }
  return true;
}

__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned *errWord) {
  __shared__ unsigned s_ok;
  __syncthreads();
  if (threadIdx.x == 0) s_ok = barrier_thread0(bar, errWord) ? 1u : 0u;
  __syncthreads();
  return s_ok != 0u;
}

// The grid barrier that closes a fused round, with the round's counts: the
// warps' sums meet in shared memory at the barrier's first block barrier,
// and thread 0 adds the block's totals into cnt[0] (active << 32 |
// in-edges) and cnt[1] (ret << 32 | out-edges) just before it arrives (one
// block barrier instead of one for the counts and one for the grid
// barrier).  Every thread of the block calls it with its own counts.
__device__ __forceinline__ bool fused_barrier(unsigned *bar, unsigned *errWord, const FusedCounts &c,
                                              unsigned long long *cnt) {
  __shared__ unsigned long long sA[32], sR[32];
  __shared__ unsigned s_ok;
  const unsigned wA = __reduce_add_sync(kFullMask, c.active);
  const unsigned wEin = __reduce_add_sync(kFullMask, c.inEdges);
  const unsigned wR = __reduce_add_sync(kFullMask, c.ret);
  const unsigned wEout = __reduce_add_sync(kFullMask, c.outEdges);
  if ((threadIdx.x & 31) == 0) {
    sA[threadIdx.x >> 5] = ((unsigned long long)wA << 32) | wEin;
    sR[threadIdx.x >> 5] = ((unsigned long long)wR << 32) | wEout;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long x = 0ull, y = 0ull;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      x += sA[k];
      y += sR[k];
    }
    if (x) atomicAdd(cnt, x);
    if (y) atomicAdd(cnt + 1, y);
    s_ok = barrier_thread0(bar, errWord) ? 1u : 0u;
  }
  __syncthreads();
  return s_ok != 0u;
}

template <class P>
union PersistentSmem {
  GatherSmem<P> g;
  ScatterSmem s;
  FusedBitsSmem<kGNT> fb;
};

// The fixed part of a dense pass's context (graph, degree bins, chunks).
__device__ __forceinline__ DenseCtx dense_ctx(const gas_run_args &ra) {
  DenseCtx dc;
  dc.nVertices = ra.g.nVertices;
  dc.nEdges = ra.g.nEdges;
  dc.inOffsets = ra.g.inOffsets;
  dc.inSources = ra.g.inSources;
  dc.outOffsets = ra.g.outOffsets;
  dc.edgeData = ra.g.edgeData;
  dc.binMid = ra.binMid;
  dc.binSmall = ra.binSmall;
  dc.binTiny = ra.binTiny;
  dc.nMid = ra.nMid;
  dc.nSmall = ra.nSmall;
  dc.nTiny = ra.nTiny;
  dc.chunkVertex = ra.chunkVertex;
  dc.chunkBegin = ra.chunkBegin;
  dc.chunkFirst = ra.chunkFirst;
  dc.chunkCount = ra.chunkCount;
  dc.chunkSlot = ra.chunkSlot;
  dc.nChunks = ra.nChunks;
  dc.chunkArrive = ra.chunkArrive;
  dc.chunkVal = ra.chunkVal;
  dc.chunkFlags = ra.chunkFlags;
  dc.haveGather = ra.g.haveGather;
  return dc;
}

// The frontier bitmap of the round with this stamp (null when the run has
// none: dense rounds disabled and no fused rounds).
__device__ __forceinline__ uint32_t *round_bits(const gas_run_args &ra, int32_t stamp) {
  return ra.retBits[0] ? ra.retBits[(unsigned)stamp % 3u] : nullptr;
}

// The active-set bitmap of the fused round with this stamp (see fused.cuh).
__device__ __forceinline__ uint32_t *front_bits(const gas_run_args &ra, int32_t stamp) {
  return ra.frontBits[(unsigned)stamp % 3u];
}

// Clears the bitmaps the rounds after this one write: the frontier bitmap
// of the next round (dense.cuh) and the active-set bitmap of the round after
// it (fused.cuh).  Every round of a run calls it, whatever its kind.
__device__ __forceinline__ void clear_ahead(const gas_run_args &ra, int32_t stamp) {
  if (ra.retBits[0]) clear_bits(round_bits(ra, stamp + 1), ra.bitWords);
  if (ra.frontBits[0]) clear_bits(front_bits(ra, stamp + 2), ra.bitWords);
}

// Round r's per-round settings of a dense pass over vdBuf[vcur]; with
// byMark, the active vertices are those round r-1's scatter marked; with
// actBits, those whose bits round r-1 (a fused round) set.
__device__ __forceinline__ void dense_round(DenseCtx &dc, const gas_run_args &ra, void *const vdBuf[2],
                                            int vcur, int r, bool allActive, bool byMark = false,
                                            const uint32_t *actBits = nullptr) {
  const int32_t stamp = ra.stampBase + r;
  dc.vdCur = vdBuf[vcur];
  dc.vdNext = vdBuf[vcur ^ 1];
  dc.prevBits = round_bits(ra, stamp - 1);
  dc.curBits = round_bits(ra, stamp);
  dc.allActive = allActive ? 1 : 0;
  dc.actMark = byMark ? ra.mark : nullptr;
  dc.markStamp = stamp - 1;
  dc.actBits = actBits;
  dc.skipBits = (allActive || byMark || actBits) ? 1 : 0;
  dc.iteration = ra.g.iteration + r;
  dc.cnt = ra.denseCnt + kDenseCntStride * (r % 3);
}

// Round-start resets by one thread: the lists this round appends to and the
// next round's dense counters.
__device__ __forceinline__ void round_resets(const gas_run_args &ra, int r, int cur, int sidx) {
  *ra.frontL[cur ^ 1].count = 0ull;  // appended by this round's scatter
  *ra.frontL[cur ^ 1].maxDeg = 0u;
  *ra.scatL[sidx ^ 1].count = 0ull;  // appended by the next round's gather
  *ra.scatL[sidx ^ 1].maxDeg = 0u;
  if (ra.denseCnt) {  // absent when dense rounds are disabled
    unsigned long long *nextCnt = ra.denseCnt + kDenseCntStride * ((r + 1) % 3);
    nextCnt[0] = 0ull;
    nextCnt[1] = 0ull;
    nextCnt[2] = 0ull;
  }
}

// Dense -> list transition at the end of dense round r (stamp): the
// vertices whose bits it set become scatL[sidx] (vertex order per block)
// and are pushed into frontL[cur ^ 1].  False when a grid barrier gave up.
template <class P>
__device__ __forceinline__ bool dense_to_list(const gas_run_args &ra, const gas_gather_args &a,
                                              ScatterArgs &sa, PersistentSmem<P> &sm, int r, int cur,
                                              int sidx) {
  const int32_t stamp = ra.stampBase + r;
  compact_ret<kGNT, kGVT>(round_bits(ra, stamp), a.outOffsets, a.nVertices, ra.scatL[sidx],
                          a.maxScatTiles, a.errWord, sm.g.app);
  if (!grid_barrier(ra.barrier, a.errWord)) return false;
  const unsigned long long sc = *ra.scatL[sidx].count;
  int ns = (int)(sc >> 32);
  if (ns > a.capacity) ns = a.capacity;
  const int Ts = (int)(sc & 0xffffffffull);
  sa.commit = 0;
  sa.scat = ra.scatL[sidx];
  sa.next = ra.frontL[cur ^ 1];
  sa.stamp = stamp;
  bool tpvS;
  const int ntS = scatter_tiles(sa.scat, ns, Ts, tpvS);
  for (int t = blockIdx.x; t < ntS; t += gridDim.x) {
    if (tpvS)
      tpv_scatter_tile(sa, t, ns, Ts, sm.s);
    else
      scatter_tile(sa, t, ns, Ts, sm.s);
    __syncthreads();
  }
  return grid_barrier(ra.barrier, a.errWord);
}

// A list round whose frontier has more than nEdges / kMarkPullFactor in-edges
// runs as a pull pass over the marked frontier.
constexpr long long kMarkPullFactor = 4;

// The leading dense rounds of a run that starts with every vertex active,
// in a kernel that holds nothing else: 40 registers a thread, 6 CTAs per SM
// (the main kernel's list-round code needs 64 or more).  It stops before
// the first list round and leaves ra.resume for the main kernel (resume[3]:
// 0 go on, 1 the run is over, 2 stopped at maxRounds before a dense round);
// the rounds, stamps, resets and statistics are the main kernel's own.
template <class P, int MinBlocks>
__global__ void __launch_bounds__(kGNT, MinBlocks) run_dense_kernel(const gas_run_args ra) {
  DenseCtx dc = dense_ctx(ra);
  void *const vdBuf[2] = {ra.g.vertexData, ra.vertexAlt};
  const long long E = ra.g.nEdges;
  int vcur = 0, r = 0, pending = 0, ended = 0;
  for (;;) {
    if (ra.maxRounds > 0 && r >= ra.maxRounds) {
      ended = 2;  // stopped before a dense round: its frontier is round r-1's stamps
      break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) round_resets(ra, r, ra.cur ^ (r & 1), ra.sidx ^ (r & 1));
    clear_ahead(ra, ra.stampBase + r);
    dense_round(dc, ra, vdBuf, vcur, r, r == 0);
    dense_pass<P>(dc);
    if (!grid_barrier(ra.barrier, ra.g.errWord)) {
      ended = 1;
      break;
    }
    const unsigned long long statA = dc.cnt[0], statR = dc.cnt[1];
    if ((statA >> 32) == 0) {  // no vertex was active: the run ended before this round
      ended = 1;
      break;
    }
    vcur ^= 1;
    if (blockIdx.x == 0 && threadIdx.x == 0 && r < ra.maxStatRounds) {
      ra.stats[2 * (size_t)r] = statA;
      ra.stats[2 * (size_t)r + 1] = statR;
    }
    ++r;
    const int nr = (int)(statR >> 32);
    const long long eout = (long long)(statR & 0xffffffffull);
    // Dense again when the out-edges of the vertices that returned true are
    // many (eout * alpha > E, as in the main kernel), and also when they
    // would activate about V / kMarkPullFactor vertices or more (eout *
    // kMarkPullFactor > V): a frontier that large has about E /
    // kMarkPullFactor in-edges at the graph's mean degree, and its list
    // round would be a pull pass anyway, after a list transition.
    const bool dense = ra.denseAlpha > 0 && nr > 0 &&
                       (eout * ra.denseAlpha > E ||
                        (ra.g.haveGather && eout * kMarkPullFactor > (long long)ra.g.nVertices));
    if (!dense) {
      pending = nr > 0 ? 1 : 0;  // else the next (list) round is empty
      ended = 1 - pending;
      break;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ra.resume[0] = r;
    ra.resume[1] = vcur;
    ra.resume[2] = pending;
    ra.resume[3] = ended;
  }
}

// MinBlocks CTAs of 256 threads per SM: the register budget a thread gets
// (2: 128, 3: 80, 4: 64).
template <class P, int MinBlocks = 3>
__global__ void __launch_bounds__(kGNT, MinBlocks) run_persistent_kernel(const gas_run_args ra) {
  enum { kList = 0, kDense = 1 };
  __shared__ PersistentSmem<P> sm;
  gas_gather_args a = ra.g;
  ScatterArgs sa;
  sa.outOffsets = a.outOffsets;
  sa.outDests = ra.outDests;
  sa.inOffsets = a.inOffsets;
  sa.vertexBytes = ra.vertexBytes;
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
  DenseCtx dc = dense_ctx(ra);
  void *vdBuf[2] = {a.vertexData, ra.vertexAlt};
  const long long E = a.nEdges;

  int cur = ra.cur, sidx = ra.sidx, vcur = 0;
  bool versioned = false;  // the vertex data lives in the fused cells
  bool frontBits = false;  // this round's active set is front_bits(stamp), not a list
  bool haveFirst = false;  // firstWord holds this thread's first-pass bytes of front_bits(stamp)
  uint32_t firstWord = 0u;
  bool capped = false;     // stopped at maxRounds
  bool rangeMode = a.rangeMode != 0;
  int mode = ra.allActive ? kDense : kList;
  bool allActive = ra.allActive != 0;
  int r = 0;
  bool ended = false;
  bool denseEnd = false;  // stopped at maxRounds before a dense round
  if (ra.denseFirst) {  // resume after run_dense_kernel's rounds
    r = ra.resume[0];
    vcur = ra.resume[1];
    ended = ra.resume[3] != 0;
    denseEnd = ra.resume[3] == 2;
    cur = ra.cur ^ (r & 1);
    sidx = ra.sidx ^ (r & 1);
    mode = kList;
    allActive = false;
    rangeMode = false;
    if (ra.resume[2] && !ended && !dense_to_list<P>(ra, a, sa, sm, r - 1, cur ^ 1, sidx ^ 1)) ended = true;
  }
  for (;;) {
    if (ended) break;
    if (ra.maxRounds > 0 && r >= ra.maxRounds) {
      denseEnd = mode == kDense;
      capped = true;
      break;
    }
    const unsigned epoch = ra.epochBase + (unsigned)r;
    const int32_t stamp = ra.stampBase + r;
    if (blockIdx.x == 0 && threadIdx.x == 0) round_resets(ra, r, cur, sidx);
    clear_ahead(ra, stamp);
    unsigned long long statA, statR;
    bool denseNext;
    bool byMark = false;  // a list round run as a pull pass over its marked frontier
    int n = 0, T = 0;
    unsigned frontMaxDeg = 0u;
    if (mode == kList) {
      a.rangeMode = rangeMode ? 1 : 0;
      a.front = ra.frontL[cur];
      a.scat = ra.scatL[sidx];
      a.epoch = epoch;
      a.iteration = ra.g.iteration + r;
      a.vertexData = vdBuf[vcur];
      if (!frontBits) {
        frontier_size(a, n, T);
        frontMaxDeg = frontier_max_degree(a);  // loaded together with the count
        if (n == 0) break;  // uniform: every block read the same count
        // A frontier whose in-edges are a large share of the graph gathers
        // faster in a pull pass that skips the unmarked vertices.
        byMark = r > 0 && !rangeMode && !versioned && a.haveGather && ra.denseAlpha > 0 &&
                 (long long)T * kMarkPullFactor > E;
      }
    }
    bool nextBits = false;  // the next round's active set is front_bits(stamp + 1)
    if (mode == kList && !byMark) {
      // ---------------- push round: list (or range) frontier, or a bitmap
      bool tpvG = true;
      const int ntG = frontBits ? 0 : gather_tiles(a, n, T, frontMaxDeg, tpvG);
      // fused rounds run in the instantiations of at most 2 CTAs per SM only
      // (launchRun launches them at 1)
      if (MinBlocks <= 2 && ra.fused && (frontBits || tpvG || !a.haveGather)) {
        // ---------------- fused round: one phase, one barrier
        FusedCtx f;
        f.cells = ra.fusedCells;
        f.vd = vdBuf[vcur];
        f.stamp = (uint32_t)stamp;
        f.nextBits = front_bits(ra, stamp + 1);
        f.ellIn = ra.ellIn;
        f.ellOut = ra.ellOut;
        f.ellEd = ra.ellEd;
        f.width = ra.ellWidth;
        if (a.haveGather && !versioned) {  // the vertex data moves into the cells
          fused_enter<P>(f, vdBuf[vcur], a.nVertices);
          versioned = true;
          if (!grid_barrier(ra.barrier, a.errWord)) break;
        }
        FusedCounts fc = {0u, 0u, 0u, 0u};
        if (frontBits)
          fused_bits_round<P, kGNT>(a, sa, f, front_bits(ra, stamp), ra.bitWords, sm.fb, fc,
                                    haveFirst, firstWord);
        else
          fused_list_round<P>(a, sa, f, n, T, fc);
        unsigned long long *cnt = ra.denseCnt + kDenseCntStride * (r % 3);
        if (!fused_barrier(ra.barrier, a.errWord, fc, cnt)) break;
        // the next round's bitmap is complete: this thread's first-pass
        // bytes of it are loaded together with the counts (independent round
        // trips in flight instead of one after the other)
        firstWord = fused_units<kGNT>(front_bits(ra, stamp + 1), ra.bitWords, 0);
        statA = cnt[0];
        statR = cnt[1];
        if ((statA >> 32) == 0) break;  // the bitmap was empty: the run ended before this round
        const int nr = (int)(statR >> 32);
        denseNext = ra.denseAlpha > 0 && nr > 0 &&
                    (long long)(statR & 0xffffffffull) * ra.denseAlpha > E;
        nextBits = true;
        if (denseNext && versioned) {  // dense rounds read the vertex data array
          fused_fold<P>(f, a.nVertices);
          versioned = false;
          if (!grid_barrier(ra.barrier, a.errWord)) break;
        }
      } else {
      if (versioned) {  // two-phase rounds read the vertex data array
        FusedCtx f;
        f.cells = ra.fusedCells;
        f.vd = vdBuf[vcur];
        fused_fold<P>(f, a.nVertices);
        versioned = false;
        if (!grid_barrier(ra.barrier, a.errWord)) break;
      }
      for (int t = blockIdx.x; t < ntG; t += gridDim.x) {
        gather_dispatch<P>(a, t, n, T, tpvG, sm.g);
        __syncthreads();
      }
      if (!grid_barrier(ra.barrier, a.errWord)) break;
      const unsigned long long sc = *a.scat.count;
      int ns = (int)(sc >> 32);
      if (ns > a.capacity) ns = a.capacity;
      const int Ts = (int)(sc & 0xffffffffull);
      statA = ((unsigned long long)n << 32) | (unsigned)T;
      statR = sc;
      denseNext = ra.denseAlpha > 0 && ns > 0 && (long long)Ts * ra.denseAlpha > E;
      sa.commit = a.haveGather;
      sa.vertexData = vdBuf[vcur];
      sa.scat = a.scat;
      sa.rangeMode = a.rangeMode;
      sa.frontVid = a.front.vid;
      sa.frontCount = a.front.count;
      sa.next = ra.frontL[cur ^ 1];
      sa.stamp = stamp;
      if (a.haveGather) commit_frontier(sa, n);
      if (denseNext) {
        bits_from_list(a.scat, ns, round_bits(ra, stamp));
      } else {
        bool tpvS;
        const int ntS = scatter_tiles(sa.scat, ns, Ts, tpvS);
        for (int t = blockIdx.x; t < ntS; t += gridDim.x) {
          if (tpvS)
            tpv_scatter_tile(sa, t, ns, Ts, sm.s);
          else
            scatter_tile(sa, t, ns, Ts, sm.s);
          __syncthreads();
        }
      }
      if constexpr (ProgramScatterEdges<P>::value) {
        if (ra.edgeScatter) {
          // Program::scatter sees the committed vertex data of every vertex
          if (!grid_barrier(ra.barrier, a.errWord)) break;
          edge_scatter_vertices<P>(a.scat.vid, ns, a.outOffsets, ra.outDests, ra.csr2csc,
                                   vdBuf[vcur], const_cast<void *>(a.edgeData));
        }
      }
      if (!grid_barrier(ra.barrier, a.errWord)) break;
      }  // two-phase round
    } else {
      // ---------------- pull round over every vertex
      dense_round(dc, ra, vdBuf, vcur, r, allActive, byMark, frontBits ? front_bits(ra, stamp) : nullptr);
      dense_pass<P>(dc);
      if (!grid_barrier(ra.barrier, a.errWord)) break;
      statA = dc.cnt[0];
      statR = dc.cnt[1];
      if ((statA >> 32) == 0) break;  // no vertex was active: the run ended before this round
      vcur ^= 1;
      const int nr = (int)(statR >> 32);
      const long long eout = (long long)(statR & 0xffffffffull);
      denseNext = ra.denseAlpha > 0 && nr > 0 && eout * ra.denseAlpha > E;
      if (!denseNext && nr > 0) {
        // dense -> list: compact the stamped vertices, then push them
        if (!dense_to_list<P>(ra, a, sa, sm, r, cur, sidx)) break;
      }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && r < ra.maxStatRounds) {
      ra.stats[2 * (size_t)r] = statA;
      ra.stats[2 * (size_t)r + 1] = statR;
    }
    ++r;
    haveFirst = nextBits && !denseNext;  // the next round is fused and reads that bitmap
    mode = denseNext ? kDense : kList;
    allActive = false;
    rangeMode = false;
    frontBits = nextBits;
    cur ^= 1;
    sidx ^= 1;
  }
  if (capped && frontBits) {
    // Stopped at maxRounds before a round whose active set is a bitmap:
    // the caller continues from a list, so the bitmap becomes frontL[cur].
    denseEnd = false;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      *ra.frontL[cur].count = 0ull;
      *ra.frontL[cur].maxDeg = 0u;
    }
    if (grid_barrier(ra.barrier, a.errWord))
      compact_active<kGNT, kGVT>(front_bits(ra, ra.stampBase + r), a.inOffsets, a.nVertices,
                                 ra.frontL[cur], ra.maxGatherTiles, a.capacity, a.errWord, sm.g.app);
  }
  if (versioned) {  // the newest values into the run's current buffer
    FusedCtx f;
    f.cells = ra.fusedCells;
    f.vd = vdBuf[vcur];
    fused_fold<P>(f, a.nVertices);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *ra.roundsOut = r;
    if (ra.vcurOut) *ra.vcurOut = vcur;
    if (ra.denseEndOut) *ra.denseEndOut = denseEnd ? 1 : 0;
  }
}

}  // namespace detail
}  // namespace gas
