// Fused rounds for graphs whose in- and out-degrees are all <= 8
// (lattices, road networks): a thread per active vertex gathers, applies
// and activates its out-neighbours in one phase, so a round costs one grid
// barrier instead of two (gather -> barrier -> commit + scatter ->
// barrier).
//
// The frontier of a fused round is a bitmap of V bits.  Activation is one
// atomicOr per out-edge into the next round's bitmap (no return value, so
// nothing waits on it), which also deduplicates: no activation stamps, no
// list append, no counter that every warp contends for.  The round of
// stamp S reads bitmap S % 3, sets bits in bitmap (S + 1) % 3 and clears
// bitmap (S + 2) % 3 (every round of a run clears one ahead, whatever its
// kind, so the bitmap a round writes is always clean).  Each block owns the
// bitmap byte slots b, b + grid, b + 2 * grid, ... (interleaved, so a
// spatially clustered wavefront spreads over all blocks); it reads them, lists their
// set bits in shared memory with a block scan, and its threads take the
// listed vertices.  The first fused round after a list round (or a range)
// reads that list instead, dealing its entries across all blocks.  Round
// counts come from per-block sums of (active, in-edges, returned,
// out-edges), added once per block.
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

#include "dense.cuh"
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
  uint32_t *nextBits;   // the next round's frontier bitmap (activated vertices)
  const int32_t *ellIn;   // [V][width] in-neighbours, -1 after the last
  const int32_t *ellOut;  // [V][width] out-neighbours, -1 after the last
  const void *ellEd;      // [V][width] edge data of the in-edges
  int32_t width;          // 4 or 8
};

// A fused round's counts, added once per block.
struct FusedCounts {
  unsigned active, inEdges, ret, outEdges;
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

// A whole cell in one store per 16 bytes: the writer's slot and version
// change, the other slot is rewritten with the value it already holds, so a
// reader that sees any mix of the old and new words still takes the right
// value (it reads the unchanged slot unless the version it sees is older
// than this round, and then the slot that version names, also unchanged).
template <class VD>
__device__ __forceinline__ void store_cell(FusedCell<VD> *p, const FusedCell<VD> &c) {
  constexpr int N = (int)(sizeof(FusedCell<VD>) / 16);
  union {
    int4 w[N];
    FusedCell<VD> c;
  } u;
  u.c = c;
#pragma unroll
  for (int k = 0; k < N; ++k) reinterpret_cast<int4 *>(p)[k] = u.w[k];
}

// Sets the bits of out-neighbours out[0..W) (-1: none) in `bits`, one
// atomic per distinct bitmap word (a lattice vertex's left and right
// neighbours usually share one).  Returns the number of out-neighbours.
template <int W>
__device__ __forceinline__ unsigned set_out_bits(uint32_t *bits, const int32_t (&out)[W]) {
  unsigned n = 0u;
  if constexpr (W <= 4) {
    uint32_t mask[W];
#pragma unroll
    for (int j = 0; j < W; ++j) mask[j] = out[j] >= 0 ? 1u << (out[j] & 31) : 0u;
#pragma unroll
    for (int j = 1; j < W; ++j)
#pragma unroll
      for (int i = 0; i < j; ++i)
        if (mask[i] && mask[j] && (out[i] >> 5) == (out[j] >> 5)) {
          mask[i] |= mask[j];
          mask[j] = 0u;
        }
#pragma unroll
    for (int j = 0; j < W; ++j) {
      n += out[j] >= 0 ? 1u : 0u;
      if (mask[j]) atomicOr(bits + (out[j] >> 5), mask[j]);  // result unused: a reduction
    }
  } else {
#pragma unroll
    for (int j = 0; j < W; ++j)
      if (out[j] >= 0) {
        bit_set(bits, out[j]);
        ++n;
      }
  }
  return n;
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

// Row v of a fixed-width adjacency: W int32 as W / 4 16-byte loads.
template <int W>
__device__ __forceinline__ void load_row(const int32_t *rows, int v, int32_t (&out)[W]) {
  const int4 *p = reinterpret_cast<const int4 *>(rows) + (size_t)v * (W / 4);
#pragma unroll
  for (int q = 0; q < W / 4; ++q) {
    const int4 t = __ldg(p + q);
    out[4 * q] = t.x;
    out[4 * q + 1] = t.y;
    out[4 * q + 2] = t.z;
    out[4 * q + 3] = t.w;
  }
}

// Vertices vs[0..K) (vs[k] < 0: none) in a fused round, their loads
// interleaved: each gathers from its in-neighbours' cells, applies, writes
// its cell, and when apply returns true sets its out-neighbours' bits in the
// next frontier.  Rows of width W (fixed-width adjacency).
template <class P, int K, int W>
__device__ __forceinline__ void fused_vertices(const gas_gather_args &a, const FusedCtx &f,
                                               const int (&vs)[K], FusedCounts &c) {
  typedef typename P::VertexData VD;
  typedef typename P::GatherResult GR;
  typedef typename P::EdgeData ED;
  constexpr bool kQuadEd = !std::is_empty<ED>::value && sizeof(ED) == 4;
  int32_t outd[K][W], src[K][W];
  int32_t edw[K][kQuadEd ? W : 1];
  FusedCell<VD> cv[K];
  VD tmp[K];
  // one round trip: the rows and the vertex's own cell
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int v = vs[k] < 0 ? 0 : vs[k];
    if (vs[k] >= 0) {
      load_row<W>(f.ellOut, v, outd[k]);
      if (a.haveGather) {
        load_row<W>(f.ellIn, v, src[k]);
        if constexpr (kQuadEd) load_row<W>(reinterpret_cast<const int32_t *>(f.ellEd), v, edw[k]);
        cv[k] = load_cell(reinterpret_cast<const FusedCell<VD> *>(f.cells) + v);
      } else {
        tmp[k] = reinterpret_cast<const VD *>(f.vd)[v];
      }
    } else {
#pragma unroll
      for (int j = 0; j < W; ++j) outd[k][j] = src[k][j] = -1;
    }
  }
  if (a.haveGather) {
    // second round trip: the in-neighbours' cells
    VD sv[K][W];
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int j = 0; j < W; ++j)
        if (src[k][j] >= 0) sv[k][j] = fused_read<VD>(f, src[k][j]);
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (vs[k] < 0) continue;
      const int own = (int)(cv[k].ver & 1u);  // v is applied once per round: its word is still old
      VD t = own ? cv[k].s[1] : cv[k].s[0];
      GR acc = P::gatherZero;
      unsigned deg = 0u;
#pragma unroll
      for (int j = 0; j < W; ++j)
        if (src[k][j] >= 0) {
          const ED *ep;
          ED e;
          if constexpr (kQuadEd) {
            memcpy(&e, &edw[k][j], sizeof(ED));
            ep = &e;
          } else if constexpr (std::is_empty<ED>::value) {
            ep = nullptr;
          } else {
            ep = reinterpret_cast<const ED *>(f.ellEd) + (size_t)vs[k] * W + j;
          }
          acc = P::gatherReduce(acc, P::gatherMap(&t, &sv[k][j], ep));
          ++deg;
        }
      const bool r = do_apply<P>(&t, acc, a.iteration);
      FusedCell<VD> nc = cv[k];
      if (own)
        nc.s[0] = t;
      else
        nc.s[1] = t;
      nc.ver = (f.stamp << 1) | (uint32_t)(own ^ 1);
      store_cell(reinterpret_cast<FusedCell<VD> *>(f.cells) + vs[k], nc);
      ++c.active;
      c.inEdges += deg;
      if (r) {
        ++c.ret;
        c.outEdges += set_out_bits<W>(f.nextBits, outd[k]);
      }
    }
  } else {  // apply only: nothing reads other vertices, update in place
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (vs[k] < 0) continue;
      const GR gz = P::gatherZero;
      const bool r = do_apply<P>(&tmp[k], gz, a.iteration);
      reinterpret_cast<VD *>(f.vd)[vs[k]] = tmp[k];
      ++c.active;
      c.inEdges += (unsigned)(a.inOffsets[vs[k] + 1] - a.inOffsets[vs[k]]);
      if (r) {
        ++c.ret;
        c.outEdges += set_out_bits<W>(f.nextBits, outd[k]);
      }
    }
  }
}

// One vertex (width from the context).
template <class P>
__device__ __forceinline__ void fused_vertex(const gas_gather_args &a, const FusedCtx &f, int v,
                                             FusedCounts &c) {
  const int vs[1] = {v};
  if (f.width == 4)
    fused_vertices<P, 1, 4>(a, f, vs, c);
  else
    fused_vertices<P, 1, 8>(a, f, vs, c);
}

// A fused round whose frontier is a list (or the range of setActive): the
// entries dealt across all blocks (entry base + k * grid + block), so a
// frontier of a few tiles still spreads its loads over every SM.
template <class P>
__device__ __forceinline__ void fused_list_round(const gas_gather_args &a, const ScatterArgs &sa,
                                                 const FusedCtx &f, int n, int T, FusedCounts &c) {
  const int per = gridDim.x * blockDim.x;
  for (int base = 0; base < n; base += per) {
    const int i = base + (int)threadIdx.x * (int)gridDim.x + (int)blockIdx.x;
    if (i < n) {
      int v, pre, end, beg;
      front_entry(a, i, n, T, v, pre, end, beg);
      fused_vertex<P>(a, f, v, c);
    }
  }
}

// The shared-memory list of the vertices a block's threads take in one pass
// of fused_bits_round (at most 32 a thread), and its scan storage.
template <int NT>
struct FusedBitsSmem {
  int32_t vid[NT * 32];
  ScanU64Smem<NT> scan;
};

// A fused round whose frontier is bitmap `bits` (nWords words), owned by
// slot: slot s is byte lane s & 3 of the 32 consecutive words of group
// s >> 2 (vertices 1024 g + 32 i + 8 j .. + 7 for word i of the group), and
// block b owns slots b, b + grid, b + 2 * grid, ...  A warp takes four slots
// a pass, a lane one word of each (32 consecutive words: one coalesced
// load), so a thread's four bytes pack into one word and a pass lists at
// most 32 vertices a thread; a block scan of their bit counts places the set
// bits' vertices in shared memory, and the block's threads take them.
// Owning bytes rather than 32-bit words spreads a clustered wavefront more
// evenly: a block's round time grows with its vertex count, and on the
// 1024x1024 lattice the slowest block's count over the mean, weighted by
// round size, falls from 1.22 (words) to 1.10 (this layout; 1.06 for bytes
// dealt one by one, whose loads do not coalesce).  Every thread of the block
// calls it.
//
// The slots' bytes this thread takes in the pass that starts at k0, packed
// (byte q: slot blockIdx.x + grid * (k0 + 4 * warp + q), word lane of its
// group); 0 past the bitmap.
template <int NT>
__device__ __forceinline__ uint32_t fused_units(const uint32_t *bits, int nWords, int k0) {
  const long long G = gridDim.x;
  const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
  const long long nSlots = 4ll * ((nWords + 31) / 32);
  uint32_t packed = 0u;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const long long s = (long long)blockIdx.x + G * (k0 + 4 * warp + q);
    const long long w = 32 * (s >> 2) + lane;
    if (s < nSlots && w < nWords) packed |= ((bits[w] >> (8 * (int)(s & 3))) & 0xffu) << (8 * q);
  }
  return packed;
}

template <class P, int NT>
__device__ __forceinline__ void fused_bits_round(const gas_gather_args &a, const ScatterArgs &sa,
                                                 const FusedCtx &f, const uint32_t *bits, int nWords,
                                                 FusedBitsSmem<NT> &sm, FusedCounts &c,
                                                 bool haveFirst = false, uint32_t first = 0u) {
  const int G = gridDim.x;
  const int nSlots = 4 * ((nWords + 31) / 32);
  const int perBlock = (nSlots - (int)blockIdx.x + G - 1) / G;  // slots this block owns
  const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
  for (int k0 = 0; k0 < perBlock; k0 += 4 * (NT / 32)) {  // block-uniform
    // the first pass's units may have been loaded already (read together
    // with the previous round's counts)
    const uint32_t packed = (k0 == 0 && haveFirst) ? first : fused_units<NT>(bits, nWords, k0);
    const unsigned long long mine = (unsigned long long)__popc(packed);
    unsigned long long excl, total;
    block_exclusive_scan_u64<NT>(mine, excl, total, sm.scan);
    if (total == 0ull) continue;  // block-uniform (the scan ends with a barrier)
    int off = (int)excl;
    uint32_t rest = packed;
    while (rest) {
      const int p = __ffs(rest) - 1;
      rest &= rest - 1u;
      const int sl = (int)blockIdx.x + G * (k0 + 4 * warp + (p >> 3));
      sm.vid[off++] = 32 * (32 * (sl >> 2) + lane) + 8 * (sl & 3) + (p & 7);
    }
    __syncthreads();
    if (f.width == 4) {  // two listed vertices a thread, their loads interleaved
      for (int i = threadIdx.x; i < (int)total; i += 2 * NT) {
        const int vs[2] = {sm.vid[i], i + NT < (int)total ? sm.vid[i + NT] : -1};
        fused_vertices<P, 2, 4>(a, f, vs, c);
      }
    } else {
      for (int i = threadIdx.x; i < (int)total; i += NT) fused_vertex<P>(a, f, sm.vid[i], c);
    }
    __syncthreads();  // sm.vid is rewritten by the next pass
  }
}

// A frontier left in bitmap `bits` becomes the list `out` (in-degree
// prefix, CSC begin, the gather's tile splits and maximum degree), in
// vertex order per block: for a run that stops at maxRounds after a fused
// round, whose caller continues from a list.
template <int NT, int KS>
__device__ void compact_active(const uint32_t *bits, const int32_t *inOffsets, int32_t nVertices,
                               const gas_vertex_list &out, int32_t maxSplit, int32_t capacity,
                               unsigned *errWord, AppendSmem<NT, KS> &sm) {
  for (int base = blockIdx.x * NT; base < nVertices; base += gridDim.x * NT) {
    const int v = base + threadIdx.x;
    bool ok[1] = {false};
    int32_t ov[1] = {v}, od[1] = {0}, ob[1] = {0};
    if (v < nVertices && bit_test(bits, v)) {
      ok[0] = true;
      ob[0] = inOffsets[v];
      od[0] = inOffsets[v + 1] - ob[0];
    }
    block_append<NT, 1, GAS_GATHER_TILE>(ok, ov, od, ob, out, maxSplit, capacity, errWord, sm);
  }
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
