// Core layer of the GB300 GAS engine (gas_gb300_core.h): device graph
// layout, frontier state, scatter/activate launches and the iteration loop.
//
// HBM layout per graph (int32 ids, as the reference's Int = int32_t):
//   inOffsets[V+1]  inSources[E]   CSC, gather side   (gpugas.h:100-103)
//   outOffsets[V+1] outDests[E]    CSR, scatter side  (gpugas.h:105-108)
//   edgeData[E]                    CSC order          (gpugas.h:259-263)
//   vertexData[V], vertexNew[V]    apply writes vertexNew, scatter commits
//   front{Vid,Pre}[2][V]           frontier lists (ids + in-degree prefix)
//   scat{Vid,Pre}[2][V]            vertices whose apply returned true
//   split arrays                   merge-path tile splits written by the
//                                  producer of each list
//   mark[V]                        round stamp of the last activation
//   carry{Val,Flag}[tiles]         published tile aggregates (look-back)
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "gas_gb300_core.h"
#include "gas_gb300/detail/dense.cuh"
#include "gas_gb300/detail/scatter.cuh"
#include "gas_internal.h"

using gas::detail::ScatterArgs;

namespace gas {
namespace internal {

thread_local std::string g_last_error;

gas_status fail(gas_status code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

gas_status cuda_fail(cudaError_t e, const char *what) {
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return fail(GAS_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
  }
  return fail(GAS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Stable counting sort of an edge list by `key` into offsets/adjacency
// (util.h:79-121 semantics; ties keep edge-list order).  perm[p] = edge
// index placed at position p.
void build_adjacency(int32_t nV, int32_t nE, const int32_t *key, const int32_t *other,
                     std::vector<int32_t> &off, std::vector<int32_t> &adj,
                     std::vector<int32_t> *perm) {
  off.assign((size_t)nV + 1, 0);
  for (int32_t i = 0; i < nE; ++i) off[(size_t)key[i] + 1]++;
  for (int32_t v = 0; v < nV; ++v) off[(size_t)v + 1] += off[v];
  std::vector<int32_t> cur(off.begin(), off.end() - 1);
  adj.resize((size_t)std::max(nE, 1));
  if (perm) perm->resize((size_t)std::max(nE, 1));
  for (int32_t i = 0; i < nE; ++i) {
    const int32_t p = cur[key[i]]++;
    adj[p] = other[i];
    if (perm) (*perm)[p] = i;
  }
}

}  // namespace internal
}  // namespace gas

using namespace gas::internal;

namespace {

struct ListCtl {
  unsigned long long cnt;  // (count << 32) | degree total
  unsigned maxd;           // largest degree in the list
  unsigned pad;
};

struct Ctl {
  ListCtl f[2];  // frontier lists
  ListCtl s[2];  // scatter lists
  unsigned tile[2];
  unsigned bar[2];  // persistent-kernel grid barrier: arrival word, unused
  int32_t rounds;   // rounds executed by the last persistent run
  int32_t vcur;     // 1 when that run's result is in the alternate buffer
  int32_t denseEnd; // 1 when that run stopped before a dense round (gas_run_args::denseEndOut)
  int32_t pad0;
  unsigned long long dense[3][4];  // per-round counters of dense rounds (kDenseCntStride)
  unsigned err;     // device error bits (kept across set_active)
  unsigned pad;
  int32_t resume[4];  // hand-over of a leading dense-rounds kernel (gas_run_args::resume)
};

enum DirtyBit : unsigned {
  kF0 = 1u, kF1 = 2u, kS0 = 4u, kS1 = 8u, kT0 = 16u, kT1 = 32u,
};

constexpr int kRing = 8;
constexpr int kLag = 3;
constexpr int kMaxRounds = 1 << 16;

template <typename T>
cudaError_t dalloc(T **p, size_t count) {
  return cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(count, 1));
}

}  // namespace

// Fixed-width rows of an adjacency (offsets, indices; optional per-edge
// bytes): row v holds v's first `width` indices in order, -1 after the last
// (zero bytes for the edge data there).
__global__ void ell_rows_kernel(int32_t nV, const int32_t *off, const int32_t *idx, const void *ed,
                                int32_t edgeBytes, int32_t width, int32_t *rows, void *edRows) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nV;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t b = off[v], d = off[v + 1] - b;
    for (int k = 0; k < width; ++k) {
      rows[v * width + k] = k < d ? idx[b + k] : -1;
      if (edRows) {
        unsigned char *dst = static_cast<unsigned char *>(edRows) + (v * width + k) * edgeBytes;
        const unsigned char *src = static_cast<const unsigned char *>(ed) + (int64_t)(b + k) * edgeBytes;
        for (int32_t x = 0; x < edgeBytes; ++x) dst[x] = k < d ? src[x] : 0;
      }
    }
  }
}

// The counters, barrier words and round-0 bitmaps a persistent run starts
// from, zeroed by one launch instead of one memset each.
struct ZeroSegments {
  static constexpr int kMax = 8;
  uint32_t *ptr[kMax];
  int32_t words[kMax];
  int32_t n;
};

__global__ void zero_segments_kernel(ZeroSegments z) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int s = 0; s < z.n; ++s)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < z.words[s]; i += stride)
      z.ptr[s][i] = 0u;
}

struct gas_core_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  int numSMs = 0;
  int scatterGrid = 0;
  // graph
  bool haveGraph = false;
  int32_t nV = 0, nE = 0;
  int32_t edgeBytes = 0, vertexBytes = 0, gatherBytes = 0;
  std::vector<int32_t> hInOff, hOutOff;
  uint32_t *cscPerm = nullptr;  // [E] edge index at each CSC position (when EdgeData is not empty)
  uint32_t *csrPerm = nullptr;  // [E] the same for the CSR, kept on request
  bool keepCsrPerm = false;
  int32_t *csr2csc = nullptr;   // [E] CSC position of each CSR edge (Program::scatter)
  void *fcell = nullptr;        // [V] cells of fused rounds (fused.cuh), fused-eligible graphs only
  int32_t *ellIn = nullptr, *ellOut = nullptr;  // fixed-width adjacency rows (fused graphs)
  void *ellEd = nullptr;
  int32_t ellWidth = 0;
  int32_t maxOutDeg = 0;
  bool fusedRounds = true;      // one-phase rounds when every degree is <= 8
  bool edgeScatterOn = false;   // keep csr2csc and run scatter-capable rounds
  bool edgeScatterReady = false;  // a scatter list awaits the Program's scatter
  int32_t *inOff = nullptr, *inSrc = nullptr, *outOff = nullptr, *outDst = nullptr;
  void *ed = nullptr;
  void *vd = nullptr, *vnew = nullptr, *vsaved = nullptr, *valt = nullptr;
  uint32_t *retBits = nullptr;  // three frontier bitmaps of bitWords words
  uint32_t *frontBits = nullptr;  // three active-set bitmaps of the fused rounds
  int32_t bitWords = 0;
  // degree bins of the dense pass (see dense.cuh)
  int32_t *binMid = nullptr, *binSmall = nullptr, *binTiny = nullptr;
  int32_t nMid = 0, nSmall = 0, nTiny = 0;
  int32_t *chunkVertex = nullptr, *chunkBegin = nullptr, *chunkFirst = nullptr;
  int32_t *chunkCount = nullptr, *chunkSlot = nullptr;
  int32_t nChunks = 0, nChunkVertices = 0;
  unsigned *chunkArrive = nullptr, *chunkFlags = nullptr;
  void *chunkVal = nullptr;
  int32_t denseAlpha = 10;  // dense (pull) round when out-edges * alpha > E
  int32_t *fvid[2] = {nullptr, nullptr}, *fpre[2] = {nullptr, nullptr};
  int32_t *fbeg[2] = {nullptr, nullptr};
  int32_t *fsplit[2] = {nullptr, nullptr}, *rsplit = nullptr;
  int32_t *svid[2] = {nullptr, nullptr}, *spre[2] = {nullptr, nullptr};
  int32_t *sbeg[2] = {nullptr, nullptr};
  int32_t *ssplit[2] = {nullptr, nullptr};
  int32_t maxInDeg = 0;
  int32_t *mark = nullptr;
  void *carryVal = nullptr;
  unsigned *carryFlag = nullptr;
  Ctl *ctl = nullptr;
  unsigned long long *stats = nullptr;
  int32_t maxGatherTiles = 0, maxScatTiles = 0;
  // protocol state
  int cur = 0, sidx = 0;
  bool rangeMode = true;
  int32_t rstart = 0, rcount = 0;
  bool pendingCommit = false;
  bool haveScatList = false;
  bool countValid = false;
  int32_t countCache = 0;
  // A persistent run that stopped at maxIters before a dense round leaves
  // its next frontier as the bits of the round densePendStamp (bitmap
  // densePendStamp % 3); materialize() turns it into a list when a later
  // call needs one.
  bool densePending = false;
  int32_t densePendStamp = 0;
  unsigned dirty = 0;
  unsigned epoch = 0;
  int32_t stamp = 0;
  int32_t iteration = 0;
  int32_t round = 0;
  // run bookkeeping
  unsigned long long *pinned = nullptr;
  cudaEvent_t ev[kRing] = {};
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  float lastMs = 0.f;
  // optional per-kernel profile of run()
  bool profiling = false;
  std::vector<cudaEvent_t> pev;  // 4 per round: gather start/end, scatter start/end
  float gatherMs = 0.f, scatterMs = 0.f;
  int32_t gatherLaunches = 0, scatterLaunches = 0;
};

// The frontier bitmap of the round with this stamp (three rotate, see
// gas_run_args::retBits).
static uint32_t *round_bits(gas_core_s *c, int32_t stamp) {
  return c->retBits + (size_t)((unsigned)stamp % 3u) * c->bitWords;
}

namespace {

void free_graph(gas_core *c) {
  void *ptrs[] = {c->inOff, c->inSrc, c->outOff, c->outDst, c->ed, c->vd, c->vnew, c->vsaved,
                  c->valt, c->retBits, c->frontBits, c->binMid, c->binSmall,
                  c->binTiny, c->chunkVertex, c->chunkBegin, c->chunkFirst, c->chunkCount,
                  c->chunkSlot, c->chunkArrive, c->chunkFlags, c->chunkVal,
                  c->fvid[0], c->fvid[1], c->fpre[0], c->fpre[1], c->fsplit[0], c->fsplit[1],
                  c->fbeg[0], c->fbeg[1], c->sbeg[0], c->sbeg[1],
                  c->rsplit, c->svid[0], c->svid[1], c->spre[0], c->spre[1], c->ssplit[0],
                  c->ssplit[1], c->mark, c->carryVal, c->carryFlag, c->ctl, c->stats,
                  c->cscPerm, c->csrPerm, c->csr2csc, c->fcell, c->ellIn, c->ellOut, c->ellEd};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  c->cscPerm = c->csrPerm = nullptr;
  c->csr2csc = nullptr;
  c->fcell = nullptr;
  c->ellIn = c->ellOut = nullptr;
  c->ellEd = nullptr;
  c->ellWidth = 0;
  c->inOff = c->inSrc = c->outOff = c->outDst = nullptr;
  c->ed = c->vd = c->vnew = c->vsaved = c->valt = nullptr;
  c->retBits = nullptr;
  c->frontBits = nullptr;
  c->binMid = c->binSmall = c->binTiny = nullptr;
  c->chunkVertex = c->chunkBegin = c->chunkFirst = c->chunkCount = c->chunkSlot = nullptr;
  c->chunkArrive = c->chunkFlags = nullptr;
  c->chunkVal = nullptr;
  c->nMid = c->nSmall = c->nTiny = c->nChunks = c->nChunkVertices = 0;
  for (int k = 0; k < 2; ++k) {
    c->fvid[k] = c->fpre[k] = c->fbeg[k] = c->fsplit[k] = nullptr;
    c->svid[k] = c->spre[k] = c->sbeg[k] = c->ssplit[k] = nullptr;
  }
  c->rsplit = nullptr;
  c->mark = nullptr;
  c->carryVal = nullptr;
  c->carryFlag = nullptr;
  c->ctl = nullptr;
  c->stats = nullptr;
  c->haveGraph = false;
}

gas_status set_device(gas_core *c) {
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  return GAS_OK;
}

gas_status clean(gas_core *c, unsigned need) {
  unsigned d = c->dirty & need;
  if (!d) return GAS_OK;
  struct {
    unsigned bit;
    void *ptr;
    size_t bytes;
  } m[] = {{kF0, &c->ctl->f[0], sizeof(ListCtl)}, {kF1, &c->ctl->f[1], sizeof(ListCtl)},
           {kS0, &c->ctl->s[0], sizeof(ListCtl)}, {kS1, &c->ctl->s[1], sizeof(ListCtl)},
           {kT0, &c->ctl->tile[0], 4}, {kT1, &c->ctl->tile[1], 4}};
  for (auto &x : m)
    if (d & x.bit) {
      cudaError_t e = cudaMemsetAsync(x.ptr, 0, x.bytes, c->stream);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    }
  c->dirty &= ~d;
  return GAS_OK;
}

unsigned fbit(int k) { return k ? kF1 : kF0; }
unsigned sbit(int k) { return k ? kS1 : kS0; }

gas_vertex_list front_list(gas_core *c, int k) {
  gas_vertex_list l;
  l.vid = c->fvid[k];
  l.pre = c->fpre[k];
  l.beg = c->fbeg[k];
  l.split = c->fsplit[k];
  l.count = &c->ctl->f[k].cnt;
  l.maxDeg = &c->ctl->f[k].maxd;
  return l;
}

gas_vertex_list scat_list(gas_core *c, int k) {
  gas_vertex_list l;
  l.vid = c->svid[k];
  l.pre = c->spre[k];
  l.beg = c->sbeg[k];
  l.split = c->ssplit[k];
  l.count = &c->ctl->s[k].cnt;
  l.maxDeg = &c->ctl->s[k].maxd;
  return l;
}

// A frontier left as round stamps (densePending) becomes the list f[cur]:
// the stamped vertices are compacted into s[sidx] and pushed, as the
// persistent kernel's dense -> list transition does.
gas_status materialize(gas_core *c) {
  if (!c->densePending) return GAS_OK;
  c->densePending = false;
  gas_status st = clean(c, sbit(c->sidx) | fbit(c->cur) | kT0 | kT1);
  if (st) return st;
  gas::detail::compact_ret_kernel<<<c->scatterGrid, 256, 0, c->stream>>>(
      round_bits(c, c->densePendStamp), c->outOff, c->nV, scat_list(c, c->sidx),
      c->maxScatTiles, &c->ctl->err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "frontier compaction launch");
  if (++c->stamp == 0x7fffffff) {
    cudaMemsetAsync(c->mark, 0, sizeof(int32_t) * std::max(c->nV, 1), c->stream);
    c->stamp = 1;
  }
  gas::detail::ScatterArgs a;
  memset(&a, 0, sizeof(a));
  a.outOffsets = c->outOff;
  a.outDests = c->outDst;
  a.inOffsets = c->inOff;
  a.scat = scat_list(c, c->sidx);
  a.commit = 0;
  a.vertexBytes = c->vertexBytes;
  a.vertexData = c->vd;
  a.vertexNew = c->vnew;
  a.next = front_list(c, c->cur);
  a.maxGatherTiles = c->maxGatherTiles;
  a.capacity = c->nV;
  a.mark = c->mark;
  a.stamp = c->stamp;
  a.tileCounter = &c->ctl->tile[1];
  a.resetTile = &c->ctl->tile[0];
  a.resetScatCount = &c->ctl->s[c->sidx ^ 1].cnt;
  a.resetScatMaxDeg = &c->ctl->s[c->sidx ^ 1].maxd;
  a.errWord = &c->ctl->err;
  gas::detail::scatter_activate_kernel<<<c->scatterGrid, gas::detail::kSNT, 0, c->stream>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "frontier push launch");
  c->dirty |= sbit(c->sidx) | kT1;
  c->dirty &= ~(fbit(c->cur) | kT0 | sbit(c->sidx ^ 1));
  c->rangeMode = false;
  c->countValid = false;
  c->pendingCommit = false;
  c->haveScatList = false;
  return GAS_OK;
}

gas_status check_device_error(gas_core *c) {
  unsigned err = 0;
  cudaError_t e = cudaMemcpyAsync(&err, &c->ctl->err, sizeof(err), cudaMemcpyDeviceToHost,
                                  c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "device sync");
  if (err) {
    cudaMemsetAsync(&c->ctl->err, 0, sizeof(unsigned), c->stream);
    if (err & GAS_DEVERR_TIMEOUT)
      return fail(GAS_ERR_TIMEOUT, "a bounded device wait (tile look-back) timed out");
    return fail(GAS_ERR_STATE, "device list capacity exceeded (error bits 0x%x)", err);
  }
  return GAS_OK;
}

}  // namespace

namespace gas {
namespace internal {
void core_keep_csr_perm(gas_core_s *c, bool keep) {
  c->keepCsrPerm = keep;
  if (!keep && c->csrPerm) {
    cudaFree(c->csrPerm);
    c->csrPerm = nullptr;
  }
}

gas_status core_permute_csr(gas_core_s *c, const int32_t *hostVals, int32_t **devOut) {
  *devOut = nullptr;
  if (!c || !c->haveGraph || !c->csrPerm) return fail(GAS_ERR_STATE, "no CSR permutation kept");
  const size_t n = (size_t)std::max(c->nE, 1);
  int32_t *tmp = nullptr, *out = nullptr;
  cudaError_t e = cudaMalloc(&tmp, 4 * n);
  if (e == cudaSuccess) e = cudaMalloc(&out, 4 * n);
  if (e == cudaSuccess && c->nE > 0)
    e = cudaMemcpyAsync(tmp, hostVals, 4 * (size_t)c->nE, cudaMemcpyHostToDevice, c->stream);
  gas_status st = e == cudaSuccess ? device_gather_bytes(c->stream, tmp, c->csrPerm, c->nE, 4, out)
                                   : cuda_fail(e, "CSR permutation");
  if (st == GAS_OK) {
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) st = cuda_fail(e, "CSR permutation");
  }
  if (tmp) cudaFree(tmp);
  if (st != GAS_OK) {
    if (out) cudaFree(out);
    return st;
  }
  *devOut = out;
  return GAS_OK;
}

bool core_graph(gas_core_s *c, CoreGraph *out) {
  if (!c || !c->haveGraph) return false;
  out->device = c->device;
  out->stream = c->stream;
  out->nV = c->nV;
  out->nE = c->nE;
  out->inOff = c->inOff;
  out->inSrc = c->inSrc;
  out->outOff = c->outOff;
  out->outDst = c->outDst;
  out->edgeData = c->ed;
  out->edgeBytes = c->edgeBytes;
  out->hInOff = &c->hInOff;
  out->hOutOff = &c->hOutOff;
  return true;
}
}  // namespace internal
}  // namespace gas

extern "C" {

gas_status gas_core_create(int32_t device, void *stream, gas_core **out) {
  if (!out) return fail(GAS_ERR_INVALID, "gas_core_create: out is NULL");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return fail(GAS_ERR_NO_DEVICE, "no CUDA device %d", device);
  }
  gas_core *c = new (std::nothrow) gas_core_s();
  if (!c) return fail(GAS_ERR_OOM, "host allocation");
  c->device = device;
  c->stream = (cudaStream_t)stream;
  if (set_device(c) != GAS_OK) {
    delete c;
    return GAS_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&c->numSMs, cudaDevAttrMultiProcessorCount, device);
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, gas::detail::scatter_activate_kernel,
                                                gas::detail::kSNT, 0);
  c->scatterGrid = std::max(1, per) * std::max(1, c->numSMs);
  e = cudaMallocHost((void **)&c->pinned, sizeof(unsigned long long) * kRing);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaMallocHost");
  }
  for (int k = 0; k < kRing; ++k) cudaEventCreateWithFlags(&c->ev[k], cudaEventDisableTiming);
  cudaEventCreate(&c->t0);
  cudaEventCreate(&c->t1);
  *out = c;
  return GAS_OK;
}

gas_status gas_core_destroy(gas_core *c) {
  if (!c) return GAS_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_graph(c);
  for (int k = 0; k < kRing; ++k)
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
  for (cudaEvent_t ev : c->pev) cudaEventDestroy(ev);
  if (c->t0) cudaEventDestroy(c->t0);
  if (c->t1) cudaEventDestroy(c->t1);
  if (c->pinned) cudaFreeHost(c->pinned);
  delete c;
  return GAS_OK;
}

gas_status gas_core_stream(gas_core *c, void **stream) {
  if (!c || !stream) return fail(GAS_ERR_INVALID, "gas_core_stream: null argument");
  *stream = (void *)c->stream;
  return GAS_OK;
}

gas_status gas_core_set_graph(gas_core *c, int32_t nV, int32_t nE, const int32_t *srcs,
                              const int32_t *dsts, const void *edgeData, int32_t edgeBytes,
                              int32_t vertexBytes, int32_t gatherBytes) {
  if (!c) return fail(GAS_ERR_INVALID, "gas_core_set_graph: engine is NULL");
  if (nV < 0 || nE < 0) return fail(GAS_ERR_INVALID, "negative vertex or edge count");
  if (nE > 0 && (!srcs || !dsts)) return fail(GAS_ERR_INVALID, "edge list is NULL");
  if (edgeBytes < 0 || vertexBytes <= 0 || gatherBytes <= 0)
    return fail(GAS_ERR_INVALID, "bad element sizes");
  if (edgeBytes > 0 && nE > 0 && !edgeData)
    return fail(GAS_ERR_INVALID, "edge data is NULL but EdgeData is not empty");
  if ((long long)nV + nE + 2LL * GAS_GATHER_TILE >= (1LL << 31))
    return fail(GAS_ERR_UNSUPPORTED, "vertices + edges must stay below 2^31 (int32 ids)");
  gas_status st = set_device(c);
  if (st) return st;
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_graph(c);

  // the edge list on the device: id check, then CSC (gather) and CSR
  // (scatter) by stable radix sorts (gas_graph_build.cu)
  int32_t *dS = nullptr, *dD = nullptr;
  cudaError_t e0 = dalloc(&dS, (size_t)nE);
  if (e0 == cudaSuccess) e0 = dalloc(&dD, (size_t)nE);
  if (e0 == cudaSuccess && nE > 0)
    e0 = cudaMemcpyAsync(dS, srcs, sizeof(int32_t) * nE, cudaMemcpyHostToDevice, c->stream);
  if (e0 == cudaSuccess && nE > 0)
    e0 = cudaMemcpyAsync(dD, dsts, sizeof(int32_t) * nE, cudaMemcpyHostToDevice, c->stream);
  auto drop_list = [&] {
    if (dS) cudaFree(dS);
    if (dD) cudaFree(dD);
  };
  if (e0 != cudaSuccess) {
    drop_list();
    return cuda_fail(e0, "setGraph edge list upload");
  }
  long long bad = -1;
  st = device_first_bad_edge(c->stream, nV, nE, dS, dD, &bad);
  if (st == GAS_OK && bad >= 0)
    st = fail(GAS_ERR_INVALID, "edge %lld (%d -> %d) has a vertex id outside [0, %d)", bad,
              srcs[bad], dsts[bad], nV);
  if (st) {
    drop_list();
    return st;
  }

  c->nV = nV;
  c->nE = nE;
  c->edgeBytes = edgeBytes;
  c->vertexBytes = vertexBytes;
  c->gatherBytes = gatherBytes;
  c->maxGatherTiles = (int32_t)(((long long)nV + nE) / GAS_GATHER_TILE + 2);
  c->maxScatTiles = (int32_t)(((long long)nV + nE) / GAS_SCATTER_TILE + 2);

  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  A(dalloc(&c->inOff, (size_t)nV + 1));
  // whole 16-byte quads: the dense pass reads source ids (and 4-byte edge
  // data) four at a time, up to the quad that holds a vertex's last edge
  A(dalloc(&c->inSrc, (size_t)nE + 4));
  A(dalloc(&c->outOff, (size_t)nV + 1));
  A(dalloc(&c->outDst, (size_t)nE));
  if (edgeBytes > 0) A(cudaMalloc(&c->ed, (size_t)edgeBytes * ((size_t)nE + 4)));
  if (edgeBytes > 0) A(dalloc(&c->cscPerm, (size_t)nE));
  const bool edgeMap = c->edgeScatterOn && edgeBytes > 0;
  if (c->keepCsrPerm || edgeMap) A(dalloc(&c->csrPerm, (size_t)nE));
  if (edgeMap) A(dalloc(&c->csr2csc, (size_t)nE));
  if (e == cudaSuccess) {
    st = device_build_adjacency(c->stream, nV, nE, dD, dS, c->inOff, c->inSrc, c->cscPerm);
    if (st == GAS_OK)
      st = device_build_adjacency(c->stream, nV, nE, dS, dD, c->outOff, c->outDst, c->csrPerm);
    if (st == GAS_OK && edgeMap)
      st = device_csr_to_csc(c->stream, nE, c->cscPerm, c->csrPerm, c->csr2csc);
    if (st == GAS_OK && edgeBytes > 0 && nE > 0) {
      void *dEd = nullptr;
      A(cudaMalloc(&dEd, (size_t)edgeBytes * nE));
      A(cudaMemcpyAsync(dEd, edgeData, (size_t)edgeBytes * nE, cudaMemcpyHostToDevice, c->stream));
      if (e == cudaSuccess) st = device_gather_bytes(c->stream, dEd, c->cscPerm, nE, edgeBytes, c->ed);
      A(cudaStreamSynchronize(c->stream));
      if (dEd) cudaFree(dEd);
    }
    c->hInOff.resize((size_t)nV + 1);
    c->hOutOff.resize((size_t)nV + 1);
    A(cudaMemcpyAsync(c->hInOff.data(), c->inOff, sizeof(int32_t) * ((size_t)nV + 1),
                      cudaMemcpyDeviceToHost, c->stream));
    A(cudaMemcpyAsync(c->hOutOff.data(), c->outOff, sizeof(int32_t) * ((size_t)nV + 1),
                      cudaMemcpyDeviceToHost, c->stream));
    A(cudaStreamSynchronize(c->stream));
  }
  drop_list();
  if (st != GAS_OK || e != cudaSuccess) {
    free_graph(c);
    return st != GAS_OK ? st : cuda_fail(e, "setGraph build");
  }
  if (edgeMap && !c->keepCsrPerm) {  // only the composed map is needed
    cudaFree(c->csrPerm);
    c->csrPerm = nullptr;
  }
  A(cudaMalloc(&c->vd, (size_t)vertexBytes * std::max(nV, 1)));
  A(cudaMalloc(&c->vnew, (size_t)vertexBytes * std::max(nV, 1)));
  A(cudaMalloc(&c->valt, (size_t)vertexBytes * std::max(nV, 1)));
  c->bitWords = (nV + 31) / 32;
  A(dalloc(&c->retBits, 3 * (size_t)c->bitWords));
  c->maxInDeg = 0;
  c->maxOutDeg = 0;
  for (int32_t v = 0; v < nV; ++v) {
    c->maxInDeg = std::max(c->maxInDeg, c->hInOff[(size_t)v + 1] - c->hInOff[v]);
    c->maxOutDeg = std::max(c->maxOutDeg, c->hOutOff[(size_t)v + 1] - c->hOutOff[v]);
  }
  if (c->maxInDeg <= GAS_TPV_MAX_DEGREE && c->maxOutDeg <= GAS_TPV_MAX_DEGREE) {  // fused rounds
    A(cudaMalloc(&c->fcell, (size_t)GAS_FUSED_CELL_BYTES(vertexBytes) * std::max(nV, 1)));
    // fixed-width adjacency rows: a vertex's neighbours in one or two 16-byte
    // loads addressed by its id, no offset lookup
    c->ellWidth = std::max(c->maxInDeg, c->maxOutDeg) <= 4 ? 4 : 8;
    const size_t cells = (size_t)std::max(nV, 1) * c->ellWidth;
    A(dalloc(&c->ellIn, cells));
    A(dalloc(&c->ellOut, cells));
    if (edgeBytes > 0) A(cudaMalloc(&c->ellEd, cells * edgeBytes));
    if (e == cudaSuccess && nV > 0) {
      const int blocks = (int)std::min<int64_t>(((int64_t)nV + 255) / 256, 65535LL * 32);
      ell_rows_kernel<<<blocks, 256, 0, c->stream>>>(nV, c->inOff, c->inSrc, c->ed, edgeBytes,
                                                     c->ellWidth, c->ellIn, c->ellEd);
      ell_rows_kernel<<<blocks, 256, 0, c->stream>>>(nV, c->outOff, c->outDst, nullptr, 0,
                                                     c->ellWidth, c->ellOut, nullptr);
      A(cudaGetLastError());
    }
    A(dalloc(&c->frontBits, 3 * (size_t)c->bitWords));
  }
  // in-degree bins of the dense pass
  std::vector<int32_t> bMid, bSmall, bTiny, chV, chB, chF, chC, chS;
  for (int32_t v = 0; v < nV; ++v) {
    const int32_t deg = c->hInOff[(size_t)v + 1] - c->hInOff[v];
    if (deg <= GAS_TPV_MAX_DEGREE) {
      bTiny.push_back(v);
    } else if (deg <= 64) {
      bSmall.push_back(v);
    } else if (deg <= gas::detail::kChunkEdges) {
      bMid.push_back(v);
    } else {
      const int32_t nch = (deg + gas::detail::kChunkEdges - 1) / gas::detail::kChunkEdges;
      const int32_t first = (int32_t)chV.size(), slot = (int32_t)(chS.empty() ? 0 : chS.back() + 1);
      for (int32_t k = 0; k < nch; ++k) {
        chV.push_back(v);
        chB.push_back(c->hInOff[v] + k * gas::detail::kChunkEdges);
        chF.push_back(first);
        chC.push_back(nch);
        chS.push_back(slot);
      }
    }
  }
  // heaviest first: the dense pass hands out work units in this order
  const auto byInDegDesc = [c](int32_t x, int32_t y) {
    return c->hInOff[(size_t)x + 1] - c->hInOff[x] > c->hInOff[(size_t)y + 1] - c->hInOff[y];
  };
  std::stable_sort(bMid.begin(), bMid.end(), byInDegDesc);
  std::stable_sort(bSmall.begin(), bSmall.end(), byInDegDesc);
  c->nMid = (int32_t)bMid.size();
  c->nSmall = (int32_t)bSmall.size();
  c->nTiny = (int32_t)bTiny.size();
  c->nChunks = (int32_t)chV.size();
  c->nChunkVertices = chS.empty() ? 0 : chS.back() + 1;
  A(dalloc(&c->binMid, bMid.size()));
  A(dalloc(&c->binSmall, bSmall.size()));
  A(dalloc(&c->binTiny, bTiny.size()));
  A(dalloc(&c->chunkVertex, chV.size()));
  A(dalloc(&c->chunkBegin, chB.size()));
  A(dalloc(&c->chunkFirst, chF.size()));
  A(dalloc(&c->chunkCount, chC.size()));
  A(dalloc(&c->chunkSlot, chS.size()));
  A(dalloc(&c->chunkArrive, (size_t)c->nChunkVertices));
  A(dalloc(&c->chunkFlags, chV.size()));
  A(cudaMalloc(&c->chunkVal, (size_t)((gatherBytes + 15) / 16 * 16) * std::max<size_t>(chV.size(), 1)));
  for (int k = 0; k < 2; ++k) {
    A(dalloc(&c->fvid[k], (size_t)nV));
    A(dalloc(&c->fpre[k], (size_t)nV));
    A(dalloc(&c->fbeg[k], (size_t)nV));
    A(dalloc(&c->sbeg[k], (size_t)nV));
    A(dalloc(&c->fsplit[k], (size_t)c->maxGatherTiles));
    A(dalloc(&c->svid[k], (size_t)nV));
    A(dalloc(&c->spre[k], (size_t)nV));
    A(dalloc(&c->ssplit[k], (size_t)c->maxScatTiles));
  }
  A(dalloc(&c->rsplit, (size_t)c->maxGatherTiles));
  A(dalloc(&c->mark, (size_t)nV));
  const size_t gb = (size_t)((gatherBytes + 15) / 16 * 16);
  A(cudaMalloc(&c->carryVal, gb * c->maxGatherTiles));
  A(dalloc(&c->carryFlag, (size_t)c->maxGatherTiles));
  A(dalloc(&c->ctl, 1));
  A(dalloc(&c->stats, (size_t)kMaxRounds * 2));
  if (e != cudaSuccess) {
    free_graph(c);
    return cuda_fail(e, "setGraph device allocation");
  }
  A(cudaMemsetAsync(c->mark, 0, sizeof(int32_t) * std::max(nV, 1), c->stream));
  A(cudaMemsetAsync(c->retBits, 0, sizeof(uint32_t) * 3 * std::max(c->bitWords, 1), c->stream));
  if (c->frontBits)
    A(cudaMemsetAsync(c->frontBits, 0, sizeof(uint32_t) * 3 * std::max(c->bitWords, 1), c->stream));
  auto up = [&](int32_t *dst, const std::vector<int32_t> &src) {
    if (!src.empty())
      A(cudaMemcpyAsync(dst, src.data(), sizeof(int32_t) * src.size(), cudaMemcpyHostToDevice,
                        c->stream));
  };
  up(c->binMid, bMid);
  up(c->binSmall, bSmall);
  up(c->binTiny, bTiny);
  up(c->chunkVertex, chV);
  up(c->chunkBegin, chB);
  up(c->chunkFirst, chF);
  up(c->chunkCount, chC);
  up(c->chunkSlot, chS);
  A(cudaMemsetAsync(c->chunkArrive, 0, sizeof(unsigned) * std::max(c->nChunkVertices, 1), c->stream));
  A(cudaMemsetAsync(c->carryFlag, 0, sizeof(unsigned) * c->maxGatherTiles, c->stream));
  A(cudaMemsetAsync(c->ctl, 0, sizeof(Ctl), c->stream));
  A(cudaMemsetAsync(c->vd, 0, (size_t)vertexBytes * std::max(nV, 1), c->stream));
  A(cudaStreamSynchronize(c->stream));  // host staging buffers die here
  if (e != cudaSuccess) {
    free_graph(c);
    return cuda_fail(e, "setGraph upload");
  }
  c->haveGraph = true;
  c->dirty = 0;
  c->densePending = false;
  c->epoch = 0;
  c->stamp = 0;
  c->iteration = 0;
  c->round = 0;
  c->rangeMode = true;
  c->rstart = 0;
  c->rcount = 0;
  c->cur = c->sidx = 0;
  c->pendingCommit = false;
  c->haveScatList = false;
  return GAS_OK;
}

gas_status gas_core_upload_vertex_data(gas_core *c, const void *host) {
  if (!c || !host) return fail(GAS_ERR_INVALID, "upload_vertex_data: null argument");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  if (c->nV == 0) return GAS_OK;
  cudaError_t e = cudaMemcpyAsync(c->vd, host, (size_t)c->vertexBytes * c->nV,
                                  cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "vertex data upload");
}

gas_status gas_core_download_vertex_data(gas_core *c, void *host) {
  if (!c || !host) return fail(GAS_ERR_INVALID, "download_vertex_data: null argument");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  gas_status st = check_device_error(c);
  if (st) return st;
  if (c->nV == 0) return GAS_OK;
  cudaError_t e = cudaMemcpyAsync(host, c->vd, (size_t)c->vertexBytes * c->nV,
                                  cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "vertex data download");
}

gas_status gas_core_download_edge_data(gas_core *c, void *host) {
  if (!c || !host) return fail(GAS_ERR_INVALID, "download_edge_data: null argument");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  if (c->edgeBytes == 0 || c->nE == 0) return GAS_OK;
  // back to edge-list order on the device, then one copy
  void *tmp = nullptr;
  const size_t bytes = (size_t)c->edgeBytes * c->nE;
  cudaError_t e = cudaMalloc(&tmp, bytes);
  if (e != cudaSuccess) return cuda_fail(e, "edge data download");
  gas_status st = device_scatter_bytes(c->stream, c->ed, c->cscPerm, c->nE, c->edgeBytes, tmp);
  if (st == GAS_OK) {
    e = cudaMemcpyAsync(host, tmp, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) st = cuda_fail(e, "edge data download");
  }
  cudaFree(tmp);
  return st;
}

gas_status gas_core_vertex_data(gas_core *c, void **dev) {
  if (!c || !dev) return fail(GAS_ERR_INVALID, "vertex_data: null argument");
  *dev = c->vd;
  return GAS_OK;
}

gas_status gas_core_set_active(gas_core *c, int32_t start, int32_t end) {
  if (!c) return fail(GAS_ERR_INVALID, "set_active: engine is NULL");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  if (start < 0 || end < start || end > c->nV)
    return fail(GAS_ERR_INVALID, "active range [%d, %d) outside [0, %d]", start, end, c->nV);
  gas_status st = set_device(c);
  if (st) return st;
  cudaError_t e = cudaMemsetAsync(c->ctl, 0, offsetof(Ctl, err), c->stream);  // keep err
  if (e != cudaSuccess) return cuda_fail(e, "set_active reset");
  c->dirty = 0;
  c->densePending = false;
  c->rangeMode = true;
  c->rstart = start;
  c->rcount = end - start;
  c->cur = c->sidx = 0;
  c->pendingCommit = false;
  c->haveScatList = false;
  c->countValid = false;
  c->round = 0;
  c->iteration = 0;  // a new traversal: rounds (and BFS depths) count from 0
  const int32_t T = c->hInOff[end] - c->hInOff[start];
  const long long items = (long long)c->rcount + T;
  const int nsplit = (int)((items + GAS_GATHER_TILE - 1) / GAS_GATHER_TILE) + 1;
  if (c->rcount > 0) {
    gas::detail::range_split_kernel<<<(nsplit + 127) / 128, 128, 0, c->stream>>>(
        c->inOff, start, c->rcount, T, c->rsplit, nsplit);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "range split launch");
  }
  return GAS_OK;
}

gas_status gas_core_count_active(gas_core *c, int32_t *n) {
  if (!c || !n) return fail(GAS_ERR_INVALID, "count_active: null argument");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  if (c->densePending) {
    gas_status st = set_device(c);
    if (!st) st = materialize(c);
    if (st) return st;
  }
  if (c->rangeMode) {
    *n = c->rcount;
    return GAS_OK;
  }
  if (c->countValid) {
    *n = c->countCache;
    return GAS_OK;
  }
  gas_status st = check_device_error(c);
  if (st) return st;
  unsigned long long v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, &c->ctl->f[c->cur].cnt, 8, cudaMemcpyDeviceToHost,
                                  c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "count_active");
  *n = (int32_t)std::min<unsigned long long>(v >> 32, (unsigned long long)c->nV);
  c->countCache = *n;
  c->countValid = true;
  return GAS_OK;
}

gas_status gas_core_set_iteration(gas_core *c, int32_t iteration) {
  if (!c) return fail(GAS_ERR_INVALID, "set_iteration: engine is NULL");
  c->iteration = iteration;
  return GAS_OK;
}

gas_status gas_core_gather_apply(gas_core *c, int32_t haveGather, gas_gather_launch_fn launch,
                                 void *user) {
  if (!c || !launch) return fail(GAS_ERR_INVALID, "gather_apply: null argument");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  gas_status st = set_device(c);
  if (st) return st;
  st = materialize(c);
  if (st) return st;
  st = clean(c, sbit(c->sidx) | kT0);
  if (st) return st;
  if (++c->epoch >= 0x7fffffffu) {  // flags hold epoch << 1
    cudaMemsetAsync(c->carryFlag, 0, sizeof(unsigned) * c->maxGatherTiles, c->stream);
    c->epoch = 1;
  }
  gas_gather_args a;
  memset(&a, 0, sizeof(a));
  a.nVertices = c->nV;
  a.nEdges = c->nE;
  a.inOffsets = c->inOff;
  a.inSources = c->inSrc;
  a.outOffsets = c->outOff;
  a.edgeData = c->ed;
  a.vertexData = c->vd;
  a.vertexNew = c->vnew;
  a.rangeMode = c->rangeMode ? 1 : 0;
  a.rangeStart = c->rstart;
  a.rangeCount = c->rcount;
  a.rangeBase = c->rangeMode ? c->hInOff[c->rstart] : 0;
  a.rangeMaxDeg = c->maxInDeg;
  a.rangeSplit = c->rsplit;
  a.front = front_list(c, c->cur);
  a.scat = scat_list(c, c->sidx);
  a.capacity = c->nV;
  a.maxScatTiles = c->maxScatTiles;
  a.resetCount = &c->ctl->f[c->cur ^ 1].cnt;
  a.resetMaxDeg = &c->ctl->f[c->cur ^ 1].maxd;
  a.resetTile = &c->ctl->tile[1];
  a.tileCounter = &c->ctl->tile[0];
  a.carryVal = c->carryVal;
  a.carryFlag = c->carryFlag;
  a.epoch = c->epoch;
  a.errWord = &c->ctl->err;
  a.statSlot = c->round < kMaxRounds ? c->stats + 2 * (size_t)c->round : nullptr;
  a.iteration = c->iteration;
  a.haveGather = haveGather ? 1 : 0;
  st = launch(user, &a, (void *)c->stream);
  if (st) return st;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "gather/apply launch");
  c->dirty |= sbit(c->sidx) | kT0;
  c->dirty &= ~(fbit(c->cur ^ 1) | kT1);
  c->pendingCommit = haveGather != 0;
  c->haveScatList = true;
  return GAS_OK;
}

gas_status gas_core_scatter_activate(gas_core *c) {
  if (!c) return fail(GAS_ERR_INVALID, "scatter_activate: engine is NULL");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  if (!c->haveScatList) return fail(GAS_ERR_STATE, "scatterActivate needs a gatherApply first");
  gas_status st = set_device(c);
  if (st) return st;
  st = clean(c, fbit(c->cur ^ 1) | kT1);
  if (st) return st;
  if (++c->stamp == 0x7fffffff) {
    cudaMemsetAsync(c->mark, 0, sizeof(int32_t) * std::max(c->nV, 1), c->stream);
    c->stamp = 1;
  }
  ScatterArgs a;
  memset(&a, 0, sizeof(a));
  a.outOffsets = c->outOff;
  a.outDests = c->outDst;
  a.inOffsets = c->inOff;
  a.scat = scat_list(c, c->sidx);
  a.commit = c->pendingCommit ? 1 : 0;
  a.vertexBytes = c->vertexBytes;
  a.vertexData = c->vd;
  a.vertexNew = c->vnew;
  a.rangeMode = c->rangeMode ? 1 : 0;
  a.rangeStart = c->rstart;
  a.rangeCount = c->rcount;
  a.frontVid = c->fvid[c->cur];
  a.frontCount = &c->ctl->f[c->cur].cnt;
  a.next = front_list(c, c->cur ^ 1);
  a.maxGatherTiles = c->maxGatherTiles;
  a.capacity = c->nV;
  a.mark = c->mark;
  a.stamp = c->stamp;
  a.tileCounter = &c->ctl->tile[1];
  a.resetTile = &c->ctl->tile[0];
  a.resetScatCount = &c->ctl->s[c->sidx ^ 1].cnt;
  a.resetScatMaxDeg = &c->ctl->s[c->sidx ^ 1].maxd;
  a.errWord = &c->ctl->err;
  a.statSlot = c->round < kMaxRounds ? c->stats + 2 * (size_t)c->round : nullptr;
  gas::detail::scatter_activate_kernel<<<c->scatterGrid, gas::detail::kSNT, 0, c->stream>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "scatter launch");
  c->dirty |= fbit(c->cur ^ 1) | kT1;
  c->dirty &= ~(kT0 | sbit(c->sidx ^ 1));
  c->pendingCommit = false;
  c->haveScatList = false;
  c->countValid = false;
  c->edgeScatterReady = true;
  ++c->round;
  return GAS_OK;
}

gas_status gas_core_next_iter(gas_core *c) {
  if (!c) return fail(GAS_ERR_INVALID, "next_iter: engine is NULL");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  if (c->densePending) {
    gas_status st = set_device(c);
    if (!st) st = materialize(c);
    if (st) return st;
  }
  c->cur ^= 1;
  c->sidx ^= 1;
  c->rangeMode = false;
  c->countValid = false;
  c->edgeScatterReady = false;
  return GAS_OK;
}

gas_status gas_core_run(gas_core *c, int32_t maxIters, int32_t haveGather,
                        gas_gather_launch_fn launch, void *user, int32_t *iterations) {
  if (!c || !launch) return fail(GAS_ERR_INVALID, "run: null argument");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  gas_status st = set_device(c);
  if (st) return st;
  if (iterations) *iterations = 0;
  int32_t n0 = 0;
  st = gas_core_count_active(c, &n0);
  if (st) return st;
  cudaEventRecord(c->t0, c->stream);
  const int32_t base = c->iteration;
  const int32_t round0 = c->round;
  int32_t done = -1, launched = 0;
  if (n0 == 0) done = 0;
  for (int32_t r = 0; done < 0 && (maxIters <= 0 || r < maxIters); ++r) {
    c->iteration = base + r;
    cudaEvent_t *pe = nullptr;
    if (c->profiling) {
      while (c->pev.size() < 4 * (size_t)(r + 1)) {
        cudaEvent_t ev;
        if (cudaEventCreate(&ev) != cudaSuccess) return cuda_fail(cudaGetLastError(), "event");
        c->pev.push_back(ev);
      }
      pe = &c->pev[4 * (size_t)r];
      cudaEventRecord(pe[0], c->stream);
    }
    if ((st = gas_core_gather_apply(c, haveGather, launch, user))) return st;
    if (pe) {
      cudaEventRecord(pe[1], c->stream);
      cudaEventRecord(pe[2], c->stream);
    }
    if ((st = gas_core_scatter_activate(c))) return st;
    if (pe) cudaEventRecord(pe[3], c->stream);
    if ((st = gas_core_next_iter(c))) return st;
    cudaError_t e = cudaMemcpyAsync(&c->pinned[r % kRing], &c->ctl->f[c->cur].cnt, 8,
                                    cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev[r % kRing], c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "run bookkeeping");
    launched = r + 1;
    if (r >= kLag) {
      const int k = r - kLag;
      cudaEventSynchronize(c->ev[k % kRing]);
      if ((c->pinned[k % kRing] >> 32) == 0) done = k + 1;
    }
  }
  cudaEventRecord(c->t1, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "run");
  if (done < 0) {
    done = launched;
    for (int k = std::max(0, launched - kLag - 1); k < launched; ++k)
      if ((c->pinned[k % kRing] >> 32) == 0) {
        done = k + 1;
        break;
      }
  }
  c->iteration = base + done;
  c->round = round0 + done;  // trailing launches saw an empty frontier
  cudaEventElapsedTime(&c->lastMs, c->t0, c->t1);
  c->gatherMs = c->scatterMs = 0.f;
  c->gatherLaunches = c->scatterLaunches = 0;
  if (c->profiling) {
    for (int32_t r = 0; r < launched; ++r) {
      float g = 0.f, sc = 0.f;
      cudaEventElapsedTime(&g, c->pev[4 * (size_t)r], c->pev[4 * (size_t)r + 1]);
      cudaEventElapsedTime(&sc, c->pev[4 * (size_t)r + 2], c->pev[4 * (size_t)r + 3]);
      c->gatherMs += g;
      c->scatterMs += sc;
    }
    c->gatherLaunches = c->scatterLaunches = launched;
  }
  if (iterations) *iterations = done;
  return check_device_error(c);
}

gas_status gas_core_run_persistent(gas_core *c, int32_t maxIters, int32_t haveGather,
                                   gas_run_launch_fn runLaunch, gas_gather_launch_fn launch,
                                   void *user, int32_t *iterations) {
  if (!c) return fail(GAS_ERR_INVALID, "run: engine is NULL");
  if (!runLaunch || c->profiling) return gas_core_run(c, maxIters, haveGather, launch, user, iterations);
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  gas_status st = set_device(c);
  if (st) return st;
  if (iterations) *iterations = 0;
  int32_t n0 = 0;
  st = gas_core_count_active(c, &n0);
  if (st) return st;
  if (n0 == 0) return GAS_OK;
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  if (c->epoch > 0x40000000u) {  // flags hold epoch << 1
    A(cudaMemsetAsync(c->carryFlag, 0, sizeof(unsigned) * c->maxGatherTiles, c->stream));
    c->epoch = 0;
  }
  if (c->stamp > 0x40000000) {
    A(cudaMemsetAsync(c->mark, 0, sizeof(int32_t) * std::max(c->nV, 1), c->stream));
    A(cudaMemsetAsync(c->retBits, 0, sizeof(uint32_t) * 3 * std::max(c->bitWords, 1), c->stream));
  if (c->frontBits)
    A(cudaMemsetAsync(c->frontBits, 0, sizeof(uint32_t) * 3 * std::max(c->bitWords, 1), c->stream));
    c->stamp = 0;
  }
  if (e != cudaSuccess) return cuda_fail(e, "run setup");

  gas_run_args ra;
  memset(&ra, 0, sizeof(ra));
  gas_gather_args &a = ra.g;
  a.nVertices = c->nV;
  a.nEdges = c->nE;
  a.inOffsets = c->inOff;
  a.inSources = c->inSrc;
  a.outOffsets = c->outOff;
  a.edgeData = c->ed;
  a.vertexData = c->vd;
  a.vertexNew = c->vnew;
  a.rangeMode = c->rangeMode ? 1 : 0;
  a.rangeStart = c->rstart;
  a.rangeCount = c->rcount;
  a.rangeBase = c->rangeMode ? c->hInOff[c->rstart] : 0;
  a.rangeMaxDeg = c->maxInDeg;
  a.rangeSplit = c->rsplit;
  a.capacity = c->nV;
  a.maxScatTiles = c->maxScatTiles;
  a.carryVal = c->carryVal;
  a.carryFlag = c->carryFlag;
  a.errWord = &c->ctl->err;
  a.iteration = c->iteration;
  a.haveGather = haveGather ? 1 : 0;
  ra.outDests = c->outDst;
  ra.vertexBytes = c->vertexBytes;
  ra.maxGatherTiles = c->maxGatherTiles;
  for (int k = 0; k < 2; ++k) {
    ra.frontL[k] = front_list(c, k);
    ra.scatL[k] = scat_list(c, k);
  }
  ra.mark = c->mark;
  ra.stats = c->stats + 2 * (size_t)std::min(c->round, kMaxRounds);
  ra.maxStatRounds = std::max(0, kMaxRounds - c->round);
  ra.cur = c->cur;
  ra.sidx = c->sidx;
  ra.maxRounds = maxIters > 0 ? maxIters : 0;
  ra.epochBase = c->epoch + 1;
  ra.stampBase = c->stamp + 1;
  ra.barrier = &c->ctl->bar[0];
  ra.roundsOut = &c->ctl->rounds;
  ra.vertexAlt = c->valt;
  for (int k = 0; k < 3; ++k) {
    ra.retBits[k] = c->retBits + (size_t)k * c->bitWords;
    ra.frontBits[k] = c->frontBits ? c->frontBits + (size_t)k * c->bitWords : nullptr;
  }
  ra.bitWords = c->bitWords;
  {
    // per-run counters, the barrier and rounds words, the bitmap round 0
    // writes (stamp stampBase; each round clears the one after it) and the
    // active-set bitmap a fused round 0 writes (stampBase + 1)
    ZeroSegments z;
    memset(&z, 0, sizeof(z));
    auto seg = [&](void *p, size_t bytes) {
      z.ptr[z.n] = static_cast<uint32_t *>(p);
      z.words[z.n++] = (int32_t)(bytes / sizeof(uint32_t));
    };
    seg(&c->ctl->dense[0][0], sizeof(c->ctl->dense));
    seg(c->chunkArrive, sizeof(unsigned) * std::max(c->nChunkVertices, 1));
    seg(&c->ctl->s[0], sizeof(c->ctl->s));
    seg(&c->ctl->f[c->cur ^ 1], sizeof(ListCtl));
    seg(&c->ctl->bar[0], sizeof(c->ctl->bar) + sizeof(int32_t));
    seg(round_bits(c, ra.stampBase), sizeof(uint32_t) * std::max(c->bitWords, 1));
    if (c->frontBits)
      seg(c->frontBits + (size_t)((unsigned)(ra.stampBase + 1) % 3u) * c->bitWords,
          sizeof(uint32_t) * std::max(c->bitWords, 1));
    const int32_t most = std::max(c->bitWords, std::max(c->nChunkVertices, 64));
    const int blocks = std::min(c->numSMs > 0 ? c->numSMs : 1, (most + 255) / 256);
    zero_segments_kernel<<<blocks, 256, 0, c->stream>>>(z);
    A(cudaGetLastError());
    if (e != cudaSuccess) return cuda_fail(e, "run setup");
  }
  ra.binMid = c->binMid;
  ra.binSmall = c->binSmall;
  ra.binTiny = c->binTiny;
  ra.nMid = c->nMid;
  ra.nSmall = c->nSmall;
  ra.nTiny = c->nTiny;
  ra.chunkVertex = c->chunkVertex;
  ra.chunkBegin = c->chunkBegin;
  ra.chunkFirst = c->chunkFirst;
  ra.chunkCount = c->chunkCount;
  ra.chunkSlot = c->chunkSlot;
  ra.nChunks = c->nChunks;
  ra.nChunkVertices = c->nChunkVertices;
  ra.chunkArrive = c->chunkArrive;
  ra.chunkVal = c->chunkVal;
  ra.chunkFlags = c->chunkFlags;
  ra.denseCnt = &c->ctl->dense[0][0];
  ra.fusedCells = c->fcell;
  ra.ellIn = c->ellIn;
  ra.ellOut = c->ellOut;
  ra.ellEd = c->ellEd;
  ra.ellWidth = c->ellWidth;
  ra.fused = (c->fcell && c->fusedRounds && !c->csr2csc && c->maxInDeg <= GAS_TPV_MAX_DEGREE &&
              c->maxOutDeg <= GAS_TPV_MAX_DEGREE)
                 ? 1
                 : 0;
  ra.edgeScatter = c->csr2csc ? 1 : 0;
  ra.csr2csc = c->csr2csc;
  ra.denseAlpha = ra.edgeScatter ? 0 : c->denseAlpha;  // Program::scatter walks list rounds
  ra.allActive =
      (c->rangeMode && c->rstart == 0 && c->rcount == c->nV && ra.denseAlpha > 0) ? 1 : 0;
  ra.vcurOut = &c->ctl->vcur;
  ra.resume = &c->ctl->resume[0];
  ra.denseEndOut = &c->ctl->denseEnd;

  cudaEventRecord(c->t0, c->stream);
  st = runLaunch(user, &ra, (void *)c->stream);
  if (st == GAS_ERR_UNSUPPORTED && ra.edgeScatter)  // the caller steps the rounds itself
    return fail(GAS_ERR_UNSUPPORTED, "persistent run unavailable");
  if (st == GAS_ERR_UNSUPPORTED) return gas_core_run(c, maxIters, haveGather, launch, user, iterations);
  if (st) return st;
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "persistent run launch");
  cudaEventRecord(c->t1, c->stream);
  int32_t rv[4] = {0, 0, 0, 0};  // rounds, vcur, denseEnd, pad (adjacent in Ctl)
  A(cudaMemcpyAsync(rv, &c->ctl->rounds, sizeof(rv), cudaMemcpyDeviceToHost, c->stream));
  A(cudaStreamSynchronize(c->stream));
  if (e != cudaSuccess) return cuda_fail(e, "persistent run");
  const int32_t rounds = rv[0];
  if (rv[1]) {  // the result ended in the alternate buffer of the dense rounds
    A(cudaMemcpyAsync(c->vd, c->valt, (size_t)c->vertexBytes * c->nV, cudaMemcpyDeviceToDevice,
                      c->stream));
    A(cudaStreamSynchronize(c->stream));
    if (e != cudaSuccess) return cuda_fail(e, "persistent run copy-back");
  }
  cudaEventElapsedTime(&c->lastMs, c->t0, c->t1);
  const int32_t R = rounds;
  if (R & 1) {
    c->cur ^= 1;
    c->sidx ^= 1;
  }
  if (R > 0) c->rangeMode = false;
  c->epoch += (unsigned)R;
  c->stamp += R;
  c->iteration += R;
  c->round += R;
  c->dirty |= kF0 | kF1 | kS0 | kS1;
  c->pendingCommit = false;
  c->haveScatList = false;
  c->countValid = false;
  if (rv[2] && R > 0) {  // the next frontier is the last round's stamps
    c->densePending = true;
    c->densePendStamp = c->stamp;  // the last round's stamp
  }
  if (iterations) *iterations = R;
  return check_device_error(c);
}

gas_status gas_core_round_stats(gas_core *c, int32_t capacity, int64_t *active,
                                int64_t *gathered, int64_t *ret, int64_t *scattered,
                                int32_t *rounds) {
  if (!c) return fail(GAS_ERR_INVALID, "round_stats: engine is NULL");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  const int nr = std::min(c->round, kMaxRounds);
  if (rounds) *rounds = nr;
  const int m = std::min(nr, std::max(capacity, 0));
  if (m == 0) return GAS_OK;
  std::vector<unsigned long long> h((size_t)m * 2);
  cudaError_t e = cudaMemcpyAsync(h.data(), c->stats, h.size() * 8, cudaMemcpyDeviceToHost,
                                  c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "round_stats");
  for (int k = 0; k < m; ++k) {
    if (active) active[k] = (int64_t)(h[2 * k] >> 32);
    if (gathered) gathered[k] = (int64_t)(h[2 * k] & 0xffffffffull);
    if (ret) ret[k] = (int64_t)(h[2 * k + 1] >> 32);
    if (scattered) scattered[k] = (int64_t)(h[2 * k + 1] & 0xffffffffull);
  }
  return GAS_OK;
}

gas_status gas_core_last_run_ms(gas_core *c, float *ms) {
  if (!c || !ms) return fail(GAS_ERR_INVALID, "last_run_ms: null argument");
  *ms = c->lastMs;
  return GAS_OK;
}

gas_status gas_core_save_vertex_data(gas_core *c) {
  if (!c) return fail(GAS_ERR_INVALID, "save_vertex_data: engine is NULL");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  gas_status st = set_device(c);
  if (st) return st;
  const size_t bytes = (size_t)c->vertexBytes * std::max(c->nV, 1);
  if (!c->vsaved) {
    cudaError_t e = cudaMalloc(&c->vsaved, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "save_vertex_data allocation");
  }
  cudaError_t e = cudaMemcpyAsync(c->vsaved, c->vd, bytes, cudaMemcpyDeviceToDevice, c->stream);
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "save_vertex_data");
}

gas_status gas_core_restore_vertex_data(gas_core *c) {
  if (!c) return fail(GAS_ERR_INVALID, "restore_vertex_data: engine is NULL");
  if (!c->haveGraph || !c->vsaved) return fail(GAS_ERR_STATE, "no saved vertex data");
  gas_status st = set_device(c);
  if (st) return st;
  const size_t bytes = (size_t)c->vertexBytes * std::max(c->nV, 1);
  cudaError_t e = cudaMemcpyAsync(c->vd, c->vsaved, bytes, cudaMemcpyDeviceToDevice, c->stream);
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "restore_vertex_data");
}

gas_status gas_core_set_fused_rounds(gas_core *c, int32_t on) {
  if (!c) return fail(GAS_ERR_INVALID, "set_fused_rounds: engine is NULL");
  c->fusedRounds = on != 0;
  return GAS_OK;
}

gas_status gas_core_set_dense_policy(gas_core *c, int32_t alpha) {
  if (!c) return fail(GAS_ERR_INVALID, "set_dense_policy: engine is NULL");
  if (alpha < 0) return fail(GAS_ERR_INVALID, "dense policy alpha must be >= 0");
  c->denseAlpha = alpha;
  return GAS_OK;
}

gas_status gas_core_set_profiling(gas_core *c, int32_t enabled) {
  if (!c) return fail(GAS_ERR_INVALID, "set_profiling: engine is NULL");
  c->profiling = enabled != 0;
  return GAS_OK;
}

gas_status gas_core_kernel_times(gas_core *c, float *gatherMs, float *scatterMs,
                                 int32_t *gatherLaunches, int32_t *scatterLaunches) {
  if (!c) return fail(GAS_ERR_INVALID, "kernel_times: engine is NULL");
  if (gatherMs) *gatherMs = c->gatherMs;
  if (scatterMs) *scatterMs = c->scatterMs;
  if (gatherLaunches) *gatherLaunches = c->gatherLaunches;
  if (scatterLaunches) *scatterLaunches = c->scatterLaunches;
  return GAS_OK;
}

gas_status gas_core_enable_edge_scatter(gas_core *c, int32_t on) {
  if (!c) return fail(GAS_ERR_INVALID, "enable_edge_scatter: engine is NULL");
  c->edgeScatterOn = on != 0;
  return GAS_OK;
}

gas_status gas_core_edge_scatter(gas_core *c, gas_edge_scatter_fn launch, void *user) {
  if (!c || !launch) return fail(GAS_ERR_INVALID, "edge_scatter: null argument");
  if (!c->haveGraph) return fail(GAS_ERR_STATE, "no graph set");
  if (!c->csr2csc)
    return fail(GAS_ERR_STATE, "edge scatter needs gas_core_enable_edge_scatter before setGraph "
                               "and non-empty EdgeData");
  if (!c->edgeScatterReady) return fail(GAS_ERR_STATE, "edge scatter needs a scatterActivate first");
  gas_status st = set_device(c);
  if (st) return st;
  gas_edge_scatter_args a;
  a.vid = c->svid[c->sidx];
  a.count = &c->ctl->s[c->sidx].cnt;
  a.outOffsets = c->outOff;
  a.outDests = c->outDst;
  a.csr2csc = c->csr2csc;
  a.vertexData = c->vd;
  a.edgeData = c->ed;
  st = launch(user, &a, (void *)c->stream);
  if (st) return st;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "edge scatter launch");
}

gas_status gas_core_sync(gas_core *c) {
  if (!c) return fail(GAS_ERR_INVALID, "sync: engine is NULL");
  if (!c->haveGraph) return GAS_OK;
  return check_device_error(c);
}

const char *gas_status_string(gas_status s) {
  switch (s) {
    case GAS_OK: return "ok";
    case GAS_ERR_INVALID: return "invalid argument";
    case GAS_ERR_OOM: return "out of memory";
    case GAS_ERR_CUDA: return "CUDA error";
    case GAS_ERR_TIMEOUT: return "device wait timed out";
    case GAS_ERR_STATE: return "invalid state";
    case GAS_ERR_UNSUPPORTED: return "unsupported";
    case GAS_ERR_NO_DEVICE: return "no supported device";
    default: return "unknown status";
  }
}

const char *gas_last_error(void) { return g_last_error.c_str(); }

int32_t gas_device_supported(int32_t device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return 0;
  }
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
  return (major == 10 && minor == 3) ? 1 : 0;
}

}  // extern "C"
