// gas_bfs_noalloc: breadth-first search that allocates no memory.
//
// Some callers cannot call cudaMalloc: a host whose device memory is
// entirely reserved by another allocator (a framework's caching pool that
// has already claimed the free HBM), or a latency-critical serving thread
// that must not pay cudaMalloc's implicit device synchronisation.  This
// entry point serves them: the caller passes the graph and the output in
// device memory it already owns, and every scratch buffer the search needs
// (frontier and scatter lists, merge-path splits, activation stamps,
// control words) lives in one file-scope __device__ array of fixed size.
// A GPU holds that array from the moment this library's device code is
// loaded on it until the process exits.  With CUDA's lazy module loading
// (the default) that moment is the first call on the device, so a caller
// whose allocator has already claimed the free device memory can see that
// first call fail with an out-of-memory status; later calls cannot.
//
// The search is the BFS vertex program (bfs.cu:31-78) run to completion by
// the same persistent kernel as gas_engine_run.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "gas_gb300.h"
#include "gas_gb300/gpugas.cuh"
#include "gas_gb300/programs.cuh"
#include "gas_internal.h"

using gas::internal::cuda_fail;
using gas::internal::fail;

namespace {

constexpr int32_t kMaxVertices = GAS_NOALLOC_MAX_VERTICES;
constexpr int32_t kMaxEdges = GAS_NOALLOC_MAX_EDGES;
constexpr int32_t kMaxTiles = (kMaxVertices + kMaxEdges) / GAS_GATHER_TILE + 2;
constexpr int kLists = 4;  // frontier 0/1, scatter 0/1

struct ListCtl {
  unsigned long long cnt;
  unsigned maxd;
  unsigned pad;
};

struct Tail {
  ListCtl ctl[kLists];
  unsigned bar[2];
  int32_t rounds;
  unsigned err;
  unsigned carryFlag[4];
  int32_t carryVal[4];
};

// byte offsets inside the scratch array
constexpr size_t kListBytes = sizeof(int32_t) * (size_t)kMaxVertices;
constexpr size_t kSplitBytes = sizeof(int32_t) * (size_t)kMaxTiles;
constexpr size_t kOffLists = 0;                                  // [4][3][kMaxVertices]
constexpr size_t kOffSplits = kOffLists + kLists * 3 * kListBytes;  // [4][kMaxTiles]
constexpr size_t kOffMark = kOffSplits + kLists * kSplitBytes;      // [kMaxVertices]
constexpr size_t kOffTail = (kOffMark + kListBytes + 255) / 256 * 256;
constexpr size_t kScratchBytes = kOffTail + sizeof(Tail);

// The scratch.  In host code this name only stands in for the symbol; the
// device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_scratch[kMaxDevices] = {};
int g_grid[kMaxDevices] = {};

__global__ void fill_minus_one(int32_t *p, int32_t n) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = -1;
}

// Once per device, with that device current: the scratch's device address
// and the co-resident grid of the persistent kernel.  Both are kept for the
// life of the process; a cudaDeviceReset (which unloads the module and may
// move the array) is not supported between calls.
gas_status setup(int dev, unsigned char **scratch, int *grid) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
    int sms = 0, per = 0, coop = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per, gas::detail::run_persistent_kernel<gas::programs::BFS>, gas::detail::kGNT, 0);
    if (e != cudaSuccess) return cuda_fail(e, "occupancy query");
    if (!coop || per <= 0 || sms <= 0)
      return fail(GAS_ERR_UNSUPPORTED, "device %d cannot run the cooperative search kernel", dev);
    g_grid[dev] = per * sms;
    g_scratch[dev] = static_cast<unsigned char *>(p);
  }
  *scratch = g_scratch[dev];
  *grid = g_grid[dev];
  return GAS_OK;
}

}  // namespace

extern "C" {

gas_status gas_bfs_noalloc(int32_t nVertices, int32_t nEdges, const int32_t *outOffsets,
                           const int32_t *outDests, int32_t source, int32_t *depth,
                           void *stream, int32_t *rounds) {
  if (nVertices <= 0 || nEdges < 0 || !outOffsets || (nEdges > 0 && !outDests) || !depth)
    return fail(GAS_ERR_INVALID, "gas_bfs_noalloc: bad graph or output argument");
  if (nVertices > kMaxVertices || nEdges > kMaxEdges)
    return fail(GAS_ERR_INVALID,
                "gas_bfs_noalloc: %d vertices / %d edges exceed the fixed scratch limit of "
                "%d vertices / %d edges",
                nVertices, nEdges, kMaxVertices, kMaxEdges);
  if (source < 0 || source >= nVertices)
    return fail(GAS_ERR_INVALID, "gas_bfs_noalloc: source %d outside [0, %d)", source, nVertices);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(GAS_ERR_UNSUPPORTED, "device id %d", dev);
  unsigned char *sc = nullptr;
  int grid = 0;
  gas_status st = setup(dev, &sc, &grid);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  Tail *tail = reinterpret_cast<Tail *>(sc + kOffTail);

  // state that must start at zero: control words and activation stamps
  e = cudaMemsetAsync(tail, 0, sizeof(Tail), s);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(sc + kOffMark, 0, sizeof(int32_t) * (size_t)nVertices, s);
  if (e != cudaSuccess) return cuda_fail(e, "no-alloc scratch reset");
  fill_minus_one<<<(nVertices + 255) / 256, 256, 0, s>>>(depth, nVertices);  // bfs.cu:143-145
  // The first round's frontier is the range [source, source + 1): its edge
  // positions are counted from outOffsets[source], as gas_engine_run counts
  // them from the CSC offset of the range start.
  int32_t base = 0;
  e = cudaMemcpyAsync(&base, outOffsets + source, sizeof(base), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "no-alloc BFS range offset");

  gas_run_args ra;
  memset(&ra, 0, sizeof(ra));
  gas_gather_args &a = ra.g;
  a.nVertices = nVertices;
  a.nEdges = nEdges;
  a.inOffsets = outOffsets;  // only feeds degree bookkeeping: BFS has no gather
  a.inSources = outDests;
  a.outOffsets = outOffsets;
  a.vertexData = depth;
  a.vertexNew = depth;
  a.rangeMode = 1;
  a.rangeStart = source;
  a.rangeCount = 1;
  a.rangeBase = base;
  a.capacity = nVertices;
  a.maxScatTiles = kMaxTiles;
  a.carryVal = tail->carryVal;
  a.carryFlag = tail->carryFlag;
  a.errWord = &tail->err;
  a.haveGather = 0;
  ra.outDests = outDests;
  ra.vertexBytes = (int32_t)sizeof(int32_t);
  ra.maxGatherTiles = kMaxTiles;
  for (int k = 0; k < kLists; ++k) {
    gas_vertex_list l;
    l.vid = reinterpret_cast<int32_t *>(sc + kOffLists + (3 * k + 0) * kListBytes);
    l.pre = reinterpret_cast<int32_t *>(sc + kOffLists + (3 * k + 1) * kListBytes);
    l.beg = reinterpret_cast<int32_t *>(sc + kOffLists + (3 * k + 2) * kListBytes);
    l.split = reinterpret_cast<int32_t *>(sc + kOffSplits + k * kSplitBytes);
    l.count = &tail->ctl[k].cnt;
    l.maxDeg = &tail->ctl[k].maxd;
    if (k < 2)
      ra.frontL[k] = l;
    else
      ra.scatL[k - 2] = l;
  }
  ra.mark = reinterpret_cast<int32_t *>(sc + kOffMark);
  ra.stats = nullptr;
  ra.maxStatRounds = 0;
  ra.cur = 0;
  ra.sidx = 0;
  ra.maxRounds = 0;
  ra.epochBase = 1;
  ra.stampBase = 1;
  ra.barrier = tail->bar;
  ra.roundsOut = &tail->rounds;

  void *args[] = {&ra};
  e = cudaLaunchCooperativeKernel(
      (const void *)gas::detail::run_persistent_kernel<gas::programs::BFS>, dim3(grid),
      dim3(gas::detail::kGNT), args, 0, s);
  if (e != cudaSuccess) return cuda_fail(e, "no-alloc BFS launch");
  int32_t r = 0;
  unsigned err = 0;
  e = cudaMemcpyAsync(&r, &tail->rounds, sizeof(r), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, &tail->err, sizeof(err), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "no-alloc BFS");
  if (err & GAS_DEVERR_TIMEOUT) return fail(GAS_ERR_TIMEOUT, "a bounded device wait timed out");
  if (err) return fail(GAS_ERR_STATE, "device list capacity exceeded (error bits 0x%x)", err);
  if (rounds) *rounds = r;
  return GAS_OK;
}

}  // extern "C"
