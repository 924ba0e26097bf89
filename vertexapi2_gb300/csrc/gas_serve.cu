// Serving loop (gas_server_* in gas_gb300.h): resident graphs, admission
// by free device memory, continuous batching over several lanes.
//
// Threads: callers submit and wait; one scheduler thread owns every CUDA
// call that touches batch state.  Each lane is a non-blocking stream that
// runs one batch at a time; a batch advances by round kernels
// (gas_gb300/detail/serve.cuh) queued a chunk at a time, two chunks ahead
// of the host's end test, so the lane never idles on the host.  Batches on
// different lanes run concurrently on the device.  Working state comes from
// a server-owned stream-ordered memory pool and returns to it when the
// batch ends; results stay until their query is fetched.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "gas_gb300.h"
#include "gas_gb300/detail/serve.cuh"
#include "gas_internal.h"

using gas::internal::BatchGraph;
using gas::internal::cuda_fail;
using gas::internal::fail;

namespace {

constexpr int kMaxLanes = 16;
constexpr int kMaxQ = 256;
constexpr int kPprRounds = 20;    // PPR iterations (a fixed count, as run(20))
constexpr int kFirstChunk = 4;    // rounds queued per chunk: 4, 8, ... 64
constexpr int kMaxChunk = 64;
constexpr int kKinds = 3;         // BFS, SSSP, PPR
constexpr int kMaxPersistent = 2; // batches in a cooperative launch at once, a third of the device each
constexpr int64_t kTieNs = 20000000;  // queries this close in arrival count as a burst
constexpr int64_t kWindowDiv = 32;         // batching window: recent run time / kWindowDiv
constexpr int64_t kWindowMaxNs = 10000000;

// Makes `device` current for the scope and restores the caller's device.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int device) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaSetDevice(device);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

int kind_of(int32_t program) {
  switch (program) {
    case GAS_PROGRAM_BFS: return 0;
    case GAS_PROGRAM_SSSP: return 1;
    case GAS_PROGRAM_PPR: return 2;
    default: return -1;
  }
}

struct ServeGraph {
  int32_t id = 0;
  gas_batch *batch = nullptr;  // CSC/CSR, weights, pull units
  BatchGraph bg;
  // PPR: out-degrees, the last round each vertex is active, work units
  // (longest first) and the partial-sum slots of hub chunks
  gas::internal::PprGraph ppr;
  bool weighted = false;
  int32_t maxOutDeg = 0;         // pair frontier when small (lattice-like graphs)
  int32_t maxWeight = 0;
  int64_t bytes = 0;
};

struct Batch;

struct Query {
  uint64_t ticket = 0;
  int32_t graph = 0, program = 0, source = 0;
  int kind = 0;
  gas_query_info info;
  bool done = false;
  std::shared_ptr<Batch> batch;  // holds the results until fetched
  int slot = 0;
};

// device control words of a batch: cnt[3] | bar[2] | rounds | err |
// listCnt[3] | done
struct Ctl {
  unsigned long long cnt[3];
  unsigned bar[2];
  int32_t rounds;
  unsigned err;
  unsigned long long listCnt[3];
  unsigned done;
  unsigned pad[3];
};

struct Batch {
  int lane = 0;
  ServeGraph *g = nullptr;
  int kind = 0;
  int32_t nQ = 0, Q = 0, W = 0;
  std::vector<Query *> queries;
  unsigned char *state = nullptr;  // working state, released when the batch ends
  int64_t stateBytes = 0;
  int32_t *out = nullptr;          // [nQ][V] results, released when all are fetched
  int64_t outBytes = 0;
  int32_t *sources = nullptr;      // inside `state`
  Ctl *ctl = nullptr;              // inside `state`
  gas::detail::BatchArgs ba;
  gas::detail::PprArgs pa;
  bool pairs = false;             // (vertex, query) pair frontier
  bool persistent = false;        // every round in one cooperative launch
  int64_t pairsSeen = 0;          // largest pair list seen at a chunk's end
  int32_t delta = 0;              // SSSP distance buckets
  int roundsIssued = 0;
  int chunk = kFirstChunk;
  int unfetched = 0;
  int64_t admitNs = 0;
  size_t cell = 0;                 // graph * kKinds + kind
  cudaStream_t stream = nullptr;
  class Server *server = nullptr;
  ~Batch();
};

struct ChunkMark {  // a queued end test: event + pinned copy of the control words
  cudaEvent_t ev = nullptr;
  Ctl *mirror = nullptr;
  bool final = false;  // the results' transpose follows (the batch is over)
  bool busy = false;
};

struct Lane {
  cudaStream_t stream = nullptr;
  // Batches on graphs of many rounds (the pair-frontier graphs: low degree,
  // high diameter) run on a high-priority stream: each of their rounds is a
  // small kernel, and under load they would otherwise queue behind the
  // large round kernels of other lanes, round after round.
  cudaStream_t streamHi = nullptr;
  std::shared_ptr<Batch> batch;
  ChunkMark marks[3];
  std::deque<int> queued;  // indices of marks in flight, in issue order
};

class Server {
 public:
  int device = 0;
  gas_server_config cfg;
  int sms = 1;
  cudaMemPool_t pool = nullptr;
  cudaStream_t fetch = nullptr;
  std::mutex fetchMu;
  Lane lanes[kMaxLanes];
  Ctl *mirrors = nullptr;  // pinned, 3 per lane
  int32_t *srcPinned = nullptr;  // pinned, kMaxQ per lane (sources of its batch)

  std::mutex mu;  // queries, pending, graphs, stats
  std::condition_variable cvWork, cvDone;
  std::map<uint64_t, Query *> queries;
  std::vector<std::deque<Query *>> pending;  // per graph * kinds
  std::vector<int64_t> cellRunNs;            // recent batch run time per graph * kinds
  std::vector<ServeGraph *> graphs;
  uint64_t nextTicket = 1;
  gas_server_stats stats;
  std::atomic<int64_t> bytesInUse{0};
  std::atomic<int64_t> launches{0};  // kernels launched (scheduler thread)
  int persistentRunning = 0;         // batches in a cooperative launch (scheduler thread)
  std::thread sched;
  bool stop = false;

  std::mutex freeMu;  // results to release (from waiting threads)
  std::vector<int32_t *> toFree;

  ~Server();
  gas_status start();
  void loop();
  bool poll_lane(int l);
  bool admit();
  gas_status launch(int l, const std::shared_ptr<Batch> &b);
  void issue_chunk(int l, int rounds, bool final);
  void finish_batch(int l, gas_status st, int32_t rounds);
  int64_t state_bytes(const ServeGraph &g, int kind, int Q) const;
  int64_t available_bytes();
};

Batch::~Batch() {}

// Queries per vertex row of a batch of n: BFS/SSSP at least 32 (a word of
// query bits), PPR the next power of two.
int row_width(int kind, int n) {
  int Q = kind == 2 ? 1 : 32;
  while (Q < n) Q *= 2;
  return Q;
}

// (vertex, query) pair frontier for graphs of small out-degree whose V * Q
// pair ids fit 32 bits (as gas_batch chooses it)
bool use_pairs(const ServeGraph &g, int kind, int Q) {
  return kind != 2 && g.maxOutDeg <= 64 && (long long)std::max(g.bg.g.nV, 1) * Q < (1ll << 31);
}

int64_t Server::state_bytes(const ServeGraph &g, int kind, int Q) const {
  const int64_t V = std::max(g.bg.g.nV, 1), W = std::max(Q / 32, 1);
  // control words, sources, bucket bounds and flags, and up to 24 arrays
  // each rounded up to 256 bytes
  const int64_t base = 256 + 4 * kMaxQ + 4 * (2 * kMaxQ + 24) + 24 * 256;
  const int64_t lists = 24 * gas::detail::batch_list_capacity(V, g.bg.g.nE) + 4 * V +
                        (use_pairs(g, kind, Q) ? 12 * V * Q : 0);
  if (kind == 0) return base + V * Q * 4 + 16 * V * W + lists;
  if (kind == 1) return base + V * Q * 4 + 12 * V * W + lists;
  return base + V * Q * 16 + (int64_t)g.ppr.slots * Q * 4 + (int64_t)g.ppr.hubs * 4;
}

int64_t Server::available_bytes() {
  size_t freeB = 0, totalB = 0;
  if (cudaMemGetInfo(&freeB, &totalB) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  uint64_t reserved = 0, used = 0;
  cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
  cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
  return (int64_t)freeB + (int64_t)(reserved - std::min(used, reserved)) - cfg.reserveBytes;
}

gas_status Server::start() {
  DeviceGuard dg(device);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaMemPoolProps props;
  memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  cudaError_t e = cudaMemPoolCreate(&pool, &props);
  if (e == cudaSuccess) {
    uint64_t keep = ~0ull;  // keep released blocks for the next batch
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&fetch, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost(&mirrors, sizeof(Ctl) * 3 * cfg.lanes);
  if (e == cudaSuccess) e = cudaMallocHost(&srcPinned, sizeof(int32_t) * kMaxQ * cfg.lanes);
  int leastPri = 0, greatestPri = 0;
  if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&leastPri, &greatestPri);
  for (int l = 0; l < cfg.lanes && e == cudaSuccess; ++l) {
    e = cudaStreamCreateWithFlags(&lanes[l].stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
      e = cudaStreamCreateWithPriority(&lanes[l].streamHi, cudaStreamNonBlocking, greatestPri);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
      e = cudaEventCreateWithFlags(&lanes[l].marks[k].ev, cudaEventDisableTiming);
      lanes[l].marks[k].mirror = mirrors + 3 * l + k;
    }
  }
  if (e != cudaSuccess) return cuda_fail(e, "server creation");
  memset(&stats, 0, sizeof(stats));
  sched = std::thread([this] { loop(); });
  return GAS_OK;
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> lk(mu);
    stop = true;
  }
  cvWork.notify_all();
  if (sched.joinable()) sched.join();
  DeviceGuard dg(device);
  for (int l = 0; l < kMaxLanes; ++l) {
    Lane &L = lanes[l];
    if (L.stream) cudaStreamSynchronize(L.stream);
    if (L.streamHi) cudaStreamSynchronize(L.streamHi);
    L.batch.reset();
    for (auto &m : L.marks)
      if (m.ev) cudaEventDestroy(m.ev);
  }
  for (auto &kv : queries) {
    if (kv.second->batch && kv.second->batch->out) {
      cudaFreeAsync(kv.second->batch->out, fetch);
      kv.second->batch->out = nullptr;
    }
    delete kv.second;
  }
  queries.clear();
  for (int32_t *p : toFree) cudaFreeAsync(p, fetch);
  if (fetch) cudaStreamSynchronize(fetch);
  for (int l = 0; l < kMaxLanes; ++l) {
    if (lanes[l].stream) cudaStreamDestroy(lanes[l].stream);
    if (lanes[l].streamHi) cudaStreamDestroy(lanes[l].streamHi);
  }
  if (fetch) cudaStreamDestroy(fetch);
  for (ServeGraph *g : graphs) {
    if (!g) continue;
    gas_batch_destroy(g->batch);
    gas::internal::free_ppr_graph(&g->ppr);
    delete g;
  }
  if (mirrors) cudaFreeHost(mirrors);
  if (srcPinned) cudaFreeHost(srcPinned);
  if (pool) cudaMemPoolDestroy(pool);
}

// ------------------------------------------------------------ launching

template <int W, int KIND>
void round_pair(const gas::detail::BatchArgs &a, int r, unsigned *done, int blocks,
                cudaStream_t s) {
  gas::detail::batch_round_kernel<W, KIND><<<blocks, 256, 0, s>>>(a, r, done);
  // push-only batches (pairs, buckets): the tail is the end test alone
  const int tailBlocks = (a.pairMode || a.delta > 0) ? 1 : blocks;
  gas::detail::batch_tail_kernel<W><<<tailBlocks, 256, 0, s>>>(a, r, done);
}

template <int QP>
void ppr_round_launch(const gas::detail::PprArgs &a, int r, int blocks, cudaStream_t s) {
  gas::detail::ppr_round_kernel<QP><<<blocks, 256, 0, s>>>(a, r);
}

template <int QP>
void ppr_start_launch(const gas::detail::PprArgs &a, int blocks, cudaStream_t s) {
  gas::detail::ppr_init_kernel<QP><<<blocks, 256, 0, s>>>(a);
  gas::detail::ppr_sources_kernel<QP><<<1, kMaxQ, 0, s>>>(a);
}

// FN<QP>(args...) for the batch's PPR row width QP (a power of two <= 256).
#define GAS_PPR_WIDTH(QPV, FN, ...)               \
  switch (QPV) {                                  \
    case 1: FN<1>(__VA_ARGS__); break;            \
    case 2: FN<2>(__VA_ARGS__); break;            \
    case 4: FN<4>(__VA_ARGS__); break;            \
    case 8: FN<8>(__VA_ARGS__); break;            \
    case 16: FN<16>(__VA_ARGS__); break;          \
    case 32: FN<32>(__VA_ARGS__); break;          \
    case 64: FN<64>(__VA_ARGS__); break;          \
    case 128: FN<128>(__VA_ARGS__); break;        \
    default: FN<256>(__VA_ARGS__); break;         \
  }

// The batch engine's persistent kernel for a pair-frontier batch of a row
// width and program.
const void *batch_run_fn(int W, bool bfs) {
#define GAS_RUN_W(w)                                                                             \
  case w:                                                                                        \
    return bfs ? (const void *)gas::detail::batch_run_kernel<w, gas::detail::kBatchBFS, true>    \
               : (const void *)gas::detail::batch_run_kernel<w, gas::detail::kBatchSSSP, true>;
  switch (W) {
    GAS_RUN_W(1)
    GAS_RUN_W(2)
    GAS_RUN_W(4)
    default:
      GAS_RUN_W(8)
  }
#undef GAS_RUN_W
}

void enqueue_round(Batch &b, int r, int blocks) {
  unsigned *done = &b.ctl->done;
  const bool bfs = b.kind == 0;
#define GAS_SERVE_W(w)                                                                       \
  case w:                                                                                    \
    if (bfs)                                                                                 \
      round_pair<w, gas::detail::kBatchBFS>(b.ba, r, done, blocks, b.stream);                \
    else                                                                                     \
      round_pair<w, gas::detail::kBatchSSSP>(b.ba, r, done, blocks, b.stream);               \
    break;
  switch (b.W) {
    GAS_SERVE_W(1)
    GAS_SERVE_W(2)
    GAS_SERVE_W(4)
    default:
      GAS_SERVE_W(8)
  }
#undef GAS_SERVE_W
}

void enqueue_ppr_round(Batch &b, int r, int blocks) {
  GAS_PPR_WIDTH(b.Q, ppr_round_launch, b.pa, r, blocks, b.stream)
}

int round_blocks(const Server &s, int64_t warpsOfWork) {
  const int64_t full = (int64_t)s.sms * 4;  // the round kernels fit 4+ CTAs/SM
  const int64_t need = (warpsOfWork + 7) / 8;
  return (int)std::max<int64_t>(1, std::min(full, need));
}

// Queue `rounds` more rounds (BFS/SSSP) or the results' transpose (final),
// then the end test's event and control-word copy.
void Server::issue_chunk(int l, int rounds, bool final) {
  Lane &L = lanes[l];
  Batch &b = *L.batch;
  const int32_t V = b.g->bg.g.nV;
  if (final) {
    const int32_t *val = b.kind == 2 ? reinterpret_cast<const int32_t *>(b.pa.rank[kPprRounds & 1])
                                     : b.ba.value;
    dim3 tb(32, 8), tg((V + 31) / 32, (b.Q + 31) / 32);
    if (V > 0 && b.kind != 2 && b.pairs) {  // query-major already: copy the first nQ rows
      cudaMemcpyAsync(b.out, val, (size_t)b.nQ * V * 4, cudaMemcpyDeviceToDevice, b.stream);
    } else if (V > 0) {
      gas::detail::batch_transpose_kernel<<<tg, tb, 0, b.stream>>>(val, V, b.Q, b.nQ, b.out);
      launches += 1;
    }
  } else if (b.kind == 2) {
    const int G = 32 / std::min(b.Q, 32);  // units per warp
    const int blocks = round_blocks(*this, (b.g->ppr.units + G - 1) / G);
    for (int k = 0; k < rounds; ++k) enqueue_ppr_round(b, b.roundsIssued + k, blocks);
    b.roundsIssued += rounds;
    launches += rounds;
  } else {
    int blocks = round_blocks(*this, std::max<int64_t>(b.g->bg.nUnits, V));
    if (b.pairs) {
      // pair rounds walk the pair list only: a grid for about twice the
      // largest list seen so far (the rounds grid-stride past it), so that
      // a small batch's rounds need few block slots on a busy device
      const int64_t want = (2 * std::max<int64_t>(b.pairsSeen, b.nQ) + 512LL * b.nQ + 255) / 256;
      blocks = (int)std::max<int64_t>(1, std::min<int64_t>(blocks, want));
    }
    for (int k = 0; k < rounds; ++k) enqueue_round(b, b.roundsIssued + k, blocks);
    b.roundsIssued += rounds;
    launches += 2 * rounds;
  }
  int mi = 0;
  while (L.marks[mi].busy) ++mi;  // at most 2 in flight of 3
  ChunkMark &m = L.marks[mi];
  m.busy = true;
  m.final = final;
  cudaMemcpyAsync(m.mirror, b.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, b.stream);
  cudaEventRecord(m.ev, b.stream);
  L.queued.push_back(mi);
}

gas_status Server::launch(int l, const std::shared_ptr<Batch> &bp) {
  Batch &b = *bp;
  Lane &L = lanes[l];
  b.lane = l;
  b.stream = b.pairs ? L.streamHi : L.stream;
  const ServeGraph &g = *b.g;
  const int32_t V = g.bg.g.nV;
  const size_t Vs = (size_t)std::max(V, 1);
  cudaError_t e = cudaMallocFromPoolAsync((void **)&b.state, (size_t)b.stateBytes, pool, b.stream);
  if (e == cudaSuccess)
    e = cudaMallocFromPoolAsync((void **)&b.out, (size_t)b.outBytes, pool, b.stream);
  if (e != cudaSuccess) {
    if (b.state) cudaFreeAsync(b.state, b.stream);
    b.state = nullptr;
    b.out = nullptr;
    cudaGetLastError();
    return cuda_fail(e, "batch state allocation");
  }
  bytesInUse += b.stateBytes + b.outBytes;
  // carve the state: ctl | sources | arrays (256-byte aligned)
  unsigned char *p = b.state;
  auto take = [&p](size_t n) {
    unsigned char *r = p;
    p += (n + 255) & ~(size_t)255;
    return r;
  };
  b.ctl = reinterpret_cast<Ctl *>(take(sizeof(Ctl)));
  b.sources = reinterpret_cast<int32_t *>(take(4 * kMaxQ));
  // the lane's pinned staging is free: its previous batch has ended
  int32_t *src = srcPinned + (size_t)l * kMaxQ;
  for (int i = 0; i < b.nQ; ++i) src[i] = b.queries[i]->source;
  cudaMemsetAsync(b.ctl, 0, sizeof(Ctl), b.stream);
  cudaMemcpyAsync(b.sources, src, 4 * (size_t)b.nQ, cudaMemcpyHostToDevice, b.stream);
  const size_t W = (size_t)b.W;
  if (b.kind == 2) {
    gas::detail::PprArgs &a = b.pa;
    memset(&a, 0, sizeof(a));
    a.nVertices = V;
    a.nQueries = b.nQ;
    a.inSources = g.bg.g.inSrc;
    gas::detail::ppr_args_graph(a, g.bg.g.inSrc, g.ppr.outDegree, g.ppr.lastActive, g.ppr.mem,
                                g.ppr.units, g.ppr.slots);
    a.sources = b.sources;
    for (int k = 0; k < 2; ++k) {
      a.rank[k] = reinterpret_cast<float *>(take(Vs * b.Q * 4));
      a.contrib[k] = reinterpret_cast<float *>(take(Vs * b.Q * 4));
    }
    a.partial = reinterpret_cast<float *>(take((size_t)g.ppr.slots * b.Q * 4));
    a.arrive = reinterpret_cast<unsigned *>(take((size_t)g.ppr.hubs * 4));
    if (g.ppr.hubs > 0) cudaMemsetAsync(a.arrive, 0, (size_t)g.ppr.hubs * 4, b.stream);
    if (p - b.state > b.stateBytes) return fail(GAS_ERR_STATE, "batch state layout overflow");
    a.teleport = 0.15f;
    a.damp = 1.0f - a.teleport;  // as PPR::apply computes it, in float
    const int blocks = 4 * sms;
    GAS_PPR_WIDTH(b.Q, ppr_start_launch, a, blocks, b.stream)
  } else {
    gas::detail::BatchArgs &a = b.ba;
    memset(&a, 0, sizeof(a));
    a.nVertices = V;
    a.nEdges = g.bg.g.nE;
    a.outOffsets = g.bg.g.outOff;
    a.outDests = g.bg.g.outDst;
    a.weightsOut = g.bg.weightsOut;
    a.alpha = 10;
    a.nQueries = b.Q;
    a.inSources = g.bg.g.inSrc;
    a.weights = reinterpret_cast<const int32_t *>(g.bg.g.edgeData);
    a.unitV = g.bg.unitV;
    a.unitBeg = g.bg.unitBeg;
    a.unitEnd = g.bg.unitEnd;
    a.nUnits = g.bg.nUnits;
    a.value = reinterpret_cast<int32_t *>(take(Vs * b.Q * 4));
    const size_t cap = (size_t)gas::detail::batch_list_capacity(V, g.bg.g.nE);
    for (int k = 0; k < 3; ++k) {
      a.mask[k] = reinterpret_cast<unsigned *>(take(Vs * W * 4));
      a.list[k] = reinterpret_cast<int32_t *>(take(cap * 4));
      a.listC[k] = reinterpret_cast<int32_t *>(take(cap * 4));
    }
    a.inList = reinterpret_cast<int32_t *>(take(Vs * 4));
    a.seen = b.kind == 0 ? reinterpret_cast<unsigned *>(take(Vs * W * 4)) : nullptr;
    a.pairMode = b.pairs ? 1 : 0;
    for (int k = 0; k < 3; ++k)
      a.pairs[k] = b.pairs ? reinterpret_cast<uint32_t *>(take(Vs * b.Q * 4)) : nullptr;
    a.delta = b.kind == 1 ? b.delta : 0;
    for (int k = 0; k < 2; ++k) a.thresh[k] = reinterpret_cast<int32_t *>(take(4 * kMaxQ));
    for (int k = 0; k < 3; ++k) a.nearFlag[k] = reinterpret_cast<unsigned *>(take(4 * 8));
    if (p - b.state > b.stateBytes) return fail(GAS_ERR_STATE, "batch state layout overflow");
    a.cnt = b.ctl->cnt;
    a.barrier = b.ctl->bar;
    a.errWord = &b.ctl->err;
    a.roundsOut = &b.ctl->rounds;
    a.listCnt = b.ctl->listCnt;
    a.maxRounds = 0;
    for (int k = 0; k < 3; ++k) cudaMemsetAsync(a.mask[k], 0, Vs * W * 4, b.stream);
    if (a.seen) cudaMemsetAsync(a.seen, 0, Vs * W * 4, b.stream);
    cudaMemsetAsync(a.inList, 0xff, Vs * 4, b.stream);
    for (int k = 0; k < 3; ++k) cudaMemsetAsync(a.nearFlag[k], 0, 4 * 8, b.stream);
    const int kb = b.kind == 0 ? gas::detail::kBatchBFS : gas::detail::kBatchSSSP;
    gas::detail::batch_init_kernel<<<4 * sms, 256, 0, b.stream>>>(kb, V, b.Q, a.value,
                                                                    a.thresh[0], a.delta);
    gas::detail::batch_sources_kernel<<<(b.nQ + 127) / 128, 128, 0, b.stream>>>(
        kb, b.nQ, b.Q, b.W, V, b.sources, a.value, a.mask[0], a.seen, g.bg.g.outOff, a.inList,
        a.list[0], a.listC[0], a.listCnt, b.pairs ? a.pairs[0] : nullptr);
  }
  launches += 2;  // init + sources
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "batch start");
  L.batch = bp;
  if (b.kind != 2 && b.pairs && persistentRunning < kMaxPersistent) {
    // A pair-frontier batch (lattice-like graph: thousands of small rounds)
    // runs every round in one cooperative launch of the batch engine's
    // kernel on its lane's high-priority stream, on a third of the device's
    // co-resident blocks: its rounds then no longer queue behind other
    // lanes' launches.  At most kMaxPersistent such batches run at once, so
    // their grids fit the device together; the other lanes' kernels are
    // ordinary and finite, so a partly placed grid waits for their blocks
    // to finish, and every grid-barrier wait in it is bounded.
    const void *fn = batch_run_fn(b.W, b.kind == 0);
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 256, 0);
    const int blocks = std::max(1, per * sms / 3);
    void *args[] = {&b.ba};
    e = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(256), args, 0, b.stream);
    if (e == cudaSuccess) {
      b.persistent = true;
      ++persistentRunning;
      launches += 1;
      issue_chunk(l, 0, true);
      return GAS_OK;
    }
    cudaGetLastError();  // cannot launch cooperatively: round by round below
  }
  if (b.kind == 2) {
    issue_chunk(l, kPprRounds, false);
    issue_chunk(l, 0, true);
  } else {
    issue_chunk(l, b.chunk, false);
    b.chunk = std::min(kMaxChunk, b.chunk * 2);
    issue_chunk(l, b.chunk, false);
    b.chunk = std::min(kMaxChunk, b.chunk * 2);
  }
  return GAS_OK;
}

// Completes a lane's batch: queries get status and timestamps; working
// state goes back to the pool; results stay until fetched.
void Server::finish_batch(int l, gas_status st, int32_t rounds) {
  Lane &L = lanes[l];
  std::shared_ptr<Batch> bp = L.batch;
  Batch &b = *bp;
  if (b.persistent) {
    --persistentRunning;
    b.persistent = false;
  }
  if (b.state) {
    cudaFreeAsync(b.state, b.stream);
    bytesInUse -= b.stateBytes;
    b.state = nullptr;
  }
  if (st != GAS_OK && b.out) {
    cudaFreeAsync(b.out, b.stream);
    bytesInUse -= b.outBytes;
    b.out = nullptr;
  }
  const int64_t t = now_ns();
  {
    std::lock_guard<std::mutex> lk(mu);
    for (Query *q : b.queries) {
      q->info.status = st;
      q->info.rounds = rounds;
      q->info.doneNs = t;
      q->done = true;
      if (st == GAS_OK) ++stats.completed; else ++stats.failed;
    }
    --stats.running;
    if (st == GAS_OK) {
      int64_t &c = cellRunNs[b.cell];
      const int64_t d = t - b.admitNs;
      c = c == 0 ? d : (3 * c + d) / 4;
    }
  }
  L.batch.reset();
  L.queued.clear();
  for (auto &m : L.marks) m.busy = false;
  cvDone.notify_all();
}

bool Server::poll_lane(int l) {
  Lane &L = lanes[l];
  if (!L.batch || L.queued.empty()) return false;
  ChunkMark &m = L.marks[L.queued.front()];
  const cudaError_t q = cudaEventQuery(m.ev);
  if (q == cudaErrorNotReady) return false;
  if (q != cudaSuccess) {
    cuda_fail(q, "batch round");
    finish_batch(l, GAS_ERR_CUDA, 0);
    return true;
  }
  L.queued.pop_front();
  m.busy = false;
  Batch &b = *L.batch;
  const Ctl c = *m.mirror;
  for (int k = 0; k < 3; ++k) b.pairsSeen = std::max<int64_t>(b.pairsSeen, (int64_t)(c.listCnt[k] >> 32));
  if (m.final) {
    finish_batch(l, c.err ? GAS_ERR_TIMEOUT : GAS_OK, b.kind == 2 ? kPprRounds : c.rounds);
    return true;
  }
  if (b.kind == 2) return true;  // the final mark is already queued
  const bool finalQueued = !L.queued.empty() && L.marks[L.queued.back()].final;
  if (c.done || c.err) {
    if (!finalQueued) issue_chunk(l, 0, true);
    return true;
  }
  if (!finalQueued) {
    issue_chunk(l, b.chunk, false);
    b.chunk = std::min(kMaxChunk, b.chunk * 2);
  }
  return true;
}

// Starts batches on free lanes, as many queries of one (graph, program)
// queue as memory admits.  A queue is ready once it holds a full batch or
// its oldest query has waited 1/kWindowDiv of the queue's recent batch run
// time (at most kWindowMaxNs): a queue whose batches run long collects the
// queries of a burst into one batch instead of starting one batch per
// arrival.  Of the ready queues, the one holding the oldest query goes
// first -- except among queues whose oldest queries arrived within kTieNs
// of it (a burst), where the one with the longest recent batch run time
// goes first, so that the longest batches do not start last.
bool Server::admit() {
  bool any = false;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (stop) return false;  // queries not yet started are dropped
  }
  for (int l = 0; l < cfg.lanes; ++l) {
    if (lanes[l].batch) continue;
    std::shared_ptr<Batch> bp;
    {
      std::lock_guard<std::mutex> lk(mu);
      const int64_t tNow = now_ns();
      auto ready = [&](size_t i) {
        if (pending[i].empty()) return false;
        const int64_t window = std::min(cellRunNs[i] / kWindowDiv, kWindowMaxNs);
        return (int64_t)pending[i].size() >= cfg.maxBatch ||
               tNow - pending[i].front()->info.submitNs >= window;
      };
      int64_t oldest = 0;
      bool anyReady = false;
      for (size_t i = 0; i < pending.size(); ++i)
        if (ready(i) && (!anyReady || pending[i].front()->info.submitNs < oldest)) {
          oldest = pending[i].front()->info.submitNs;
          anyReady = true;
        }
      int best = -1;
      for (size_t i = 0; anyReady && i < pending.size(); ++i) {
        if (!ready(i) || pending[i].front()->info.submitNs > oldest + kTieNs) continue;
        if (best < 0 || cellRunNs[i] > cellRunNs[best] ||
            (cellRunNs[i] == cellRunNs[best] &&
             pending[i].front()->info.submitNs < pending[best].front()->info.submitNs))
          best = (int)i;
      }
      if (best < 0) return any;
      std::deque<Query *> &pq = pending[best];
      ServeGraph *g = graphs[best / kKinds];
      const int kind = best % kKinds;
      int nQ = (int)std::min<size_t>(pq.size(), (size_t)cfg.maxBatch);
      const int64_t avail = available_bytes();
      auto need = [&](int n) {
        return state_bytes(*g, kind, row_width(kind, n)) + (int64_t)std::max(g->bg.g.nV, 1) * n * 4;
      };
      bool shrunk = false;
      while (nQ > 0 && need(nQ) > avail) {
        nQ = nQ > 32 ? ((nQ - 1) / 32) * 32 : nQ / 2;
        shrunk = true;
      }
      if (shrunk) ++stats.memoryWaits;
      if (nQ == 0) {
        // wait while running batches or unfetched results hold memory
        bool idle = bytesInUse.load() == 0;
        for (int k = 0; k < cfg.lanes; ++k) idle = idle && !lanes[k].batch;
        if (!idle) return any;
        Query *q = pq.front();  // cannot fit even alone on an idle device
        pq.pop_front();
        q->info.status = fail(GAS_ERR_OOM, "query needs %lld bytes of device memory",
                              (long long)need(1));
        q->info.doneNs = now_ns();
        q->done = true;
        ++stats.failed;
        --stats.pending;
        cvDone.notify_all();
        any = true;
        --l;  // try this lane again
        continue;
      }
      bp = std::make_shared<Batch>();
      bp->g = g;
      bp->kind = kind;
      bp->cell = (size_t)best;
      bp->nQ = nQ;
      bp->Q = row_width(kind, nQ);
      bp->W = std::max(bp->Q / 32, 1);
      bp->pairs = use_pairs(*g, kind, bp->Q);
      // distance buckets for SSSP on pair-frontier (high-diameter) graphs
      bp->delta = (kind == 1 && bp->pairs) ? 4 * std::max(g->maxWeight, 1) : 0;
      bp->stateBytes = state_bytes(*g, kind, bp->Q);
      bp->outBytes = (int64_t)std::max(g->bg.g.nV, 1) * nQ * 4;
      bp->unfetched = nQ;
      bp->server = this;
      bp->admitNs = now_ns();
      for (int i = 0; i < nQ; ++i) {
        Query *q = pq.front();
        pq.pop_front();
        q->batch = bp;
        q->slot = i;
        q->info.admitNs = bp->admitNs;
        q->info.batchSize = nQ;
        q->info.lane = l;
        bp->queries.push_back(q);
      }
      stats.pending -= nQ;
      ++stats.batches;
      stats.batchedQueries += nQ;
      ++stats.running;
    }
    gas_status st = launch(l, bp);
    if (st != GAS_OK) {
      lanes[l].batch = bp;
      finish_batch(l, st, 0);
    }
    const int64_t u = bytesInUse.load();
    {
      std::lock_guard<std::mutex> lk(mu);
      stats.peakBytesInUse = std::max(stats.peakBytesInUse, u);
    }
    any = true;
  }
  return any;
}

void Server::loop() {
  cudaSetDevice(device);
  for (;;) {
    {
      std::lock_guard<std::mutex> lk(freeMu);
      for (int32_t *p : toFree) cudaFreeAsync(p, fetch);
      toFree.clear();
    }
    bool busy = false;
    for (int l = 0; l < cfg.lanes; ++l)
      while (poll_lane(l)) busy = true;
    busy = admit() || busy;
    bool running = false;
    for (int l = 0; l < cfg.lanes; ++l) running = running || (bool)lanes[l].batch;
    std::unique_lock<std::mutex> lk(mu);
    if (stop && !running) return;
    if (busy) continue;
    if (running) {
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(20));
    } else {
      bool waiting = false;
      for (auto &pq : pending) waiting = waiting || !pq.empty();
      if (!waiting && !stop) {
        cvWork.wait_for(lk, std::chrono::milliseconds(2));
      } else if (waiting) {  // queries inside their batching window
        lk.unlock();
        std::this_thread::sleep_for(std::chrono::microseconds(20));
      }
    }
  }
}

}  // namespace

namespace {

// PPR structures of a graph: out-degrees; work units (a vertex's in-edges,
// hubs cut into kPprChunk-edge chunks with partial-sum slots), ordered
// longest first by a counting sort; and lastActive[v], the last of the
// `rounds` rounds in which v is active, from rounds - 1 pull steps of the
// source-independent active sets on the device.
gas_status build_ppr(ServeGraph &g, int sms) {
  return gas::internal::build_ppr_graph(g.bg.g, sms, kPprRounds, &g.ppr);
}

}  // namespace

struct gas_server_s {
  Server *impl;
};

extern "C" {

gas_status gas_server_create(int32_t device, const gas_server_config *cfg, gas_server **out) {
  if (!out) return fail(GAS_ERR_INVALID, "gas_server_create: out is NULL");
  *out = nullptr;
  gas_server_config c;
  c.lanes = 4;
  c.maxBatch = kMaxQ;
  c.reserveBytes = 1ll << 30;
  if (cfg) c = *cfg;
  if (c.lanes < 1 || c.lanes > kMaxLanes) return fail(GAS_ERR_INVALID, "lanes must be in [1, 16]");
  if (c.maxBatch < 1 || c.maxBatch > kMaxQ)
    return fail(GAS_ERR_INVALID, "maxBatch must be in [1, 256]");
  if (c.reserveBytes < 0) return fail(GAS_ERR_INVALID, "reserveBytes must be >= 0");
  if (!gas_device_supported(device)) return fail(GAS_ERR_NO_DEVICE, "device %d is not sm_103", device);
  Server *s = new (std::nothrow) Server();
  gas_server *h = new (std::nothrow) gas_server_s();
  if (!s || !h) {
    delete s;
    delete h;
    return fail(GAS_ERR_OOM, "host allocation");
  }
  s->device = device;
  s->cfg = c;
  gas_status st = s->start();
  if (st) {
    delete s;
    delete h;
    return st;
  }
  h->impl = s;
  *out = h;
  return GAS_OK;
}

gas_status gas_server_destroy(gas_server *h) {
  if (!h) return GAS_OK;
  delete h->impl;
  delete h;
  return GAS_OK;
}

gas_status gas_server_add_graph(gas_server *h, int32_t nVertices, int32_t nEdges,
                                const int32_t *srcs, const int32_t *dsts, const int32_t *weights,
                                int32_t *graphId) {
  if (!h || !graphId) return fail(GAS_ERR_INVALID, "null argument");
  Server &s = *h->impl;
  if (nVertices < 0 || nEdges < 0 || (nEdges > 0 && (!srcs || !dsts)))
    return fail(GAS_ERR_INVALID, "bad edge list");
  DeviceGuard dg(s.device);
  // admission of the graph itself: CSC + CSR + weights (both orders) + units
  const int64_t need = (int64_t)nEdges * (weights ? 20 : 12) + (int64_t)nVertices * 24 + (1 << 20);
  if (need > s.available_bytes())
    return fail(GAS_ERR_OOM, "graph needs %lld bytes of device memory", (long long)need);
  ServeGraph *g = new (std::nothrow) ServeGraph();
  if (!g) return fail(GAS_ERR_OOM, "host allocation");
  gas_status st = gas_batch_create(s.device, nullptr, &g->batch);
  if (st == GAS_OK) st = gas_batch_set_graph(g->batch, nVertices, nEdges, srcs, dsts, weights);
  if (st == GAS_OK && !gas::internal::batch_graph(g->batch, &g->bg))
    st = fail(GAS_ERR_STATE, "graph upload");
  if (st == GAS_OK) st = build_ppr(*g, s.sms);
  if (st != GAS_OK) {
    gas_batch_destroy(g->batch);
    gas::internal::free_ppr_graph(&g->ppr);
    delete g;
    return st;
  }
  g->weighted = weights != nullptr;
  g->bytes = need;
  {
    const std::vector<int32_t> &off = *g->bg.g.hOutOff;
    for (int32_t v = 0; v < nVertices; ++v) g->maxOutDeg = std::max(g->maxOutDeg, off[v + 1] - off[v]);
    for (int32_t i = 0; weights && i < nEdges; ++i) g->maxWeight = std::max(g->maxWeight, weights[i]);
  }
  std::lock_guard<std::mutex> lk(s.mu);
  g->id = (int32_t)s.graphs.size();
  s.graphs.push_back(g);
  s.pending.resize(s.graphs.size() * kKinds);
  s.cellRunNs.resize(s.graphs.size() * kKinds, 0);
  *graphId = g->id;
  return GAS_OK;
}

gas_status gas_server_submit(gas_server *h, int32_t graphId, int32_t program, int32_t source,
                             uint64_t *ticket) {
  if (!h || !ticket) return fail(GAS_ERR_INVALID, "null argument");
  Server &s = *h->impl;
  const int kind = kind_of(program);
  if (kind < 0) return fail(GAS_ERR_UNSUPPORTED, "served programs are BFS, SSSP and PPR");
  Query *q = new (std::nothrow) Query();
  if (!q) return fail(GAS_ERR_OOM, "host allocation");
  {
    std::lock_guard<std::mutex> lk(s.mu);
    if (graphId < 0 || graphId >= (int32_t)s.graphs.size()) {
      delete q;
      return fail(GAS_ERR_INVALID, "no graph %d", graphId);
    }
    const ServeGraph &g = *s.graphs[graphId];
    if (source < 0 || source >= g.bg.g.nV) {
      delete q;
      return fail(GAS_ERR_INVALID, "source %d outside [0, %d)", source, g.bg.g.nV);
    }
    if (kind == 1 && !g.weighted) {
      delete q;
      return fail(GAS_ERR_STATE, "SSSP needs a graph added with weights");
    }
    memset(&q->info, 0, sizeof(q->info));
    q->ticket = s.nextTicket++;
    q->graph = graphId;
    q->program = program;
    q->source = source;
    q->kind = kind;
    q->info.program = program;
    q->info.graph = graphId;
    q->info.source = source;
    q->info.submitNs = now_ns();
    s.queries[q->ticket] = q;
    s.pending[(size_t)graphId * kKinds + kind].push_back(q);
    ++s.stats.submitted;
    ++s.stats.pending;
    *ticket = q->ticket;
  }
  s.cvWork.notify_one();
  return GAS_OK;
}

gas_status gas_server_poll(gas_server *h, uint64_t ticket, int32_t *done) {
  if (!h || !done) return fail(GAS_ERR_INVALID, "null argument");
  Server &s = *h->impl;
  std::lock_guard<std::mutex> lk(s.mu);
  auto it = s.queries.find(ticket);
  if (it == s.queries.end()) return fail(GAS_ERR_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
  *done = it->second->done ? 1 : 0;
  return GAS_OK;
}

gas_status gas_server_wait(gas_server *h, uint64_t ticket, int32_t timeoutMs, void *result,
                           int64_t resultBytes, gas_query_info *info) {
  if (!h) return fail(GAS_ERR_INVALID, "server is NULL");
  Server &s = *h->impl;
  Query *q = nullptr;
  {
    std::unique_lock<std::mutex> lk(s.mu);
    auto it = s.queries.find(ticket);
    if (it == s.queries.end())
      return fail(GAS_ERR_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
    q = it->second;
    auto ready = [q] { return q->done; };
    if (timeoutMs < 0) {
      s.cvDone.wait(lk, ready);
    } else if (!s.cvDone.wait_for(lk, std::chrono::milliseconds(timeoutMs), ready)) {
      return fail(GAS_ERR_TIMEOUT, "query %llu still running", (unsigned long long)ticket);
    }
    s.queries.erase(it);
  }
  gas_status st = q->info.status;
  std::shared_ptr<Batch> b = q->batch;
  const int32_t V = b ? b->g->bg.g.nV : 0;
  if (st == GAS_OK && result && b && b->out) {
    if (resultBytes < (int64_t)V * 4) {
      st = fail(GAS_ERR_INVALID, "result buffer of %lld bytes, %lld needed", (long long)resultBytes,
                (long long)V * 4);
    } else if (V > 0) {
      std::lock_guard<std::mutex> lk(s.fetchMu);
      DeviceGuard dg(s.device);
      cudaError_t e = cudaMemcpyAsync(result, b->out + (size_t)q->slot * V, (size_t)V * 4,
                                      cudaMemcpyDeviceToHost, s.fetch);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s.fetch);
      if (e != cudaSuccess) st = cuda_fail(e, "result copy");
    }
  }
  if (info) *info = q->info;
  if (b) {
    std::lock_guard<std::mutex> lk(s.freeMu);
    if (--b->unfetched == 0 && b->out) {
      s.toFree.push_back(b->out);
      s.bytesInUse -= b->outBytes;
      b->out = nullptr;
    }
  }
  delete q;
  return st;
}

gas_status gas_server_get_stats(gas_server *h, gas_server_stats *st) {
  if (!h || !st) return fail(GAS_ERR_INVALID, "null argument");
  Server &s = *h->impl;
  std::lock_guard<std::mutex> lk(s.mu);
  *st = s.stats;
  st->bytesInUse = s.bytesInUse.load();
  st->kernelLaunches = s.launches.load();
  return GAS_OK;
}

}  // extern "C"

namespace gas {
namespace internal {

gas_status build_ppr_graph(const CoreGraph &cg, int sms, int rounds, PprGraph *out) {
  PprGraph &g = *out;
  free_ppr_graph(out);
  constexpr int C = gas::detail::kPprChunk;
  const int32_t V = cg.nV;
  const std::vector<int32_t> &inOff = *cg.hInOff, &outOff = *cg.hOutOff;
  std::vector<int32_t> deg((size_t)std::max(V, 1), 0);
  for (int32_t v = 0; v < V; ++v) deg[v] = outOff[(size_t)v + 1] - outOff[v];
  std::vector<int32_t> uv, ub, ul, us, sf, sc, sh;
  uv.reserve(V);
  ub.reserve(V);
  ul.reserve(V);
  us.reserve(V);
  int32_t hubs = 0;
  for (int32_t v = 0; v < V; ++v) {
    const int32_t b = inOff[v], d = inOff[(size_t)v + 1] - b;
    if (d <= C) {
      uv.push_back(v); ub.push_back(b); ul.push_back(d); us.push_back(-1);
      continue;
    }
    const int32_t n = (d + C - 1) / C, first = (int32_t)sf.size();
    for (int32_t c = 0; c < n; ++c) {
      uv.push_back(v); ub.push_back(b + c * C); ul.push_back(std::min(C, d - c * C));
      us.push_back(first + c);
      sf.push_back(first); sc.push_back(n); sh.push_back(hubs);
    }
    ++hubs;
  }
  const size_t nu = uv.size(), ns = sf.size();
  // counting sort by length, longest first (stable)
  std::vector<int64_t> pos((size_t)C + 2, 0);
  for (size_t i = 0; i < nu; ++i) ++pos[(size_t)(C - ul[i]) + 1];
  for (size_t k = 1; k < pos.size(); ++k) pos[k] += pos[k - 1];
  std::vector<int32_t> mem(4 * std::max<size_t>(nu, 1) + 3 * std::max<size_t>(ns, 1), 0);
  const size_t nuA = std::max<size_t>(nu, 1), nsA = std::max<size_t>(ns, 1);
  for (size_t i = 0; i < nu; ++i) {
    const size_t p = (size_t)pos[(size_t)(C - ul[i])]++;
    mem[p] = uv[i];
    mem[nuA + p] = ub[i];
    mem[2 * nuA + p] = ul[i];
    mem[3 * nuA + p] = us[i];
  }
  for (size_t i = 0; i < ns; ++i) {
    mem[4 * nuA + i] = sf[i];
    mem[4 * nuA + nsA + i] = sc[i];
    mem[4 * nuA + 2 * nsA + i] = sh[i];
  }
  g.units = (int32_t)nu;
  g.slots = (int32_t)ns;
  g.hubs = hubs;
  uint8_t *tmp = nullptr;
  const size_t Vs = (size_t)std::max(V, 1);
  cudaError_t e = cudaMalloc(&g.outDegree, 4 * Vs);
  if (e == cudaSuccess) e = cudaMalloc(&g.mem, 4 * mem.size());
  if (e == cudaSuccess) e = cudaMalloc(&g.lastActive, Vs);
  if (e == cudaSuccess) e = cudaMalloc(&tmp, 2 * Vs);
  if (e == cudaSuccess) e = cudaMemcpy(g.outDegree, deg.data(), 4 * Vs, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(g.mem, mem.data(), 4 * mem.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(g.lastActive, 0, Vs);
  if (e == cudaSuccess) e = cudaMemset(tmp, 1, Vs);  // A0: every vertex
  for (int k = 1; k < rounds && e == cudaSuccess && V > 0; ++k) {
    uint8_t *cur = tmp + ((k - 1) & 1) * Vs, *nxt = tmp + (k & 1) * Vs;
    gas::detail::ppr_active_step_kernel<<<4 * sms, 256>>>(V, cg.inOff, cg.inSrc, cur, nxt,
                                                           g.lastActive, k);
    e = cudaGetLastError();
  }
  // the legacy default stream: ordered after the memsets, not with the lanes
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (tmp) cudaFree(tmp);
  if (e != cudaSuccess) {
    free_ppr_graph(out);
    return cuda_fail(e, "PPR graph structures");
  }
  return GAS_OK;
}

void free_ppr_graph(PprGraph *p) {
  if (p->outDegree) cudaFree(p->outDegree);
  if (p->lastActive) cudaFree(p->lastActive);
  if (p->mem) cudaFree(p->mem);
  *p = PprGraph();
}

}  // namespace internal
}  // namespace gas
