// Batched multi-source BFS / SSSP / personalised PageRank (gas_batch_* in
// gas_gb300.h).
//
// Many queries with their own sources on one resident graph: each batch of
// up to 256 queries is one persistent cooperative launch (kernels in
// gas_gb300/detail/batch.cuh; PPR's round body is the serving loop's, in
// gas_gb300/detail/serve.cuh), and the whole batch -- source upload, state
// reset, the run and the query-major transpose of the results -- is
// captured once per shape into a CUDA graph and replayed.  Work units (a
// vertex's in-edges, hubs split into chunks), the push/pull switch, the
// frontier form and the launch shape are chosen by gas_batch_autotune.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "gas_gb300.h"
#include "gas_gb300_core.h"
#include "gas_gb300/detail/serve.cuh"
#include "gas_internal.h"

using gas::internal::CoreGraph;
using gas::internal::cuda_fail;
using gas::internal::fail;

namespace {

constexpr int kMaxBatch = 256;  // queries per launch (8 words of query bits)
constexpr int kKindPPR = 3;     // GraphCache kind of a PPR batch

struct GraphCache {
  int kind, W, nQ, blocksPerSM, chunk, delta, pairs;
  cudaGraphExec_t exec;
};

}  // namespace

struct gas_batch_s {
  gas_core *core = nullptr;
  int device = 0;
  cudaStream_t stream = nullptr;
  int sms = 0;
  int32_t chunk = 256;
  int32_t blocksPerSM = 0;  // 0 = as many as fit
  bool useGraphs = true;
  int32_t alpha = 10;  // push round when list out-degree total * alpha <= E
  int32_t delta = 0;   // SSSP bucket width (0 = Bellman-Ford rounds)
  int32_t frontier = -1;  // -1 automatic, 0 vertex masks, 1 (vertex, query) pairs
  int32_t maxOutDeg = 0;
  uint32_t *pairs[3] = {nullptr, nullptr, nullptr};
  size_t pairCap = 0;
  int32_t *bucketMem = nullptr;  // thresh[2][256] | nearFlag[3][8]
  int32_t unitChunk = 0;
  int32_t *list[3] = {nullptr, nullptr, nullptr};
  int32_t *listC[3] = {nullptr, nullptr, nullptr};
  int32_t *inList = nullptr;
  int32_t *weightsOut = nullptr;  // CSR order
  int32_t *unitV = nullptr, *unitBeg = nullptr, *unitEnd = nullptr;
  int32_t nUnits = 0;
  int32_t capQ = 0;
  int32_t *value = nullptr, *srcDev = nullptr, *outDev = nullptr;
  unsigned *mask[3] = {nullptr, nullptr, nullptr};
  unsigned *seen = nullptr;
  unsigned char *ctl = nullptr;  // cnt[3] | barrier[2] | rounds | err
  int32_t *srcPinned = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  float lastMs = 0.f;
  std::vector<GraphCache> graphs;
  // personalised PageRank: the graph's PPR structures (built at the first
  // PPR batch) and the batch state for rows of pprQP queries
  gas::internal::PprGraph ppr;
  int32_t pprRounds = 20;
  unsigned char *pprState = nullptr;
  int32_t pprQP = 0;
};

namespace {

// control block: cnt[3] | barrier[2] | rounds | err | listCnt[3]
struct CtlView {
  unsigned long long *cnt;
  unsigned *bar;
  int32_t *rounds;
  unsigned *err;
  unsigned long long *listCnt;
};
CtlView ctl_view(gas_batch *b) {
  CtlView v;
  v.cnt = reinterpret_cast<unsigned long long *>(b->ctl);
  v.bar = reinterpret_cast<unsigned *>(b->ctl + 24);
  v.rounds = reinterpret_cast<int32_t *>(b->ctl + 32);
  v.err = reinterpret_cast<unsigned *>(b->ctl + 36);
  v.listCnt = reinterpret_cast<unsigned long long *>(b->ctl + 40);
  return v;
}
constexpr size_t kCtlBytes = 64;

void drop_graphs(gas_batch *b) {
  for (auto &g : b->graphs) cudaGraphExecDestroy(g.exec);
  b->graphs.clear();
}

void free_state(gas_batch *b) {
  void *ps[] = {b->value, b->srcDev, b->outDev, b->mask[0], b->mask[1], b->mask[2], b->seen,
                b->list[0], b->list[1], b->list[2], b->listC[0], b->listC[1], b->listC[2],
                b->inList};
  for (void *p : ps)
    if (p) cudaFree(p);
  b->value = b->srcDev = b->outDev = nullptr;
  b->mask[0] = b->mask[1] = b->mask[2] = nullptr;
  b->seen = nullptr;
  b->list[0] = b->list[1] = b->list[2] = nullptr;
  b->listC[0] = b->listC[1] = b->listC[2] = nullptr;
  b->inList = nullptr;
  for (int k = 0; k < 3; ++k) {
    if (b->pairs[k]) cudaFree(b->pairs[k]);
    b->pairs[k] = nullptr;
  }
  b->pairCap = 0;
  b->capQ = 0;
  if (b->pprState) cudaFree(b->pprState);
  b->pprState = nullptr;
  b->pprQP = 0;
  drop_graphs(b);
}

// Pair frontier for graphs whose out-degrees are small (a lane walks a
// vertex's out-edges alone) and whose V * Q entries fit 32 bits.
bool use_pairs(const gas_batch *b, const CoreGraph &g, int32_t Q) {
  const bool allowed = b->maxOutDeg <= 64 && (long long)g.nV * Q < (1ll << 31);
  return b->frontier == 0 ? false : allowed;
}

gas_status ensure_pairs(gas_batch *b, const CoreGraph &g, int32_t Q) {
  const size_t need = (size_t)std::max(g.nV, 1) * Q;
  if (b->pairCap >= need) return GAS_OK;
  for (int k = 0; k < 3; ++k) {
    if (b->pairs[k]) cudaFree(b->pairs[k]);
    b->pairs[k] = nullptr;
  }
  b->pairCap = 0;
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaMalloc(&b->pairs[k], need * 4);
  if (e != cudaSuccess) return cuda_fail(e, "batch pair lists");
  b->pairCap = need;
  drop_graphs(b);
  return GAS_OK;
}

void free_units(gas_batch *b) {
  if (b->unitV) cudaFree(b->unitV);
  if (b->unitBeg) cudaFree(b->unitBeg);
  if (b->unitEnd) cudaFree(b->unitEnd);
  b->unitV = b->unitBeg = b->unitEnd = nullptr;
  b->nUnits = 0;
  b->unitChunk = 0;
  drop_graphs(b);
}

gas_status build_units(gas_batch *b, const CoreGraph &g, int32_t chunk) {
  if (b->unitChunk == chunk && b->unitV) return GAS_OK;
  free_units(b);
  std::vector<int32_t> uv, ub, ue;
  const std::vector<int32_t> &off = *g.hInOff;
  for (int32_t v = 0; v < g.nV; ++v)
    for (int32_t e = off[v]; e < off[(size_t)v + 1]; e += chunk) {
      uv.push_back(v);
      ub.push_back(e);
      ue.push_back(std::min(e + chunk, off[(size_t)v + 1]));
    }
  const size_t n = std::max<size_t>(uv.size(), 1);
  cudaError_t e = cudaMalloc(&b->unitV, n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&b->unitBeg, n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&b->unitEnd, n * 4);
  if (e == cudaSuccess && !uv.empty()) {
    cudaMemcpyAsync(b->unitV, uv.data(), uv.size() * 4, cudaMemcpyHostToDevice, b->stream);
    cudaMemcpyAsync(b->unitBeg, ub.data(), ub.size() * 4, cudaMemcpyHostToDevice, b->stream);
    e = cudaMemcpyAsync(b->unitEnd, ue.data(), ue.size() * 4, cudaMemcpyHostToDevice, b->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) {
    free_units(b);
    return cuda_fail(e, "batch work units");
  }
  b->nUnits = (int32_t)uv.size();
  b->unitChunk = chunk;
  return GAS_OK;
}

gas_status ensure_state(gas_batch *b, const CoreGraph &g, int32_t Q) {
  if (b->capQ >= Q && b->value) return GAS_OK;
  free_state(b);
  const size_t V = (size_t)std::max(g.nV, 1);
  const int W = Q / 32;
  cudaError_t e = cudaMalloc(&b->value, V * Q * 4);
  if (e == cudaSuccess) e = cudaMalloc(&b->outDev, V * Q * 4);
  if (e == cudaSuccess) e = cudaMalloc(&b->srcDev, kMaxBatch * 4);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaMalloc(&b->mask[k], V * W * 4);
  if (e == cudaSuccess) e = cudaMalloc(&b->seen, V * W * 4);
  const size_t cap = (size_t)gas::detail::batch_list_capacity(g.nV, g.nE);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaMalloc(&b->list[k], cap * 4);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaMalloc(&b->listC[k], cap * 4);
  if (e == cudaSuccess) e = cudaMalloc(&b->inList, V * 4);
  if (e != cudaSuccess) {
    free_state(b);
    return cuda_fail(e, "batch state allocation");
  }
  b->capQ = Q;
  return GAS_OK;
}

template <int W, int KIND>
gas_status launch_run(gas_batch *b, const CoreGraph &g, int32_t Q, int blocks, bool pairs) {
  gas::detail::BatchArgs a;
  memset(&a, 0, sizeof(a));
  a.nVertices = g.nV;
  a.nEdges = g.nE;
  a.outOffsets = g.outOff;
  a.outDests = g.outDst;
  a.weightsOut = b->weightsOut;
  for (int k = 0; k < 3; ++k) {
    a.list[k] = b->list[k];
    a.listC[k] = b->listC[k];
  }
  a.inList = b->inList;
  a.alpha = b->alpha;
  a.nQueries = Q;
  a.inSources = g.inSrc;
  a.weights = reinterpret_cast<const int32_t *>(g.edgeData);
  a.unitV = b->unitV;
  a.unitBeg = b->unitBeg;
  a.unitEnd = b->unitEnd;
  a.nUnits = b->nUnits;
  a.value = b->value;
  for (int k = 0; k < 3; ++k) a.mask[k] = b->mask[k];
  a.seen = b->seen;
  CtlView cv = ctl_view(b);
  a.cnt = cv.cnt;
  a.barrier = cv.bar;
  a.errWord = cv.err;
  a.roundsOut = cv.rounds;
  a.listCnt = cv.listCnt;
  a.maxRounds = 0;
  a.delta = KIND == gas::detail::kBatchSSSP ? b->delta : 0;
  a.thresh[0] = b->bucketMem;
  a.thresh[1] = b->bucketMem + kMaxBatch;
  for (int k = 0; k < 3; ++k)
    a.nearFlag[k] = reinterpret_cast<unsigned *>(b->bucketMem + 2 * kMaxBatch + 8 * k);
  a.pairMode = pairs ? 1 : 0;
  for (int k = 0; k < 3; ++k) a.pairs[k] = pairs ? b->pairs[k] : nullptr;
  void *args[] = {&a};
  const void *fn = pairs ? (const void *)gas::detail::batch_run_kernel<W, KIND, true>
                         : (const void *)gas::detail::batch_run_kernel<W, KIND, false>;
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(256), args, 0, b->stream);
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "batch run launch");
}

template <int W>
gas_status launch_run_kind(gas_batch *b, const CoreGraph &g, int kind, int32_t Q, int blocks,
                           bool pairs) {
  return kind == gas::detail::kBatchBFS
             ? launch_run<W, gas::detail::kBatchBFS>(b, g, Q, blocks, pairs)
             : launch_run<W, gas::detail::kBatchSSSP>(b, g, Q, blocks, pairs);
}

int grid_blocks(gas_batch *b, int kind, int W, bool pairs) {
  int per = 0;
  const void *fn = nullptr;
#define GAS_BATCH_FN(w)                                                                       \
  if (W == w)                                                                                 \
    fn = kind == gas::detail::kBatchBFS                                                       \
             ? (pairs ? (const void *)gas::detail::batch_run_kernel<w, gas::detail::kBatchBFS, true> \
                      : (const void *)gas::detail::batch_run_kernel<w, gas::detail::kBatchBFS, false>) \
             : (pairs ? (const void *)gas::detail::batch_run_kernel<w, gas::detail::kBatchSSSP, true> \
                      : (const void *)gas::detail::batch_run_kernel<w, gas::detail::kBatchSSSP, false>);
  GAS_BATCH_FN(1) GAS_BATCH_FN(2) GAS_BATCH_FN(4) GAS_BATCH_FN(8)
#undef GAS_BATCH_FN
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 256, 0);
  if (b->blocksPerSM > 0 && b->blocksPerSM < per) per = b->blocksPerSM;
  return std::max(per, 1) * std::max(b->sms, 1);
}

// The whole batch on b->stream: sources (from pinned staging), state reset,
// initial values, the persistent run, query-major results in outDev.
gas_status enqueue_batch(gas_batch *b, const CoreGraph &g, int kind, int32_t nQ, int32_t Q,
                         bool pairs) {
  const int W = Q / 32;
  const size_t V = (size_t)g.nV;
  cudaError_t e = cudaMemcpyAsync(b->srcDev, b->srcPinned, sizeof(int32_t) * nQ,
                                  cudaMemcpyHostToDevice, b->stream);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k)
    e = cudaMemsetAsync(b->mask[k], 0, V * W * 4, b->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->seen, 0, V * W * 4, b->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->inList, 0xff, V * 4, b->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->ctl, 0, kCtlBytes, b->stream);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(b->bucketMem + 2 * kMaxBatch, 0, 4 * 3 * 8, b->stream);
  if (e != cudaSuccess) return cuda_fail(e, "batch reset");
  gas::detail::batch_init_kernel<<<4 * b->sms, 256, 0, b->stream>>>(kind, g.nV, Q, b->value,
                                                                     b->bucketMem, b->delta);
  CtlView cv = ctl_view(b);
  gas::detail::batch_sources_kernel<<<(nQ + 127) / 128, 128, 0, b->stream>>>(
      kind, nQ, Q, W, g.nV, b->srcDev, b->value, b->mask[0], b->seen, g.outOff, b->inList,
      b->list[0], b->listC[0], cv.listCnt, pairs ? b->pairs[0] : nullptr);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "batch init");
  const int blocks = grid_blocks(b, kind, W, pairs);
  gas_status st;
  switch (W) {
    case 1: st = launch_run_kind<1>(b, g, kind, Q, blocks, pairs); break;
    case 2: st = launch_run_kind<2>(b, g, kind, Q, blocks, pairs); break;
    case 4: st = launch_run_kind<4>(b, g, kind, Q, blocks, pairs); break;
    default: st = launch_run_kind<8>(b, g, kind, Q, blocks, pairs); break;
  }
  if (st) return st;
  if (pairs) {  // query-major already: the first nQ rows are the results
    e = cudaMemcpyAsync(b->outDev, b->value, sizeof(int32_t) * (size_t)nQ * g.nV,
                        cudaMemcpyDeviceToDevice, b->stream);
    return e == cudaSuccess ? GAS_OK : cuda_fail(e, "batch results");
  }
  dim3 tb(32, 8), tg((g.nV + 31) / 32, (Q + 31) / 32);
  gas::detail::batch_transpose_kernel<<<tg, tb, 0, b->stream>>>(b->value, g.nV, Q, nQ, b->outDev);
  e = cudaGetLastError();
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "batch transpose");
}

// ---- personalised PageRank batches
// State of a batch with rows of QP queries: rank[2] | contrib[2] ([V][QP]
// floats each) | partial ([slots][QP]) | arrive ([hubs]) | out ([QP][V]).
size_t ppr_state_bytes(const gas_batch *b, const CoreGraph &g, int QP) {
  const size_t V = (size_t)std::max(g.nV, 1);
  return 4 * (5 * V * QP + (size_t)std::max(b->ppr.slots, 1) * QP + (size_t)std::max(b->ppr.hubs, 1)) + 256;
}

gas::detail::PprArgs ppr_args(gas_batch *b, const CoreGraph &g, int32_t nQ, int QP) {
  gas::detail::PprArgs a;
  memset(&a, 0, sizeof(a));
  a.nVertices = g.nV;
  a.nQueries = nQ;
  gas::detail::ppr_args_graph(a, g.inSrc, b->ppr.outDegree, b->ppr.lastActive, b->ppr.mem,
                              b->ppr.units, b->ppr.slots);
  const size_t V = (size_t)std::max(g.nV, 1);
  float *p = reinterpret_cast<float *>(b->pprState);
  a.rank[0] = p;
  a.rank[1] = p + V * QP;
  a.contrib[0] = p + 2 * V * QP;
  a.contrib[1] = p + 3 * V * QP;
  a.partial = p + 4 * V * QP;
  a.arrive = reinterpret_cast<unsigned *>(a.partial + (size_t)std::max(b->ppr.slots, 1) * QP);
  a.sources = b->srcDev;
  a.teleport = 0.15f;
  a.damp = 1.0f - a.teleport;  // as PPR::apply computes it, in float
  return a;
}

float *ppr_out(gas_batch *b, const CoreGraph &g, int QP) {
  const size_t V = (size_t)std::max(g.nV, 1);
  return reinterpret_cast<float *>(b->pprState) + 4 * V * QP + (size_t)std::max(b->ppr.slots, 1) * QP +
         (size_t)std::max(b->ppr.hubs, 1);
}

template <int QP>
const void *ppr_run_fn() {
  return (const void *)gas::detail::ppr_run_kernel<QP>;
}

const void *ppr_run_fn_for(int QP) {
  switch (QP) {
    case 1: return ppr_run_fn<1>();
    case 2: return ppr_run_fn<2>();
    case 4: return ppr_run_fn<4>();
    case 8: return ppr_run_fn<8>();
    case 16: return ppr_run_fn<16>();
    case 32: return ppr_run_fn<32>();
    case 64: return ppr_run_fn<64>();
    case 128: return ppr_run_fn<128>();
    default: return ppr_run_fn<256>();
  }
}

template <int QP>
void ppr_start(const gas::detail::PprArgs &a, int blocks, cudaStream_t s) {
  gas::detail::ppr_init_kernel<QP><<<blocks, 256, 0, s>>>(a);
  gas::detail::ppr_sources_kernel<QP><<<1, kMaxBatch, 0, s>>>(a);
}

void ppr_start_for(int QP, const gas::detail::PprArgs &a, int blocks, cudaStream_t s) {
  switch (QP) {
    case 1: ppr_start<1>(a, blocks, s); break;
    case 2: ppr_start<2>(a, blocks, s); break;
    case 4: ppr_start<4>(a, blocks, s); break;
    case 8: ppr_start<8>(a, blocks, s); break;
    case 16: ppr_start<16>(a, blocks, s); break;
    case 32: ppr_start<32>(a, blocks, s); break;
    case 64: ppr_start<64>(a, blocks, s); break;
    case 128: ppr_start<128>(a, blocks, s); break;
    default: ppr_start<256>(a, blocks, s); break;
  }
}

// The whole PPR batch on b->stream: sources, arrival counters, initial
// ranks, every round in one cooperative launch, query-major ranks in out.
gas_status enqueue_ppr(gas_batch *b, const CoreGraph &g, int32_t nQ, int QP) {
  cudaError_t e = cudaMemcpyAsync(b->srcDev, b->srcPinned, sizeof(int32_t) * nQ,
                                  cudaMemcpyHostToDevice, b->stream);
  gas::detail::PprArgs a = ppr_args(b, g, nQ, QP);
  if (e == cudaSuccess && b->ppr.hubs > 0)
    e = cudaMemsetAsync(a.arrive, 0, 4 * (size_t)b->ppr.hubs, b->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->ctl, 0, kCtlBytes, b->stream);
  if (e != cudaSuccess) return cuda_fail(e, "PPR batch reset");
  ppr_start_for(QP, a, 4 * b->sms, b->stream);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "PPR batch init");
  const void *fn = ppr_run_fn_for(QP);
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 256, 0);
  if (b->blocksPerSM > 0 && b->blocksPerSM < per) per = b->blocksPerSM;
  const int blocks = std::max(per, 1) * std::max(b->sms, 1);
  CtlView cv = ctl_view(b);
  int rounds = b->pprRounds;
  void *args[] = {&a, &rounds, &cv.bar, &cv.err, &cv.rounds};
  e = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(256), args, 0, b->stream);
  if (e != cudaSuccess) return cuda_fail(e, "PPR batch run launch");
  dim3 tb(32, 8), tg((g.nV + 31) / 32, (QP + 31) / 32);
  gas::detail::batch_transpose_kernel<<<tg, tb, 0, b->stream>>>(
      reinterpret_cast<const int32_t *>(a.rank[rounds & 1]), g.nV, QP, nQ,
      reinterpret_cast<int32_t *>(ppr_out(b, g, QP)));
  e = cudaGetLastError();
  return e == cudaSuccess ? GAS_OK : cuda_fail(e, "PPR batch transpose");
}

gas_status run_one_ppr(gas_batch *b, const CoreGraph &g, int32_t nQ, const int32_t *sources,
                       float *results, int32_t *rounds) {
  int QP = 1;
  while (QP < nQ) QP *= 2;
  if (!b->ppr.mem) {
    gas_status st = gas::internal::build_ppr_graph(g, b->sms, b->pprRounds, &b->ppr);
    if (st) return st;
  }
  if (!b->srcDev) {  // the sources' device copy (also part of the BFS/SSSP state)
    cudaError_t e = cudaMalloc(&b->srcDev, kMaxBatch * 4);
    if (e != cudaSuccess) return cuda_fail(e, "PPR batch sources");
    drop_graphs(b);
  }
  if (!b->pprState || b->pprQP < QP) {
    if (b->pprState) cudaFree(b->pprState);
    b->pprState = nullptr;
    b->pprQP = 0;
    drop_graphs(b);
    cudaError_t e = cudaMalloc(&b->pprState, ppr_state_bytes(b, g, QP));
    if (e != cudaSuccess) return cuda_fail(e, "PPR batch state");
    b->pprQP = QP;
  }
  memcpy(b->srcPinned, sources, sizeof(int32_t) * nQ);
  bool launched = false;
  if (b->useGraphs) {
    cudaGraphExec_t exec = nullptr;
    for (auto &c : b->graphs)
      if (c.kind == kKindPPR && c.W == QP && c.nQ == nQ && c.blocksPerSM == b->blocksPerSM &&
          c.delta == b->pprRounds)
        exec = c.exec;
    if (!exec) {
      cudaGraph_t graph = nullptr;
      if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        gas_status cst = enqueue_ppr(b, g, nQ, QP);
        cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
        if (cst == GAS_OK && ce == cudaSuccess && graph &&
            cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
          b->graphs.push_back({kKindPPR, QP, nQ, b->blocksPerSM, 0, b->pprRounds, 0, exec});
        } else {
          exec = nullptr;
          b->useGraphs = false;  // this runtime cannot capture the batch: launch directly
        }
        if (graph) cudaGraphDestroy(graph);
      } else {
        b->useGraphs = false;
      }
      cudaGetLastError();
    }
    if (exec) {
      cudaEventRecord(b->t0, b->stream);  // after any capture: device time only
      cudaError_t e = cudaGraphLaunch(exec, b->stream);
      if (e != cudaSuccess) return cuda_fail(e, "PPR batch graph launch");
      launched = true;
    }
  }
  if (!launched) {
    cudaEventRecord(b->t0, b->stream);
    gas_status st = enqueue_ppr(b, g, nQ, QP);
    if (st) return st;
  }
  cudaEventRecord(b->t1, b->stream);
  CtlView cv = ctl_view(b);
  int32_t re[2] = {0, 0};  // rounds, err
  cudaError_t e = cudaMemcpyAsync(re, cv.rounds, 8, cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess && results)
    e = cudaMemcpyAsync(results, ppr_out(b, g, QP), sizeof(float) * (size_t)nQ * g.nV,
                        cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return cuda_fail(e, "PPR batch run");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, b->t0, b->t1);
  b->lastMs += ms;
  if (re[1]) {
    cudaMemsetAsync(cv.err, 0, 4, b->stream);
    return fail(GAS_ERR_TIMEOUT, "a bounded device wait of the batched PPR run timed out");
  }
  if (rounds) *rounds = std::max(*rounds, re[0]);
  return GAS_OK;
}

gas_status run_one(gas_batch *b, const CoreGraph &g, int kind, int32_t nQ, const int32_t *sources,
                   int32_t *results, int32_t *rounds) {
  int32_t Q = 32;
  while (Q < nQ) Q *= 2;
  gas_status st = ensure_state(b, g, std::max(Q, 32));
  if (st) return st;
  const bool pairs = use_pairs(b, g, Q);
  if (pairs) {
    st = ensure_pairs(b, g, Q);
    if (st) return st;
  }
  memcpy(b->srcPinned, sources, sizeof(int32_t) * nQ);
  bool launched = false;
  if (b->useGraphs) {
    cudaGraphExec_t exec = nullptr;
    for (auto &c : b->graphs)
      if (c.kind == kind && c.W == Q / 32 && c.nQ == nQ && c.blocksPerSM == b->blocksPerSM &&
          c.chunk == b->unitChunk && c.delta == b->delta && c.pairs == (int)pairs)
        exec = c.exec;
    if (!exec) {
      cudaGraph_t graph = nullptr;
      if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        gas_status cst = enqueue_batch(b, g, kind, nQ, Q, pairs);
        cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
        if (cst == GAS_OK && ce == cudaSuccess && graph &&
            cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
          b->graphs.push_back(
              {kind, Q / 32, nQ, b->blocksPerSM, b->unitChunk, b->delta, (int)pairs, exec});
        } else {
          exec = nullptr;
          b->useGraphs = false;  // this runtime cannot capture the batch: launch directly
        }
        if (graph) cudaGraphDestroy(graph);
      } else {
        b->useGraphs = false;
      }
      cudaGetLastError();
    }
    if (exec) {
      cudaEventRecord(b->t0, b->stream);  // after any capture: device time only
      cudaError_t e = cudaGraphLaunch(exec, b->stream);
      if (e != cudaSuccess) return cuda_fail(e, "batch graph launch");
      launched = true;
    }
  }
  if (!launched) {
    cudaEventRecord(b->t0, b->stream);
    st = enqueue_batch(b, g, kind, nQ, Q, pairs);
    if (st) return st;
  }
  cudaEventRecord(b->t1, b->stream);
  CtlView cv = ctl_view(b);
  int32_t re[2] = {0, 0};  // rounds, err
  cudaError_t e = cudaMemcpyAsync(re, cv.rounds, 8, cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess && results)
    e = cudaMemcpyAsync(results, b->outDev, sizeof(int32_t) * (size_t)nQ * g.nV,
                        cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return cuda_fail(e, "batch run");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, b->t0, b->t1);
  b->lastMs += ms;
  if (re[1]) {
    cudaMemsetAsync(cv.err, 0, 4, b->stream);
    return fail(GAS_ERR_TIMEOUT, "a bounded device wait of the batched run timed out");
  }
  if (rounds) *rounds = std::max(*rounds, re[0]);
  return GAS_OK;
}

}  // namespace

namespace gas {
namespace internal {
bool batch_graph(gas_batch_s *b, BatchGraph *out) {
  if (!b || !core_graph(b->core, &out->g)) return false;
  out->weightsOut = b->weightsOut;
  out->unitV = b->unitV;
  out->unitBeg = b->unitBeg;
  out->unitEnd = b->unitEnd;
  out->nUnits = b->nUnits;
  return true;
}
}  // namespace internal
}  // namespace gas

extern "C" {

gas_status gas_batch_create(int32_t device, void *stream, gas_batch **out) {
  if (!out) return fail(GAS_ERR_INVALID, "gas_batch_create: out is NULL");
  *out = nullptr;
  gas_batch *b = new (std::nothrow) gas_batch_s();
  if (!b) return fail(GAS_ERR_OOM, "host allocation");
  gas_status st = gas_core_create(device, stream, &b->core);
  if (st) {
    delete b;
    return st;
  }
  gas::internal::core_keep_csr_perm(b->core, true);
  b->device = device;
  b->stream = (cudaStream_t)stream;
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device);
  cudaError_t e = cudaMalloc(&b->ctl, kCtlBytes);
  if (e == cudaSuccess) e = cudaMemset(b->ctl, 0, kCtlBytes);
  if (e == cudaSuccess) e = cudaMalloc(&b->bucketMem, 4 * (2 * kMaxBatch + 3 * 8));
  if (e == cudaSuccess) e = cudaMallocHost(&b->srcPinned, sizeof(int32_t) * kMaxBatch);
  if (e == cudaSuccess) e = cudaEventCreate(&b->t0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->t1);
  if (e != cudaSuccess) {
    gas_batch_destroy(b);
    return cuda_fail(e, "batch creation");
  }
  *out = b;
  return GAS_OK;
}

gas_status gas_batch_destroy(gas_batch *b) {
  if (!b) return GAS_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  free_state(b);
  free_units(b);
  gas::internal::free_ppr_graph(&b->ppr);
  if (b->weightsOut) cudaFree(b->weightsOut);
  if (b->ctl) cudaFree(b->ctl);
  if (b->bucketMem) cudaFree(b->bucketMem);
  if (b->srcPinned) cudaFreeHost(b->srcPinned);
  if (b->t0) cudaEventDestroy(b->t0);
  if (b->t1) cudaEventDestroy(b->t1);
  gas_core_destroy(b->core);
  delete b;
  return GAS_OK;
}

gas_status gas_batch_set_graph(gas_batch *b, int32_t nVertices, int32_t nEdges,
                               const int32_t *srcs, const int32_t *dsts, const int32_t *weights) {
  if (!b) return fail(GAS_ERR_INVALID, "batch is NULL");
  cudaSetDevice(b->device);
  free_state(b);
  free_units(b);
  gas::internal::free_ppr_graph(&b->ppr);
  if (b->weightsOut) cudaFree(b->weightsOut);
  b->weightsOut = nullptr;
  gas_status st = gas_core_set_graph(b->core, nVertices, nEdges, srcs, dsts, weights,
                                     weights ? 4 : 0, 4, 4);
  if (st) return st;
  CoreGraph g;
  gas::internal::core_graph(b->core, &g);
  b->maxOutDeg = 0;
  for (int32_t v = 0; v < nVertices; ++v)
    b->maxOutDeg = std::max(b->maxOutDeg, (*g.hOutOff)[(size_t)v + 1] - (*g.hOutOff)[v]);
  st = build_units(b, g, b->chunk);
  if (st == GAS_OK && weights && nEdges > 0)  // weights in CSR order for push rounds
    st = gas::internal::core_permute_csr(b->core, weights, &b->weightsOut);
  gas::internal::core_keep_csr_perm(b->core, false);  // the permutation is not needed after this
  gas::internal::core_keep_csr_perm(b->core, true);   // (kept again by the next set_graph)
  return st;
}

gas_status gas_batch_set_config(gas_batch *b, int32_t chunkEdges, int32_t blocksPerSM,
                                int32_t useGraphs) {
  if (!b) return fail(GAS_ERR_INVALID, "batch is NULL");
  if (chunkEdges < 1 || blocksPerSM < 0) return fail(GAS_ERR_INVALID, "bad batch config");
  const bool same = b->chunk == chunkEdges && b->blocksPerSM == blocksPerSM &&
                    b->useGraphs == (useGraphs != 0);
  b->chunk = chunkEdges;
  b->blocksPerSM = blocksPerSM;
  b->useGraphs = useGraphs != 0;
  if (same) return GAS_OK;  // captured batches stay valid
  drop_graphs(b);
  CoreGraph g;
  if (gas::internal::core_graph(b->core, &g)) return build_units(b, g, chunkEdges);
  return GAS_OK;
}

gas_status gas_batch_run(gas_batch *b, int32_t program, int32_t nQueries, const int32_t *sources,
                         int32_t *results, int32_t *rounds) {
  if (!b) return fail(GAS_ERR_INVALID, "batch is NULL");
  CoreGraph g;
  if (!gas::internal::core_graph(b->core, &g)) return fail(GAS_ERR_STATE, "no graph set");
  int kind;
  if (program == GAS_PROGRAM_BFS) {
    kind = gas::detail::kBatchBFS;
  } else if (program == GAS_PROGRAM_PPR) {
    kind = kKindPPR;
  } else if (program == GAS_PROGRAM_SSSP) {
    kind = gas::detail::kBatchSSSP;
    if (g.edgeBytes != 4 || !g.edgeData)
      return fail(GAS_ERR_STATE, "batched SSSP needs int32 edge weights in setGraph");
  } else {
    return fail(GAS_ERR_UNSUPPORTED, "batched runs support BFS, SSSP and PPR");
  }
  if (nQueries < 0 || (nQueries > 0 && !sources)) return fail(GAS_ERR_INVALID, "bad sources");
  for (int32_t q = 0; q < nQueries; ++q)
    if (sources[q] < 0 || sources[q] >= g.nV)
      return fail(GAS_ERR_INVALID, "source %d of query %d outside [0, %d)", sources[q], q, g.nV);
  cudaSetDevice(b->device);
  b->lastMs = 0.f;
  if (rounds) *rounds = 0;
  for (int32_t q0 = 0; q0 < nQueries; q0 += kMaxBatch) {
    const int32_t nq = std::min(kMaxBatch, nQueries - q0);
    int32_t *res = results ? results + (size_t)q0 * g.nV : nullptr;
    gas_status st = kind == kKindPPR
                        ? run_one_ppr(b, g, nq, sources + q0, reinterpret_cast<float *>(res), rounds)
                        : run_one(b, g, kind, nq, sources + q0, res, rounds);
    if (st) return st;
  }
  return GAS_OK;
}

gas_status gas_batch_set_policy(gas_batch *b, int32_t alpha) {
  if (!b) return fail(GAS_ERR_INVALID, "batch is NULL");
  if (alpha < 0) return fail(GAS_ERR_INVALID, "alpha must be >= 0");
  if (b->alpha == alpha) return GAS_OK;
  b->alpha = alpha;
  drop_graphs(b);
  return GAS_OK;
}

gas_status gas_batch_set_delta(gas_batch *b, int32_t delta) {
  if (!b) return fail(GAS_ERR_INVALID, "batch is NULL");
  if (delta < 0) return fail(GAS_ERR_INVALID, "delta must be >= 0");
  if (b->delta == delta) return GAS_OK;
  b->delta = delta;
  drop_graphs(b);
  return GAS_OK;
}

gas_status gas_batch_set_frontier(gas_batch *b, int32_t mode) {
  if (!b) return fail(GAS_ERR_INVALID, "batch is NULL");
  if (mode < -1 || mode > 1) return fail(GAS_ERR_INVALID, "frontier mode must be -1, 0 or 1");
  if (b->frontier == mode) return GAS_OK;
  b->frontier = mode;
  drop_graphs(b);
  return GAS_OK;
}

gas_status gas_batch_get_delta(gas_batch *b, int32_t *delta) {
  if (!b || !delta) return fail(GAS_ERR_INVALID, "null argument");
  *delta = b->delta;
  return GAS_OK;
}

gas_status gas_batch_last_ms(gas_batch *b, float *ms) {
  if (!b || !ms) return fail(GAS_ERR_INVALID, "null argument");
  *ms = b->lastMs;
  return GAS_OK;
}

gas_status gas_batch_autotune(gas_batch *b, int32_t program, int32_t nQueries,
                              int32_t *chunkOut, int32_t *blocksOut) {
  if (!b) return fail(GAS_ERR_INVALID, "batch is NULL");
  CoreGraph g;
  if (!gas::internal::core_graph(b->core, &g)) return fail(GAS_ERR_STATE, "no graph set");
  const int32_t nq = std::max(1, std::min(nQueries, kMaxBatch));
  std::vector<int32_t> src(nq);
  std::mt19937 rng(12345);
  for (auto &s : src) s = (int32_t)(rng() % (uint32_t)std::max(g.nV, 1));
  // time of one batch on these sources with the current settings (the first
  // run of a shape warms up and captures its graph)
  auto timed = [&](float *ms) -> gas_status {
    int32_t r = 0;
    gas_status st = gas_batch_run(b, program, nq, src.data(), nullptr, &r);
    if (st == GAS_OK) st = gas_batch_run(b, program, nq, src.data(), nullptr, &r);
    *ms = b->lastMs;
    return st;
  };
  // one coordinate at a time: try each value, keep the fastest
  auto tune = [&](const int32_t *vals, int n, gas_status (*set)(gas_batch *, int32_t),
                  int32_t keep) -> gas_status {
    float best = 1e30f;
    int32_t bv = keep;
    for (int i = 0; i < n; ++i) {
      gas_status st = set(b, vals[i]);
      float ms = 0.f;
      if (st == GAS_OK) st = timed(&ms);
      if (st) return st;
      if (ms < best) {
        best = ms;
        bv = vals[i];
      }
    }
    return set(b, bv);
  };
  gas_status st = GAS_OK;
  if (program != GAS_PROGRAM_PPR) {
    // SSSP: the bucket width (Bellman-Ford rounds or delta-stepping)
    if (program == GAS_PROGRAM_SSSP) {
      const int32_t deltas[] = {0, 128, 512, 2048};
      st = tune(deltas, 4, gas_batch_set_delta, b->delta);
      if (st) return st;
    }
    // frontier form: (vertex, query) pairs where the graph allows them,
    // else vertices with query masks; then, for masks, the push/pull switch
    if (b->maxOutDeg <= 64) {
      const int32_t forms[] = {-1, 0};
      st = tune(forms, 2, gas_batch_set_frontier, b->frontier);
      if (st) return st;
    }
    int32_t Q = 32;
    while (Q < nq) Q *= 2;
    if (!use_pairs(b, g, Q)) {
      const int32_t alphas[] = {2, 10, 50};
      st = tune(alphas, 3, gas_batch_set_policy, b->alpha);
      if (st) return st;
    }
  }
  const int32_t chunks[] = {32, 128, 512, 2048};
  const int32_t blocks[] = {0, 4, 2, 1};
  float best = 1e30f;
  int32_t bc = b->chunk, bb = b->blocksPerSM;
  const int nc = program == GAS_PROGRAM_PPR ? 1 : 4;  // PPR's units are fixed (kPprChunk)
  for (int i = 0; i < nc; ++i)
    for (int32_t k : blocks) {
      const int32_t c = program == GAS_PROGRAM_PPR ? b->chunk : chunks[i];
      st = gas_batch_set_config(b, c, k, b->useGraphs ? 1 : 0);
      float ms = 0.f;
      if (st == GAS_OK) st = timed(&ms);
      if (st) return st;
      if (ms < best) {
        best = ms;
        bc = c;
        bb = k;
      }
    }
  st = gas_batch_set_config(b, bc, bb, b->useGraphs ? 1 : 0);
  if (chunkOut) *chunkOut = bc;
  if (blocksOut) *blocksOut = bb;
  return st;
}

gas_status gas_batch_get_tuning(gas_batch *b, int32_t *chunkEdges, int32_t *blocksPerSM,
                                int32_t *alpha, int32_t *frontier, int32_t *delta) {
  if (!b) return fail(GAS_ERR_INVALID, "batch is NULL");
  if (chunkEdges) *chunkEdges = b->chunk;
  if (blocksPerSM) *blocksPerSM = b->blocksPerSM;
  if (alpha) *alpha = b->alpha;
  if (frontier) *frontier = b->frontier;
  if (delta) *delta = b->delta;
  return GAS_OK;
}

}  // extern "C"
