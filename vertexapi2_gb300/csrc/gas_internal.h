// Internal helpers shared by the translation units of libgas_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "gas_gb300.h"

namespace gas {
namespace internal {

// Records a one-line message for gas_last_error() and returns `code`.
gas_status fail(gas_status code, const char *fmt, ...);
// Maps a CUDA error to GAS_ERR_OOM / GAS_ERR_CUDA with a message.
gas_status cuda_fail(cudaError_t e, const char *what);

// Stable counting sort of an edge list by `key`: off[V+1], adj[E] and
// optionally perm[p] = edge index placed at position p.
void build_adjacency(int32_t nV, int32_t nE, const int32_t *key, const int32_t *other,
                     std::vector<int32_t> &off, std::vector<int32_t> &adj,
                     std::vector<int32_t> *perm);

// Device graph of a gas_core (CSC, CSR, edge data in CSC order), for the
// other engines of the library that share its graph build.
struct CoreGraph {
  int device;
  cudaStream_t stream;
  int32_t nV, nE;
  const int32_t *inOff, *inSrc, *outOff, *outDst;
  const void *edgeData;
  int32_t edgeBytes;
  const std::vector<int32_t> *hInOff;
  const std::vector<int32_t> *hOutOff;
};
bool core_graph(struct gas_core_s *c, CoreGraph *out);

// A gas_batch's graph with its batched-run extras: out-edge weights in CSR
// order and the pull work units (a vertex's in-edges, hubs in chunks).
struct BatchGraph {
  CoreGraph g;
  const int32_t *weightsOut;
  const int32_t *unitV, *unitBeg, *unitEnd;
  int32_t nUnits;
};
bool batch_graph(struct gas_batch_s *b, BatchGraph *out);

}  // namespace internal
}  // namespace gas
