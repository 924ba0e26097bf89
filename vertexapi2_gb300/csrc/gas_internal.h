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

// Stable counting sort of an edge list by `key` on the host: off[V+1],
// adj[E] and optionally perm[p] = edge index placed at position p.
void build_adjacency(int32_t nV, int32_t nE, const int32_t *key, const int32_t *other,
                     std::vector<int32_t> &off, std::vector<int32_t> &adj,
                     std::vector<int32_t> *perm);

// The same on the device (gas_graph_build.cu): stable radix sort of
// (key, edge index); dOff[V+1], dAdj[E], optional dPerm[E].  Device arrays,
// stream-ordered on `s`.
gas_status device_build_adjacency(cudaStream_t s, int32_t nV, int32_t nE, const int32_t *dKey,
                                  const int32_t *dOther, int32_t *dOff, int32_t *dAdj,
                                  uint32_t *dPerm);
// Index of the first edge with an id outside [0, nV), or -1 (waits).
gas_status device_first_bad_edge(cudaStream_t s, int32_t nV, int32_t nE, const int32_t *dSrcs,
                                 const int32_t *dDsts, long long *firstBad);
// out[q] = CSC position of the edge at CSR position q.
gas_status device_csr_to_csc(cudaStream_t s, int32_t n, const uint32_t *cscPerm,
                             const uint32_t *csrPerm, int32_t *out);
// out[p] = in[perm[p]] / out[perm[p]] = in[p] for n elements of `bytes`.
gas_status device_gather_bytes(cudaStream_t s, const void *dIn, const uint32_t *dPerm, int32_t n,
                               int32_t bytes, void *dOut);
gas_status device_scatter_bytes(cudaStream_t s, const void *dIn, const uint32_t *dPerm, int32_t n,
                                int32_t bytes, void *dOut);

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
// Keep the CSR permutation at the next set_graph (false also frees a kept
// one), and gather host values (one int32 per edge, edge-list order) into a
// new device array in CSR order (the caller frees it).
void core_keep_csr_perm(struct gas_core_s *c, bool keep);
gas_status core_permute_csr(struct gas_core_s *c, const int32_t *hostVals, int32_t **devOut);

// A gas_batch's graph with its batched-run extras: out-edge weights in CSR
// order and the pull work units (a vertex's in-edges, hubs in chunks).
struct BatchGraph {
  CoreGraph g;
  const int32_t *weightsOut;
  const int32_t *unitV, *unitBeg, *unitEnd;
  int32_t nUnits;
};
bool batch_graph(struct gas_batch_s *b, BatchGraph *out);

// Personalised PageRank structures of a graph (gas_serve.cu): out-degrees,
// the pull work units (a vertex's in-edges, hubs cut into
// gas::detail::kPprChunk-edge chunks with partial-sum slots) longest first,
// and lastActive[v], the last of `rounds` rounds in which v is active.
struct PprGraph {
  int32_t *outDegree = nullptr;  // [V]
  uint8_t *lastActive = nullptr; // [V]
  int32_t *mem = nullptr;        // unitV | unitBeg | unitLen | unitSlot | slotFirst | slotCount | slotHub
  int32_t units = 0, slots = 0, hubs = 0;
};
gas_status build_ppr_graph(const CoreGraph &g, int sms, int rounds, PprGraph *out);
void free_ppr_graph(PprGraph *p);

}  // namespace internal
}  // namespace gas
