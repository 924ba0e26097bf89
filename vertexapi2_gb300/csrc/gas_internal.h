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

}  // namespace internal
}  // namespace gas
