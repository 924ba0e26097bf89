// Built-in engine of gas::programs::PageRank (GAS_PROGRAM_PAGERANK).
#include "gas_builtin_engine.h"
#include "gas_gb300/programs.cuh"

namespace gas {
namespace internal {

EngineBase *new_engine_pagerank(int device, cudaStream_t stream) {
  return new (std::nothrow) BuiltinEngine<programs::PageRank>(device, stream);
}

}  // namespace internal
}  // namespace gas
