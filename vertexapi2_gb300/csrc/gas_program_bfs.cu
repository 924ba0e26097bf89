// Built-in engine of gas::programs::BFS (GAS_PROGRAM_BFS).
#include "gas_builtin_engine.h"
#include "gas_gb300/programs.cuh"

namespace gas {
namespace internal {

EngineBase *new_engine_bfs(int device, cudaStream_t stream) {
  return new (std::nothrow) BuiltinEngine<programs::BFS>(device, stream);
}

}  // namespace internal
}  // namespace gas
