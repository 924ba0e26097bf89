// Built-in engine of gas::programs::PPR (GAS_PROGRAM_PPR).
#include "gas_builtin_engine.h"
#include "gas_gb300/programs.cuh"

namespace gas {
namespace internal {

EngineBase *new_engine_ppr(int device, cudaStream_t stream) {
  return new (std::nothrow) BuiltinEngine<programs::PPR>(device, stream);
}

}  // namespace internal
}  // namespace gas
