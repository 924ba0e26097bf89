// Built-in engine of gas::programs::SSSP (GAS_PROGRAM_SSSP).
#include "gas_builtin_engine.h"
#include "gas_gb300/programs.cuh"

namespace gas {
namespace internal {

EngineBase *new_engine_sssp(int device, cudaStream_t stream) {
  return new (std::nothrow) BuiltinEngine<programs::SSSP>(device, stream);
}

}  // namespace internal
}  // namespace gas
