// Built-in engine of gas::programs::CC (GAS_PROGRAM_CC).
#include "gas_builtin_engine.h"
#include "gas_gb300/programs.cuh"

namespace gas {
namespace internal {

EngineBase *new_engine_cc(int device, cudaStream_t stream) {
  return new (std::nothrow) BuiltinEngine<programs::CC>(device, stream);
}

}  // namespace internal
}  // namespace gas
