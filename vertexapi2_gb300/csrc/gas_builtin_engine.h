// Program-independent face of the built-in engines (gas_engine_* in
// gas_builtin.cu) and the per-program factories, one translation unit per
// program (gas_program_*.cu) so that the kernels of the five programs
// compile in parallel.
#pragma once

#include <new>

#include "gas_gb300.h"
#include "gas_gb300/gpugas.cuh"

namespace gas {
namespace internal {

struct EngineBase {
  virtual ~EngineBase() {}
  virtual gas_status status() const = 0;
  virtual gas_core *core() = 0;
  virtual gas_status setGraph(int32_t nV, void *vd, int32_t nE, void *ed, const int32_t *s,
                              const int32_t *d) = 0;
  virtual gas_status getResults() = 0;
  virtual gas_status setActive(int32_t a, int32_t b) = 0;
  virtual gas_status gatherApply(bool g) = 0;
  virtual gas_status scatterActivate(bool s) = 0;
  virtual gas_status run(int32_t maxIters, int32_t *iters) = 0;
  virtual void setLaunch(bool persistent, int blocksPerSM) = 0;
};

template <class P>
struct BuiltinEngine final : EngineBase {
  gas::EngineGPU<P> eng;
  BuiltinEngine(int device, cudaStream_t stream) : eng(device, stream) {}
  gas_status status() const override { return eng.lastStatus(); }
  gas_core *core() override { return eng.core(); }
  gas_status setGraph(int32_t nV, void *vd, int32_t nE, void *ed, const int32_t *s,
                      const int32_t *d) override {
    eng.setGraph(nV, reinterpret_cast<typename P::VertexData *>(vd), nE,
                 reinterpret_cast<typename P::EdgeData *>(ed), s, d);
    return eng.lastStatus();
  }
  gas_status getResults() override {
    eng.getResults();
    return eng.lastStatus();
  }
  gas_status setActive(int32_t a, int32_t b) override {
    eng.setActive(a, b);
    return eng.lastStatus();
  }
  gas_status gatherApply(bool g) override {
    eng.gatherApply(g);
    return eng.lastStatus();
  }
  gas_status scatterActivate(bool s) override {
    eng.scatterActivate(s);
    return eng.lastStatus();
  }
  gas_status run(int32_t maxIters, int32_t *iters) override {
    int32_t it = eng.runFor(maxIters);
    if (iters) *iters = it;
    return eng.lastStatus();
  }
  void setLaunch(bool persistent, int blocksPerSM) override {
    eng.setPersistent(persistent);
    eng.setRunBlocksPerSM(blocksPerSM);
  }
};

// new-allocated engine of one built-in program (nullptr when out of memory)
EngineBase *new_engine_bfs(int device, cudaStream_t stream);
EngineBase *new_engine_sssp(int device, cudaStream_t stream);
EngineBase *new_engine_cc(int device, cudaStream_t stream);
EngineBase *new_engine_pagerank(int device, cudaStream_t stream);
EngineBase *new_engine_ppr(int device, cudaStream_t stream);

}  // namespace internal
}  // namespace gas
