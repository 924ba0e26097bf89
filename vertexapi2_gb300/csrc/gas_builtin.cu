// Engine layer of the C ABI (gas_gb300.h): gas_engine_* for the built-in
// vertex programs.  Each program id maps to gas::EngineGPU<Program> (the
// same template a C++ user instantiates from gas_gb300/gpugas.cuh), so the
// FFI path and the C++ path run identical kernels; the engines are made in
// gas_program_*.cu.
#include "gas_builtin_engine.h"
#include "gas_internal.h"

using gas::internal::EngineBase;
using gas::internal::fail;

struct gas_engine_s {
  int32_t program;
  EngineBase *impl;
};

extern "C" {

gas_status gas_engine_create(int32_t program, int32_t device, void *stream, gas_engine **out) {
  if (!out) return fail(GAS_ERR_INVALID, "gas_engine_create: out is NULL");
  *out = nullptr;
  EngineBase *impl = nullptr;
  cudaStream_t s = (cudaStream_t)stream;
  switch (program) {
    case GAS_PROGRAM_BFS: impl = gas::internal::new_engine_bfs(device, s); break;
    case GAS_PROGRAM_SSSP: impl = gas::internal::new_engine_sssp(device, s); break;
    case GAS_PROGRAM_CC: impl = gas::internal::new_engine_cc(device, s); break;
    case GAS_PROGRAM_PAGERANK: impl = gas::internal::new_engine_pagerank(device, s); break;
    case GAS_PROGRAM_PPR: impl = gas::internal::new_engine_ppr(device, s); break;
    default: return fail(GAS_ERR_INVALID, "unknown program id %d", program);
  }
  if (!impl) return fail(GAS_ERR_OOM, "host allocation");
  gas_status st = impl->status();
  if (st != GAS_OK || !impl->core()) {
    delete impl;
    return st ? st : fail(GAS_ERR_CUDA, "engine creation failed");
  }
  gas_engine *e = new (std::nothrow) gas_engine_s{program, impl};
  if (!e) {
    delete impl;
    return fail(GAS_ERR_OOM, "host allocation");
  }
  *out = e;
  return GAS_OK;
}

gas_status gas_engine_destroy(gas_engine *e) {
  if (!e) return GAS_OK;
  delete e->impl;
  delete e;
  return GAS_OK;
}

#define GAS_ENGINE_CHECK(e)                                                   \
  if (!(e) || !(e)->impl) return fail(GAS_ERR_INVALID, "engine is NULL");

gas_status gas_engine_set_graph(gas_engine *e, int32_t nVertices, void *vertexData,
                                int32_t nEdges, void *edgeData, const int32_t *srcs,
                                const int32_t *dsts) {
  GAS_ENGINE_CHECK(e);
  return e->impl->setGraph(nVertices, vertexData, nEdges, edgeData, srcs, dsts);
}

gas_status gas_engine_get_results(gas_engine *e) {
  GAS_ENGINE_CHECK(e);
  return e->impl->getResults();
}

gas_status gas_engine_set_vertex_data(gas_engine *e, const void *host) {
  GAS_ENGINE_CHECK(e);
  return gas_core_upload_vertex_data(e->impl->core(), host);
}

gas_status gas_engine_set_active(gas_engine *e, int32_t vertexStart, int32_t vertexEnd) {
  GAS_ENGINE_CHECK(e);
  return e->impl->setActive(vertexStart, vertexEnd);
}

gas_status gas_engine_count_active(gas_engine *e, int32_t *nActive) {
  GAS_ENGINE_CHECK(e);
  if (!nActive) return fail(GAS_ERR_INVALID, "nActive is NULL");
  return gas_core_count_active(e->impl->core(), nActive);
}

gas_status gas_engine_gather_apply(gas_engine *e, int32_t haveGather) {
  GAS_ENGINE_CHECK(e);
  return e->impl->gatherApply(haveGather != 0);
}

gas_status gas_engine_scatter_activate(gas_engine *e, int32_t haveScatter) {
  GAS_ENGINE_CHECK(e);
  return e->impl->scatterActivate(haveScatter != 0);
}

gas_status gas_engine_next_iter(gas_engine *e, int32_t *nActive) {
  GAS_ENGINE_CHECK(e);
  gas_status st = gas_core_next_iter(e->impl->core());
  if (st || !nActive) return st;
  return gas_core_count_active(e->impl->core(), nActive);
}

gas_status gas_engine_run(gas_engine *e, int32_t maxIters, int32_t *iterations) {
  GAS_ENGINE_CHECK(e);
  return e->impl->run(maxIters, iterations);
}

gas_status gas_engine_set_iteration(gas_engine *e, int32_t iteration) {
  GAS_ENGINE_CHECK(e);
  return gas_core_set_iteration(e->impl->core(), iteration);
}

gas_status gas_engine_round_stats(gas_engine *e, int32_t capacity, int64_t *active,
                                  int64_t *gathered, int64_t *ret, int64_t *scattered,
                                  int32_t *rounds) {
  GAS_ENGINE_CHECK(e);
  return gas_core_round_stats(e->impl->core(), capacity, active, gathered, ret, scattered,
                              rounds);
}

gas_status gas_engine_save_vertex_data(gas_engine *e) {
  GAS_ENGINE_CHECK(e);
  return gas_core_save_vertex_data(e->impl->core());
}

gas_status gas_engine_restore_vertex_data(gas_engine *e) {
  GAS_ENGINE_CHECK(e);
  return gas_core_restore_vertex_data(e->impl->core());
}

gas_status gas_engine_set_profiling(gas_engine *e, int32_t enabled) {
  GAS_ENGINE_CHECK(e);
  return gas_core_set_profiling(e->impl->core(), enabled);
}

gas_status gas_engine_kernel_times(gas_engine *e, float *gatherMs, float *scatterMs,
                                   int32_t *gatherLaunches, int32_t *scatterLaunches) {
  GAS_ENGINE_CHECK(e);
  return gas_core_kernel_times(e->impl->core(), gatherMs, scatterMs, gatherLaunches,
                               scatterLaunches);
}

gas_status gas_engine_set_launch_config(gas_engine *e, int32_t persistent,
                                        int32_t runBlocksPerSM) {
  GAS_ENGINE_CHECK(e);
  if (runBlocksPerSM < 0) return fail(GAS_ERR_INVALID, "runBlocksPerSM must be >= 0");
  e->impl->setLaunch(persistent != 0, runBlocksPerSM);
  return GAS_OK;
}

gas_status gas_engine_set_fused_rounds(gas_engine *e, int32_t on) {
  if (!e) return fail(GAS_ERR_INVALID, "engine is NULL");
  return gas_core_set_fused_rounds(e->impl->core(), on);
}

gas_status gas_engine_set_dense_policy(gas_engine *e, int32_t alpha) {
  GAS_ENGINE_CHECK(e);
  return gas_core_set_dense_policy(e->impl->core(), alpha);
}

gas_status gas_engine_last_run_ms(gas_engine *e, float *ms) {
  GAS_ENGINE_CHECK(e);
  return gas_core_last_run_ms(e->impl->core(), ms);
}

}  // extern "C"
