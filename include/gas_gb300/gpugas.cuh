// gpugas.cuh -- drop-in replacement for vertexAPI2's gpugas.h on GB300.
//
// A user vertex Program (VertexData / EdgeData / GatherResult, gatherZero,
// gatherMap, gatherReduce, apply, scatter) runs unchanged on
//
//     GASEngineGPU<Program, Int = int32_t, sortEdgesForGather = true>
//
// with the reference's methods (gpugas.h:212-772): setGraph, getResults,
// setActive, countActive, gatherApply, scatterActivate, nextIter, run.
// Include this header from a .cu file compiled for sm_103a and link
// libgas_gb300.so.  The Program's gather+apply kernel is instantiated here,
// in the caller's translation unit; graph build, frontier and scatter live
// in the library behind the C ABI of gas_gb300_core.h.
//
// Differences from the reference, all additive:
//   * the constructor takes a device and stream (the reference hard-codes
//     device 0 and the default stream, gpugas.h:171);
//   * errors are not fatal: every method records a status, read with
//     lastStatus() / lastError();
//   * runFor(maxIters) bounds run(); apply() may take the round number as a
//     third argument; a Program may declare `static constexpr bool
//     haveGather = false` to make run() skip the gather (as bfs.cu does by
//     calling gatherApply(false));
//   * getResults() returns edge data in the caller's original order (the
//     reference copies CSC-sorted data back, gpugas.h:333-336);
//   * a Program declaring `static constexpr bool scatterEdges = true` (and
//     a non-empty EdgeData) has scatter(src, dst, edge) called on every
//     out-edge of the vertices whose apply returned true, by
//     scatterActivate(true) and by run(), as the reference's CPU engine
//     does (refgas.h:171-197); otherwise scatter is not called, as in the
//     reference's GPU engine (gpugas.h:666-668).
// gatherZero must be usable in device code (constexpr or an integral
// static const).
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "../gas_gb300_core.h"
#include "detail/persistent.cuh"

namespace gas {

template <class P>
struct ProgramHaveGather {
  template <class Q>
  static constexpr bool get(decltype(Q::haveGather) *) {
    return Q::haveGather;
  }
  template <class Q>
  static constexpr bool get(...) {
    return true;
  }
  static constexpr bool value = get<P>(nullptr);
};

template <typename Program, typename Int = int32_t, bool sortEdgesForGather = true>
class EngineGPU {
  static_assert(std::is_same<Int, int32_t>::value, "vertex and edge ids are int32");

 public:
  typedef typename Program::VertexData VertexData;
  typedef typename Program::EdgeData EdgeData;
  typedef typename Program::GatherResult GatherResult;

  explicit EngineGPU(int device = 0, cudaStream_t stream = 0) {
    status_ = gas_core_create(device, (void *)stream, &core_);
  }
  ~EngineGPU() { gas_core_destroy(core_); }
  EngineGPU(const EngineGPU &) = delete;
  EngineGPU &operator=(const EngineGPU &) = delete;

  // gpugas.h:212-322
  void setGraph(Int nVertices, VertexData *vertexData, Int nEdges, EdgeData *edgeData,
                const Int *edgeListSrcs, const Int *edgeListDsts) {
    vdHost_ = vertexData;
    edHost_ = edgeData;
    const int32_t eb = kEdgeBytes;
    if (kScatterEdges && !note(gas_core_enable_edge_scatter(core_, 1))) return;
    if (!note(gas_core_set_graph(core_, nVertices, nEdges, edgeListSrcs, edgeListDsts,
                                 eb ? (const void *)edgeData : nullptr, eb,
                                 (int32_t)sizeof(VertexData), (int32_t)sizeof(GatherResult))))
      return;
    if (vertexData) note(gas_core_upload_vertex_data(core_, vertexData));
  }

  // gpugas.h:329-338.  Edge data changes only through Program::scatter
  // (scatterEdges); without it the device copy still equals what setGraph
  // read from the caller's edge array, so it is not copied back (on R-MAT-22
  // that copy is 0.5 GB, 10 ms).
  void getResults() {
    if (vdHost_ && !note(gas_core_download_vertex_data(core_, vdHost_))) return;
    if constexpr (kScatterEdges) {
      if (edHost_ && kEdgeBytes) note(gas_core_download_edge_data(core_, edHost_));
    }
  }

  // gpugas.h:342-349
  void setActive(Int vertexStart, Int vertexEnd) {
    note(gas_core_set_active(core_, vertexStart, vertexEnd));
  }

  // gpugas.h:353-356
  Int countActive() {
    int32_t n = 0;
    if (!note(gas_core_count_active(core_, &n))) return 0;
    return n;
  }

  // gpugas.h:421-513
  void gatherApply(bool haveGather = true) {
    note(gas_core_gather_apply(core_, haveGather ? 1 : 0, &launch, this));
  }

  // gpugas.h:669-751.  Program::scatter runs only for Programs that opt in
  // (scatterEdges), after the activation.
  void scatterActivate(bool haveScatter = true) {
    if (!note(gas_core_scatter_activate(core_))) return;
    if constexpr (kScatterEdges) {
      if (haveScatter) note(gas_core_edge_scatter(core_, &launchEdgeScatter, this));
    }
  }

  // gpugas.h:754-758
  Int nextIter() {
    if (!note(gas_core_next_iter(core_))) return 0;
    return countActive();
  }

  // gpugas.h:764-772
  void run() { runFor(0); }

  // run() bounded to maxIters rounds (0 = until no vertex is active);
  // returns the number of rounds executed.
  int32_t runFor(int32_t maxIters) {
    int32_t it = 0;
    if (kScatterEdges && persistent_) {
      const gas_status st =
          gas_core_run_persistent(core_, maxIters, ProgramHaveGather<Program>::value ? 1 : 0,
                                  &launchRun, &launch, this, &it);
      if (st != GAS_ERR_UNSUPPORTED) {
        note(st);
        return it;
      }
    }
    if (kScatterEdges) {  // the rounds one call at a time (refgas.h:216-224)
      while ((maxIters <= 0 || it < maxIters) && countActive() > 0 && status_ == GAS_OK) {
        gatherApply(ProgramHaveGather<Program>::value);
        scatterActivate(true);
        nextIter();
        ++it;
      }
      return it;
    }
    note(gas_core_run_persistent(core_, maxIters, ProgramHaveGather<Program>::value ? 1 : 0,
                                 persistent_ ? &launchRun : nullptr, &launch, this, &it));
    return it;
  }

  // run() as one persistent cooperative kernel (default) or one launch per
  // phase and round.
  void setPersistent(bool on) { persistent_ = on; }

  // CTAs per SM of the persistent run kernel (0 = the default: 2 on graphs
  // whose degrees are all <= 8 -- 1 for apply-only runs --, else 4; at most
  // what fits).
  void setRunBlocksPerSM(int n) {
    runBlocksPerSM_ = n > 0 ? n : 0;
    runGrid_ = 0;
    runGridFused_ = 0;
    runGridFusedApply_ = 0;
  }

  // Round number handed to apply(v, g, round) by the stepwise API.
  void setIteration(int32_t it) { note(gas_core_set_iteration(core_, it)); }

  gas_status lastStatus() const { return status_; }
  const char *lastError() const { return gas_last_error(); }
  gas_core *core() { return core_; }

 private:
  static constexpr int32_t kEdgeBytes =
      std::is_empty<EdgeData>::value ? 0 : (int32_t)sizeof(EdgeData);
  static constexpr bool kScatterEdges =
      detail::ProgramScatterEdges<Program>::value && kEdgeBytes > 0;

  bool note(gas_status s) {
    status_ = s;
    return s == GAS_OK;
  }

  static gas_status launch(void *user, const gas_gather_args *a, void *stream) {
    EngineGPU *self = static_cast<EngineGPU *>(user);
    if (self->grid_ == 0) {
      int dev = 0, sms = 0, per = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per, detail::gather_apply_kernel<Program>, detail::kGNT, 0);
      self->grid_ = (per > 0 ? per : 1) * (sms > 0 ? sms : 1);
    }
    detail::gather_apply_kernel<Program>
        <<<self->grid_, detail::kGNT, 0, (cudaStream_t)stream>>>(*a);
    return cudaGetLastError() == cudaSuccess ? GAS_OK : GAS_ERR_CUDA;
  }

  // CTAs per SM of the persistent kernel.  Fused-round graphs (small
  // degrees, latency-bound rounds) launch 1 CTA per SM: the grid barrier and
  // the wait for the slowest block are cheaper with fewer blocks, and a
  // block's bitmap words still fit one pass (lattice SSSP 16.65 -> 16.41 ms
  // per run against 2 CTAs per SM).  Their instantiation is compiled for 1
  // CTA per SM, so it keeps its state in registers (about 250, where a
  // 128-register budget spilled about 900 bytes a thread to local memory:
  // 15.68 -> 14.64 ms).  Other graphs run 4 with 64 registers: more warps in
  // flight for the pull passes, whose dependent gathers are L2-latency bound.
  static constexpr int kFusedBlocksPerSM = 1;  // the fused instantiation's register budget
  static constexpr int kRunBlocksPerSM = 4;
  static constexpr int kFusedGatherBlocksPerSM = 1;
  // Fused rounds of an apply-only run (BFS: no gather) also use 1 CTA per SM.
  static constexpr int kFusedApplyBlocksPerSM = 1;
  // A run that starts with every vertex active runs its leading dense rounds
  // in run_dense_kernel (40 registers, 6 CTAs per SM), then resumes here.
  static constexpr int kDenseBlocksPerSM = 6;

  static gas_status launchRun(void *user, const gas_run_args *ra, void *stream) {
    EngineGPU *self = static_cast<EngineGPU *>(user);
    if (ra->allActive && ra->resume && !ra->denseFirst && self->runBlocksPerSM_ == 0) {
      const void *dk = (const void *)detail::run_dense_kernel<Program, kDenseBlocksPerSM>;
      if (self->denseGrid_ == 0) {
        int dev = 0, sms = 0, per = 0, coop = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, dk, detail::kGNT, 0);
        if (per > kDenseBlocksPerSM) per = kDenseBlocksPerSM;
        self->denseGrid_ = (coop && per > 0 && sms > 0) ? per * sms : -1;
      }
      if (self->denseGrid_ > 0) {
        void *dargs[] = {const_cast<gas_run_args *>(ra)};
        cudaError_t e = cudaLaunchCooperativeKernel(dk, dim3(self->denseGrid_), dim3(detail::kGNT), dargs, 0,
                                                    (cudaStream_t)stream);
        if (e == cudaSuccess) {
          gas_run_args rest = *ra;
          rest.denseFirst = 1;
          const gas_status st = launchRun(user, &rest, stream);
          // rounds already ran: a per-phase fallback would repeat them
          return st == GAS_ERR_UNSUPPORTED ? GAS_ERR_CUDA : st;
        }
        cudaGetLastError();
        self->denseGrid_ = -1;  // not co-resident: the main kernel runs every round
      }
    }
    const bool applyOnly = ra->fused && !ra->g.haveGather;
    int &grid = !ra->fused ? self->runGrid_ : (applyOnly ? self->runGridFusedApply_ : self->runGridFused_);
    const void *kern = ra->fused ? (const void *)detail::run_persistent_kernel<Program, kFusedBlocksPerSM>
                                 : (const void *)detail::run_persistent_kernel<Program, kRunBlocksPerSM>;
    if (grid == 0) {
      int dev = 0, sms = 0, per = 0, coop = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, detail::kGNT, 0);
      const int want = self->runBlocksPerSM_ > 0
                           ? self->runBlocksPerSM_
                           : (!ra->fused ? kRunBlocksPerSM
                                         : applyOnly ? kFusedApplyBlocksPerSM : kFusedGatherBlocksPerSM);
      if (want > 0 && want < per) per = want;
      grid = (coop && per > 0 && sms > 0) ? per * sms : -1;
    }
    if (grid < 0) return GAS_ERR_UNSUPPORTED;
    void *args[] = {const_cast<gas_run_args *>(ra)};
    cudaError_t e = cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(detail::kGNT), args,
                                                0, (cudaStream_t)stream);
    if (e == cudaErrorCooperativeLaunchTooLarge) {
      cudaGetLastError();
      return GAS_ERR_UNSUPPORTED;
    }
    return e == cudaSuccess ? GAS_OK : GAS_ERR_CUDA;
  }

  static gas_status launchEdgeScatter(void *user, const gas_edge_scatter_args *a, void *stream) {
    EngineGPU *self = static_cast<EngineGPU *>(user);
    if (self->scatterGrid_ == 0) {
      int dev = 0, sms = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      self->scatterGrid_ = 4 * (sms > 0 ? sms : 1);
    }
    if constexpr (kScatterEdges)
      detail::edge_scatter_kernel<Program><<<self->scatterGrid_, 256, 0, (cudaStream_t)stream>>>(*a);
    return cudaGetLastError() == cudaSuccess ? GAS_OK : GAS_ERR_CUDA;
  }

  gas_core *core_ = nullptr;
  gas_status status_ = GAS_OK;
  int scatterGrid_ = 0;
  bool persistent_ = true;
  int runGrid_ = 0;
  int runGridFused_ = 0;
  int runGridFusedApply_ = 0;
  int denseGrid_ = 0;
  int runBlocksPerSM_ = 0;
  VertexData *vdHost_ = nullptr;
  EdgeData *edHost_ = nullptr;
  int grid_ = 0;
};

}  // namespace gas

#ifndef GAS_GB300_NO_GLOBAL_NAME
// Same name and template parameters as gpugas.h:74-77.
template <typename Program, typename Int = int32_t, bool sortEdgesForGather = true>
using GASEngineGPU = gas::EngineGPU<Program, Int, sortEdgesForGather>;
#endif
