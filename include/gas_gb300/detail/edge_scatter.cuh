// Program::scatter over the out-edges of the vertices whose apply returned
// true (the reference's CPU engine, refgas.h:171-197; its GPU engine never
// calls it, gpugas.h:666-668).  A Program opts in with
//
//     static constexpr bool scatterEdges = true;
//
// scatter(src, dst, edge) may only write its own edge (the VertexData
// pointers are const), so the calls of one round are independent and run
// in any order: a warp per vertex, lanes over its out-edges.  Edge data is
// kept in CSC order; csr2csc maps each CSR edge to it.
#pragma once

#include "../../gas_gb300_core.h"
#include "primitives.cuh"

namespace gas {
namespace detail {

template <class P>
struct ProgramScatterEdges {
  template <class Q>
  static constexpr bool get(decltype(Q::scatterEdges) *) {
    return Q::scatterEdges;
  }
  template <class Q>
  static constexpr bool get(...) {
    return false;
  }
  static constexpr bool value = get<P>(nullptr);
};

// The grid's warps over n listed vertices.
template <class P>
__device__ __forceinline__ void edge_scatter_vertices(const int32_t *vid, long long n,
                                                      const int32_t *outOffsets,
                                                      const int32_t *outDests,
                                                      const int32_t *csr2csc, const void *vdata,
                                                      void *edata) {
  typedef typename P::VertexData VD;
  typedef typename P::EdgeData ED;
  const VD *vd = reinterpret_cast<const VD *>(vdata);
  ED *ed = reinterpret_cast<ED *>(edata);
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  for (long long i = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; i < n;
       i += warps) {
    const int u = vid[i];
    const int end = outOffsets[u + 1];
    for (int e = outOffsets[u] + lane; e < end; e += 32)
      P::scatter(vd + u, vd + outDests[e], ed + csr2csc[e]);
  }
}

template <class P>
__global__ void __launch_bounds__(256) edge_scatter_kernel(const gas_edge_scatter_args a) {
  const long long n = (long long)(*a.count >> 32);
  edge_scatter_vertices<P>(a.vid, n, a.outOffsets, a.outDests, a.csr2csc, a.vertexData,
                           a.edgeData);
}

}  // namespace detail
}  // namespace gas
