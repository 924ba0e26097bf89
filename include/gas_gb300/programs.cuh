// Built-in vertex programs of the GB300 GAS engine.
//
// The four example programs of vertexAPI2, restated member for member with
// the reference's constants (bfs.cu:31-78, sssp.cu:25-64,
// connected_component.cu:25-63, pagerank.cu:27-73), plus personalised
// PageRank written against the same Program contract.  Differences from the
// reference sources:
//   * gatherZero is constexpr (in-class float constants are an old GCC
//     extension in pagerank.cu:29-30,43);
//   * BFS takes the iteration number as a third apply() argument instead of
//     reading the driver's __constant__ g_iterationCountGPU (bfs.cu:28,63);
//     the engine passes the round number (or gas_engine_set_iteration's);
//   * BFS declares haveGather = false, which is how the reference driver
//     runs it (gatherApply(false), bfs.cu:104).
#pragma once

#include <climits>
#include <cmath>

namespace gas {
namespace programs {

struct BFS {
  struct VertexData {
    int depth;
  };
  struct EdgeData {};
  typedef int GatherResult;
  static constexpr int gatherZero = INT_MAX - 1;
  static constexpr bool haveGather = false;

  __host__ __device__ static int gatherReduce(const int &, const int &) { return 0; }
  __host__ __device__ static int gatherMap(const VertexData *, const VertexData *,
                                           const EdgeData *) {
    return 0;
  }
  __host__ __device__ static bool apply(VertexData *vert, int, int iteration) {
    if (vert->depth == -1) {
      vert->depth = iteration;
      return true;
    }
    return false;
  }
  __host__ __device__ static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

struct SSSP {
  typedef int VertexData;
  typedef int EdgeData;
  typedef int GatherResult;
  static constexpr int maxLength = 100000;
  static constexpr int gatherZero = INT_MAX - maxLength;

  __host__ __device__ static int gatherReduce(const int &left, const int &right) {
    return left < right ? left : right;
  }
  __host__ __device__ static int gatherMap(const VertexData *, const VertexData *srcDist,
                                           const EdgeData *edgeLen) {
    return *srcDist + *edgeLen;
  }
  __host__ __device__ static bool apply(VertexData *curDist, GatherResult dist) {
    bool changed = dist < *curDist;
    *curDist = dist < *curDist ? dist : *curDist;
    return changed;
  }
  __host__ __device__ static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

struct CC {
  typedef int VertexData;
  struct EdgeData {};
  typedef int GatherResult;
  static constexpr int gatherZero = INT_MAX;

  __host__ __device__ static int gatherReduce(const int &left, const int &right) {
    return left < right ? left : right;
  }
  __host__ __device__ static int gatherMap(const VertexData *, const VertexData *srcLabel,
                                           const EdgeData *) {
    return *srcLabel;
  }
  __host__ __device__ static bool apply(VertexData *curLabel, GatherResult label) {
    bool changed = label < *curLabel;
    *curLabel = label < *curLabel ? label : *curLabel;
    return changed;
  }
  __host__ __device__ static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

struct PageRank {
  static constexpr float pageConst = 0.15f;
  static constexpr float tol = 0.01f;
  struct VertexData {
    float rank;
    int numOutEdges;
  };
  struct EdgeData {};
  typedef float GatherResult;
  static constexpr float gatherZero = 0.0f;

  __host__ __device__ static float gatherMap(const VertexData *, const VertexData *src,
                                             const EdgeData *) {
    return src->rank / src->numOutEdges;
  }
  __host__ __device__ static float gatherReduce(const float &left, const float &right) {
    return left + right;
  }
  __host__ __device__ static bool apply(VertexData *vertexData, const float &gatherResult) {
    float newRank = pageConst + (1.0f - pageConst) * gatherResult;
    bool ret = fabsf(newRank - vertexData->rank) >= tol;
    vertexData->rank = newRank;
    return ret;
  }
  __host__ __device__ static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

// Personalised PageRank: rank_v <- teleport_v + (1-alpha) * sum rank_u/outdeg_u,
// teleport_v = alpha for the source, 0 elsewhere; every vertex stays active.
struct PPR {
  static constexpr float alpha = 0.15f;
  struct VertexData {
    float rank;
    int numOutEdges;
    float teleport;
  };
  struct EdgeData {};
  typedef float GatherResult;
  static constexpr float gatherZero = 0.0f;

  __host__ __device__ static float gatherMap(const VertexData *, const VertexData *src,
                                             const EdgeData *) {
    return src->rank / src->numOutEdges;
  }
  __host__ __device__ static float gatherReduce(const float &left, const float &right) {
    return left + right;
  }
  __host__ __device__ static bool apply(VertexData *v, const float &g) {
    v->rank = v->teleport + (1.0f - alpha) * g;
    return true;
  }
  __host__ __device__ static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

}  // namespace programs
}  // namespace gas
