// The reference's own example vertex programs, driven through the C++
// engine template (gas_gb300/gpugas.cuh) the way the reference's example
// drivers drive them -- the drop-in check of the Program contract.
//
// BFS restates bfs.cu:24-78 member for member: a two-argument apply that
// reads the round from a file-scope `__device__ __constant__` variable,
// which the host driver loop updates with cudaMemcpyToSymbol between rounds
// (bfs.cu:81-112: setActive(source), countActive / gatherApply(false) /
// scatterActivate(false) / nextIter, no gather).
//
// PageRank restates pagerank.cu:27-73 member for member with one change
// the engine's documentation asks for: the in-class `static const float`
// constants (pagerank.cu:29-30, 43), which C++11 and later reject, become
// `static constexpr float`.  The driver is pagerank.cu:76-101: ranks
// initialised to pageConst, every vertex active, run() until no vertex is
// active.
//
//   ref_programs in.bin out.bin
//     in:  int32 nV, nE, source, which (0 = BFS, 1 = PageRank), then
//          srcs[nE], dsts[nE]
//     out: int32 status, rounds (BFS; 0 for PageRank, whose driver calls
//          run()), then depth[nV] (int32) or rank[nV] (float)
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <vector>

#include <gas_gb300/gpugas.cuh>

// bfs.cu:24-28
int g_iterationCount;
__device__ __constant__ int g_iterationCountGPU;

// bfs.cu:31-78
struct BFS {
  struct VertexData {
    int depth;
  };

  struct EdgeData {};  // nothing

  typedef int GatherResult;
  static const int gatherZero = INT_MAX - 1;

  __host__ __device__ static int gatherReduce(const int &left, const int &right) {
    return 0;  // do nothing
  }

  __host__ __device__ static int gatherMap(const VertexData *dst, const VertexData *src,
                                           const EdgeData *edge) {
    return 0;  // do nothing
  }

  __host__ __device__ static bool apply(VertexData *vert, int dist) {
    if (vert->depth == -1) {
#ifdef __CUDA_ARCH__
      vert->depth = g_iterationCountGPU;
#else
      vert->depth = g_iterationCount;
#endif
      return true;
    }
    return false;
  }

  __host__ __device__ static void scatter(const VertexData *src, const VertexData *dst,
                                          EdgeData *edge) {}
};

// bfs.cu:81-88
template <bool GPU>
void setIterationCount(int v) {
  if (GPU)
    cudaMemcpyToSymbol(g_iterationCountGPU, &v, sizeof(v));
  else
    g_iterationCount = v;
}

// pagerank.cu:27-73 (static const float -> static constexpr float)
struct PageRank {
  static constexpr float pageConst = 0.15f;
  static constexpr float tol = 0.01f;

  struct VertexData {
    float rank;
    int numOutEdges;
    friend std::ostream &operator<<(std::ostream &out, const VertexData &data);
  };

  struct EdgeData {};

  typedef float GatherResult;

  static constexpr float gatherZero = 0.0f;

  __host__ __device__ static float gatherMap(const VertexData *dst, const VertexData *src,
                                             const EdgeData *edge) {
    return src->rank / src->numOutEdges;
  }

  __host__ __device__ static float gatherReduce(const float &left, const float &right) {
    return left + right;
  }

  __host__ __device__ static bool apply(VertexData *vertexData, const float &gatherResult) {
    float newRank = pageConst + (1.0f - pageConst) * gatherResult;
    bool ret = fabs(newRank - vertexData->rank) >= tol;
    vertexData->rank = newRank;
    return ret;
  }

  __host__ __device__ static void scatter(const VertexData *src, const VertexData *dst,
                                          EdgeData *edge) {}
};

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int32_t h[4];
  if (fread(h, 4, 4, f) != 4) return 2;
  const int32_t nV = h[0], nE = h[1], source = h[2], which = h[3];
  std::vector<int32_t> s(nE), d(nE);
  if (nE && (fread(s.data(), 4, nE, f) != (size_t)nE || fread(d.data(), 4, nE, f) != (size_t)nE))
    return 2;
  fclose(f);
  int32_t status = 0, rounds = 0;
  std::vector<float> out(nV);
  if (which == 0) {
    // bfs.cu:91-112 (depths start at -1, bfs.cu:143-145)
    std::vector<BFS::VertexData> vd(nV);
    for (auto &v : vd) v.depth = -1;
    GASEngineGPU<BFS> engine;
    engine.setGraph(nV, vd.data(), nE, 0, s.data(), d.data());
    engine.setActive(source, source + 1);
    int iter = 0;
    setIterationCount<true>(iter);
    while (engine.countActive() && engine.lastStatus() == GAS_OK) {
      engine.gatherApply(false);
      engine.scatterActivate(false);
      engine.nextIter();
      setIterationCount<true>(++iter);
    }
    engine.getResults();
    status = engine.lastStatus();
    rounds = iter;
    for (int i = 0; i < nV; ++i) memcpy(&out[i], &vd[i].depth, 4);
  } else {
    // pagerank.cu:114-132 (numOutEdges from the CSR), then :85-101
    std::vector<PageRank::VertexData> vd(nV);
    for (auto &v : vd) v.numOutEdges = 0;
    for (int i = 0; i < nE; ++i) vd[s[i]].numOutEdges++;
    for (auto &v : vd) v.rank = PageRank::pageConst;
    GASEngineGPU<PageRank> engine;
    engine.setGraph(nV, vd.data(), nE, 0, s.data(), d.data());
    engine.setActive(0, nV);
    engine.run();  // until no vertex is active
    engine.getResults();
    status = engine.lastStatus();
    for (int i = 0; i < nV; ++i) out[i] = vd[i].rank;
  }
  FILE *o = fopen(argv[2], "wb");
  if (!o) return 2;
  const int32_t head[2] = {status, rounds};
  fwrite(head, 4, 2, o);
  fwrite(out.data(), 4, nV, o);
  fclose(o);
  return status == GAS_OK ? 0 : 1;
}
