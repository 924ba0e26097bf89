// A user vertex Program whose scatter writes its edge, driven through the
// C++ engine template (gas_gb300/gpugas.cuh) as a reference driver would
// (sssp.cu:67-82): every vertex active, run to the end, results back.
//
//   edge_scatter in.bin out.bin
//     in:  int32 nV, nE, source, mode (0 = stepwise gatherApply /
//          scatterActivate / nextIter loop, 1 = run(), 2 = run() one
//          launch per phase), then srcs[nE], dsts[nE], weights[nE]
//     out: int32 status, rounds, then dist[nV], visits[nE], last[nE]
#include <climits>
#include <cstdio>
#include <vector>

#include <gas_gb300/gpugas.cuh>

struct SSSPVisits {
  typedef int VertexData;
  struct EdgeData {
    int w, visits, last;
  };
  typedef int GatherResult;
  static constexpr int gatherZero = INT_MAX - 100000;
  static constexpr bool scatterEdges = true;
  __host__ __device__ static int gatherReduce(const int &l, const int &r) { return l < r ? l : r; }
  __host__ __device__ static int gatherMap(const VertexData *, const VertexData *s,
                                           const EdgeData *e) {
    return *s + e->w;
  }
  __host__ __device__ static bool apply(VertexData *cur, GatherResult d) {
    const bool changed = d < *cur;
    *cur = d < *cur ? d : *cur;
    return changed;
  }
  __host__ __device__ static void scatter(const VertexData *src, const VertexData *,
                                          EdgeData *e) {
    e->visits += 1;
    e->last = *src;
  }
};

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int32_t h[4];
  if (fread(h, 4, 4, f) != 4) return 2;
  const int32_t nV = h[0], nE = h[1], source = h[2], mode = h[3];
  std::vector<int32_t> s(nE), d(nE), w(nE);
  if (nE && (fread(s.data(), 4, nE, f) != (size_t)nE || fread(d.data(), 4, nE, f) != (size_t)nE ||
             fread(w.data(), 4, nE, f) != (size_t)nE))
    return 2;
  fclose(f);
  std::vector<int> dist(nV, SSSPVisits::gatherZero);
  dist[source] = 0;
  std::vector<SSSPVisits::EdgeData> ed(nE > 0 ? nE : 1);
  for (int i = 0; i < nE; ++i) ed[i] = {w[i], 0, 0};
  GASEngineGPU<SSSPVisits> engine;
  engine.setGraph(nV, dist.data(), nE, ed.data(), s.data(), d.data());
  engine.setActive(0, nV);
  int32_t rounds = 0;
  if (mode == 0) {
    while (engine.countActive() && engine.lastStatus() == GAS_OK) {
      engine.gatherApply();
      engine.scatterActivate();
      engine.nextIter();
      ++rounds;
    }
  } else {
    engine.setPersistent(mode == 1);
    rounds = engine.runFor(0);
  }
  engine.getResults();
  const int32_t status = engine.lastStatus();
  FILE *o = fopen(argv[2], "wb");
  if (!o) return 2;
  const int32_t head[2] = {status, rounds};
  fwrite(head, 4, 2, o);
  fwrite(dist.data(), 4, nV, o);
  for (int i = 0; i < nE; ++i) fwrite(&ed[i].visits, 4, 1, o);
  for (int i = 0; i < nE; ++i) fwrite(&ed[i].last, 4, 1, o);
  fclose(o);
  return status == GAS_OK ? 0 : 1;
}
