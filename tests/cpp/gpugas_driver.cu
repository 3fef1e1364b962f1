// Test driver for include/gpugas.h: user-defined vertex programs (written
// here, with the semantics of the reference apps' programs) compiled through
// the drop-in GASEngineGPU template and run the way the apps run them.
//
//   gpugas_driver <in.bin> <out.bin>
// in.bin : int32 nV, nE, source, then src[nE], dst[nE], w[nE]
// out.bin: bfs depth[nV], iters; sssp dist[nV], iters; cc label[nV], iters;
//          pagerank rank[nV] (float), iters; graph launches of the CC and
//          PageRank run() calls
#include <climits>
#include <cmath>
#include <cstdio>
#include <vector>

#include "gpugas.h"

int g_level_host;
__device__ __constant__ int g_level_dev;

struct TBFS {
  struct VertexData { int depth; };
  struct EdgeData {};
  typedef int GatherResult;
  static const int gatherZero = INT_MAX - 1;
  __host__ __device__ static int gatherReduce(const int &, const int &) { return 0; }
  __host__ __device__ static int gatherMap(const VertexData *, const VertexData *,
                                           const EdgeData *) { return 0; }
  __host__ __device__ static bool apply(VertexData *v, int) {
    if (v->depth == -1) {
#ifdef __CUDA_ARCH__
      v->depth = g_level_dev;
#else
      v->depth = g_level_host;
#endif
      return true;
    }
    return false;
  }
  __host__ __device__ static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

struct TSSSP {
  typedef int VertexData;
  typedef int EdgeData;
  typedef int GatherResult;
  static const int gatherZero = INT_MAX - 100000;
  __host__ __device__ static int gatherReduce(const int &a, const int &b) { return a < b ? a : b; }
  __host__ __device__ static int gatherMap(const int *, const int *s, const int *e) { return *s + *e; }
  __host__ __device__ static bool apply(int *c, int d) {
    bool ch = d < *c;
    *c = d < *c ? d : *c;
    return ch;
  }
  __host__ __device__ static void scatter(const int *, const int *, int *) {}
};

struct TCC {
  typedef int VertexData;
  struct EdgeData {};
  typedef int GatherResult;
  static const int gatherZero = INT_MAX;
  __host__ __device__ static int gatherReduce(const int &a, const int &b) { return a < b ? a : b; }
  __host__ __device__ static int gatherMap(const int *, const int *s, const EdgeData *) { return *s; }
  __host__ __device__ static bool apply(int *c, int l) {
    bool ch = l < *c;
    *c = l < *c ? l : *c;
    return ch;
  }
  __host__ __device__ static void scatter(const int *, const int *, EdgeData *) {}
};

struct TPR {
  struct VertexData { float rank; int numOutEdges; };
  struct EdgeData {};
  typedef float GatherResult;
  static constexpr float gatherZero = 0.0f;
  __host__ __device__ static float gatherMap(const VertexData *, const VertexData *s,
                                             const EdgeData *) {
    return s->rank / s->numOutEdges;
  }
  __host__ __device__ static float gatherReduce(const float &a, const float &b) { return a + b; }
  __host__ __device__ static bool apply(VertexData *v, const float &g) {
    float nr = 0.15f + (1.0f - 0.15f) * g;
    bool ret = fabsf(nr - v->rank) >= 0.01f;
    v->rank = nr;
    return ret;
  }
  __host__ __device__ static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

int main(int argc, char **argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: gpugas_driver in.bin out.bin\n");
    return 2;
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 3;
  int hdr[3];
  if (fread(hdr, 4, 3, f) != 3) return 3;
  const int nV = hdr[0], nE = hdr[1], source = hdr[2];
  std::vector<int> src(nE), dst(nE), w(nE);
  if (nE && (fread(src.data(), 4, nE, f) != (size_t)nE || fread(dst.data(), 4, nE, f) != (size_t)nE ||
             fread(w.data(), 4, nE, f) != (size_t)nE))
    return 3;
  fclose(f);
  FILE *o = fopen(argv[2], "wb");
  if (!o) return 4;

  {  // bfs.cu:93-134
    std::vector<TBFS::VertexData> vd(nV);
    for (int i = 0; i < nV; ++i) vd[i].depth = -1;
    GASEngineGPU<TBFS> engine;
    engine.setGraph(nV, vd.data(), nE, 0, src.data(), dst.data());
    engine.setActive(source, source + 1);
    int it = 0;
    cudaMemcpyToSymbol(g_level_dev, &it, sizeof(it));
    while (engine.countActive()) {
      engine.gather(false);
      engine.apply();
      engine.scatterActivate(false);
      engine.nextIter();
      ++it;
      cudaMemcpyToSymbol(g_level_dev, &it, sizeof(it));
    }
    engine.getResults();
    fwrite(vd.data(), 4, nV, o);
    fwrite(&it, 4, 1, o);
  }
  {  // sssp.cu:69-111, twice on one engine (setGraph is re-callable)
    std::vector<int> vd(nV);
    GASEngineGPU<TSSSP> engine;
    int it = 0;
    for (int rep = 0; rep < 2; ++rep) {
      it = 0;
      for (int i = 0; i < nV; ++i) vd[i] = TSSSP::gatherZero;
      if (nV) vd[source] = 0;
      engine.setGraph(nV, vd.data(), nE, w.data(), src.data(), dst.data());
      engine.setActive(0, nV);
      while (engine.countActive()) {
        engine.gather();
        engine.apply();
        engine.scatterActivate();
        engine.nextIter();
        ++it;
      }
      engine.getResults();
    }
    fwrite(vd.data(), 4, nV, o);
    fwrite(&it, 4, 1, o);
  }
  int launches[2] = {-1, -1};  // graph launches of the two run() calls
  {  // connected_component.cu:66-81, through run()
    std::vector<int> vd(nV);
    for (int i = 0; i < nV; ++i) vd[i] = i;
    GASEngineGPU<TCC> engine;
    engine.setGraph(nV, vd.data(), nE, 0, src.data(), dst.data());
    engine.setActive(0, nV);
    engine.run();
    engine.getResults();
    const int it = engine.lastRun().iterations;
    launches[0] = engine.lastRun().graph_launches;
    fwrite(vd.data(), 4, nV, o);
    fwrite(&it, 4, 1, o);
  }
  {  // pagerank.cu:85-101 and 374-382
    std::vector<int> outdeg(nV, 0);
    for (int i = 0; i < nE; ++i) ++outdeg[src[i]];
    std::vector<TPR::VertexData> vd(nV);
    for (int i = 0; i < nV; ++i) {
      vd[i].rank = 0.15f;
      vd[i].numOutEdges = outdeg[i];
    }
    GASEngineGPU<TPR> engine;
    engine.setGraph(nV, vd.data(), nE, 0, src.data(), dst.data());
    engine.setActive(0, nV);
    engine.run();
    engine.getResults();
    std::vector<float> r(nV);
    for (int i = 0; i < nV; ++i) r[i] = vd[i].rank;
    fwrite(r.data(), 4, nV, o);
    const int it = engine.lastRun().iterations;
    launches[1] = engine.lastRun().graph_launches;
    fwrite(&it, 4, 1, o);
  }
  fwrite(launches, 4, 2, o);
  fclose(o);
  return 0;
}
