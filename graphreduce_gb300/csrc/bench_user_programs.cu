// bench_user_programs.cu -- times the drop-in path: vertex programs written
// the way the reference apps write them (bfs.cu:31-80, sssp.cu:25-66,
// connected_component.cu:25-63), compiled through include/gpugas.h and run
// the way the apps run them: BFS and SSSP through the step API from the
// host (bfs.cu:93-134, sssp.cu:69-111), CC through run()
// (connected_component.cu:66-81), whose loop runs on the device.  Each
// program's timed region is the apps' own: from after setActive to after
// getResults, with setGraph outside it (sssp.cu:88-105).
//
//   bench_user_programs <graph.bin> <reps> <out.bin> [<cc_graph.bin>]
// graph.bin: int32 nV, nE, n_sources, then src[nE], dst[nE], w[nE],
//            sources[n_sources] (source 0 also runs BFS); CC runs on
//            cc_graph.bin (same layout, no sources) when it is given
// out.bin:   bfs depth[nV]; sssp dist[n_sources][nV]; cc label[nV of the CC graph]
// stdout:    one JSON line with per-run milliseconds (mean of reps runs
//            after one untimed) and iteration counts.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdio>
#include <vector>

#include "gpugas.h"

namespace {

__device__ __constant__ int g_level;

struct UBfs {  // bfs.cu:31-80
  struct VertexData { int depth; };
  struct EdgeData {};
  typedef int GatherResult;
  static const int gatherZero = INT_MAX - 1;
  __host__ __device__ static int gatherReduce(const int &, const int &) { return 0; }
  __host__ __device__ static int gatherMap(const VertexData *, const VertexData *,
                                           const EdgeData *) { return 0; }
  __host__ __device__ static bool apply(VertexData *v, int) {
#ifdef __CUDA_ARCH__
    if (v->depth == -1) {
      v->depth = g_level;
      return true;
    }
#endif
    return false;
  }
  __host__ __device__ static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

struct USssp {  // sssp.cu:25-66
  typedef int VertexData;
  typedef int EdgeData;
  typedef int GatherResult;
  static const int gatherZero = INT_MAX - 100000;
  __host__ __device__ static int gatherReduce(const int &a, const int &b) { return a < b ? a : b; }
  __host__ __device__ static int gatherMap(const int *, const int *s, const int *e) {
    return *s + *e;
  }
  __host__ __device__ static bool apply(int *c, int d) {
    const bool ch = d < *c;
    if (ch) *c = d;
    return ch;
  }
  __host__ __device__ static void scatter(const int *, const int *, int *) {}
};

struct UCc {  // connected_component.cu:25-63
  typedef int VertexData;
  struct EdgeData {};
  typedef int GatherResult;
  static const int gatherZero = INT_MAX;
  __host__ __device__ static int gatherReduce(const int &a, const int &b) { return a < b ? a : b; }
  __host__ __device__ static int gatherMap(const int *, const int *s, const EdgeData *) {
    return *s;
  }
  __host__ __device__ static bool apply(int *c, int l) {
    const bool ch = l < *c;
    if (ch) *c = l;
    return ch;
  }
  __host__ __device__ static void scatter(const int *, const int *, EdgeData *) {}
};

struct Timer {
  cudaEvent_t a, b;
  Timer() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~Timer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  void start() { cudaEventRecord(a, 0); }
  float stop() {
    cudaEventRecord(b, 0);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
};

}  // namespace

struct Graph {
  int nV = 0, nE = 0;
  std::vector<int> src, dst, w, sources;
};

bool read_graph(const char *path, Graph &g) {
  FILE *f = fopen(path, "rb");
  if (!f) return false;
  int hdr[3];
  bool ok = fread(hdr, 4, 3, f) == 3 && hdr[0] >= 0 && hdr[1] >= 0 && hdr[2] >= 0;
  if (ok) {
    g.nV = hdr[0];
    g.nE = hdr[1];
    g.src.resize(g.nE);
    g.dst.resize(g.nE);
    g.w.resize(g.nE);
    g.sources.resize(hdr[2]);
    ok = (g.nE == 0 || (fread(g.src.data(), 4, g.nE, f) == (size_t)g.nE &&
                        fread(g.dst.data(), 4, g.nE, f) == (size_t)g.nE &&
                        fread(g.w.data(), 4, g.nE, f) == (size_t)g.nE)) &&
         (hdr[2] == 0 || fread(g.sources.data(), 4, hdr[2], f) == (size_t)hdr[2]);
  }
  fclose(f);
  return ok;
}

int main(int argc, char **argv) {
  if (argc != 4 && argc != 5) {
    fprintf(stderr, "usage: bench_user_programs graph.bin reps out.bin [cc_graph.bin]\n");
    return 2;
  }
  const int reps = atoi(argv[2]);
  Graph g, gc;  // the main graph (BFS, SSSP) and the CC graph
  if (reps < 1 || !read_graph(argv[1], g) || g.sources.empty()) return 3;
  if (argc == 5 && !read_graph(argv[4], gc)) return 3;
  const Graph &ccg = argc == 5 ? gc : g;
  const int nV = g.nV, nE = g.nE, ns = (int)g.sources.size();
  const std::vector<int> &src = g.src, &dst = g.dst, &sources = g.sources;
  std::vector<int> &w = g.w;  // setGraph takes EdgeData* (sssp.cu passes its own vector)
  FILE *o = fopen(argv[3], "wb");
  if (!o) return 4;
  Timer tm;

  // BFS from sources[0] (bfs.cu:93-134: the level goes to the device before
  // every apply)
  double bfs_ms = 0.0;
  int bfs_levels = 0;
  {
    std::vector<UBfs::VertexData> vd(nV);
    GASEngineGPU<UBfs> engine;
    for (int r = 0; r <= reps; ++r) {
      for (int i = 0; i < nV; ++i) vd[i].depth = -1;
      engine.setGraph(nV, vd.data(), nE, 0, src.data(), dst.data());
      engine.setActive(sources[0], sources[0] + 1);
      tm.start();
      int it = 0;
      cudaMemcpyToSymbol(g_level, &it, sizeof(it));
      while (engine.countActive()) {
        engine.gather(false);
        engine.apply();
        engine.scatterActivate(false);
        engine.nextIter();
        ++it;
        cudaMemcpyToSymbol(g_level, &it, sizeof(it));
      }
      engine.getResults();
      const float ms = tm.stop();
      if (r) bfs_ms += ms;
      bfs_levels = it;
    }
    fwrite(vd.data(), 4, nV, o);
  }

  // SSSP from every source (sssp.cu:69-111)
  double sssp_ms = 0.0;
  std::vector<int> sssp_iters(ns);
  {
    std::vector<int> vd(nV);
    GASEngineGPU<USssp> engine;
    for (int k = 0; k < ns; ++k) {
      for (int r = 0; r <= reps; ++r) {
        for (int i = 0; i < nV; ++i) vd[i] = USssp::gatherZero;
        vd[sources[k]] = 0;
        engine.setGraph(nV, vd.data(), nE, w.data(), src.data(), dst.data());
        engine.setActive(0, nV);
        tm.start();
        int it = 0;
        while (engine.countActive()) {
          engine.gather();
          engine.apply();
          engine.scatterActivate();
          engine.nextIter();
          ++it;
        }
        engine.getResults();
        const float ms = tm.stop();
        if (r) sssp_ms += ms;
        sssp_iters[k] = it;
      }
      fwrite(vd.data(), 4, nV, o);
    }
  }

  // CC through run() (connected_component.cu:66-81)
  double cc_ms = 0.0;
  int cc_iters = 0, cc_graph_launches = 0;
  {
    std::vector<int> vd(ccg.nV);
    GASEngineGPU<UCc> engine;
    for (int r = 0; r <= reps; ++r) {
      for (int i = 0; i < ccg.nV; ++i) vd[i] = i;
      engine.setGraph(ccg.nV, vd.data(), ccg.nE, 0, ccg.src.data(), ccg.dst.data());
      engine.setActive(0, ccg.nV);
      tm.start();
      engine.run();
      engine.getResults();
      const float ms = tm.stop();
      if (r) cc_ms += ms;
      cc_iters = engine.lastRun().iterations;
      cc_graph_launches = engine.lastRun().graph_launches;
    }
    fwrite(vd.data(), 4, ccg.nV, o);
  }
  fclose(o);
  printf("{\"bfs_ms\": %.4f, \"bfs_levels\": %d, \"sssp_ms_per_source\": %.4f, "
         "\"sssp_iterations\": [",
         bfs_ms / reps, bfs_levels, sssp_ms / reps / ns);
  for (int k = 0; k < ns; ++k) printf("%s%d", k ? ", " : "", sssp_iters[k]);
  printf("], \"cc_ms\": %.4f, \"cc_iterations\": %d, \"cc_graph_launches\": %d}\n",
         cc_ms / reps, cc_iters, cc_graph_launches);
  return 0;
}
