// ref_driver.cu -- part of THE ORACLE (test infrastructure, not product code).
//
// Compiles the reference's own CPU engine GASEngineRef (refgas.h) and graph
// I/O (graphio.cpp) from the reference sources, by oracle/Makefile, into
// oracle/_ref/libref.so.  Nothing from the reference is copied here: this file
// only #includes refgas.h / util.cuh / graphio.h from the reference directory
// and exposes flat extern "C" entry points so that tests/golden/make_golden.py
// can produce golden vectors from the reference itself.
//
// The Program structs below restate the reference apps' vertex programs
// (bfs.cu:31-80, sssp.cu:25-66, connected_component.cu:25-63,
// pagerank.cu:27-73); each run_* function drives GASEngineRef the way the
// matching app's run<> template does.
#include <climits>
#include <cmath>
#include <cstdint>
#include <vector>

#include "refgas.h"
#include "graphio.h"

namespace {

int g_level;  // bfs.cu:27 g_iterationCount

struct RefBFS {
  struct VertexData { int depth; };
  struct EdgeData {};
  typedef int GatherResult;
  static const int gatherZero = INT_MAX - 1;
  static int gatherReduce(const int &, const int &) { return 0; }
  static int gatherMap(const VertexData *, const VertexData *, const EdgeData *) { return 0; }
  static bool apply(VertexData *v, int) {
    if (v->depth == -1) { v->depth = g_level; return true; }
    return false;
  }
  static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};

struct RefSSSP {
  typedef int VertexData;
  typedef int EdgeData;
  typedef int GatherResult;
  static const int gatherZero = INT_MAX - 100000;
  static int gatherReduce(const int &a, const int &b) { return a < b ? a : b; }
  static int gatherMap(const int *, const int *src, const int *len) { return *src + *len; }
  static bool apply(int *cur, int d) {
    bool changed = d < *cur;
    *cur = d < *cur ? d : *cur;
    return changed;
  }
  static void scatter(const int *, const int *, int *) {}
};

struct RefCC {
  typedef int VertexData;
  struct EdgeData {};
  typedef int GatherResult;
  static const int gatherZero = INT_MAX;
  static int gatherReduce(const int &a, const int &b) { return a < b ? a : b; }
  static int gatherMap(const int *, const int *src, const EdgeData *) { return *src; }
  static bool apply(int *cur, int l) {
    bool changed = l < *cur;
    *cur = l < *cur ? l : *cur;
    return changed;
  }
  static void scatter(const int *, const int *, EdgeData *) {}
};

struct RefPR {
  struct VertexData { float rank; int numOutEdges; };
  struct EdgeData {};
  typedef float GatherResult;
  static const float gatherZero;
  static float gatherMap(const VertexData *, const VertexData *src, const EdgeData *) {
    return src->rank / src->numOutEdges;
  }
  static float gatherReduce(const float &a, const float &b) { return a + b; }
  static bool apply(VertexData *v, const float &g) {
    const float pageConst = 0.15f, tol = 0.01f;
    float newRank = pageConst + (1.0f - pageConst) * g;
    bool ret = std::fabs(newRank - v->rank) >= tol;
    v->rank = newRank;
    return ret;
  }
  static void scatter(const VertexData *, const VertexData *, EdgeData *) {}
};
const float RefPR::gatherZero = 0.0f;

}  // namespace

extern "C" {

// bfs.cu:93-134
int64_t ref_bfs(int nV, int nE, const int *srcs, const int *dsts, int source,
                int *depth) {
  std::vector<RefBFS::VertexData> vd(nV);
  for (int i = 0; i < nV; ++i) vd[i].depth = -1;
  GASEngineRef<RefBFS> engine;
  engine.setGraph(nV, vd.data(), nE, 0, srcs, dsts);
  engine.setActive(source, source + 1);
  int64_t it = 0;
  g_level = 0;
  while (engine.countActive()) {
    engine.gather(false);
    engine.apply();
    engine.scatterActivate(false);
    engine.nextIter();
    g_level = (int)(++it);
  }
  engine.getResults();
  for (int i = 0; i < nV; ++i) depth[i] = vd[i].depth;
  return it;
}

// sssp.cu:69-111, one run
int64_t ref_sssp(int nV, int nE, const int *srcs, const int *dsts,
                 const int *weights, int source, int *dist) {
  for (int i = 0; i < nV; ++i) dist[i] = RefSSSP::gatherZero;
  dist[source] = 0;
  std::vector<int> ed(weights, weights + nE);
  GASEngineRef<RefSSSP> engine;
  engine.setGraph(nV, dist, nE, ed.data(), srcs, dsts);
  engine.setActive(0, nV);
  int64_t it = 0;
  while (engine.countActive()) {
    engine.gather();
    engine.apply();
    engine.scatterActivate();
    engine.nextIter();
    ++it;
  }
  engine.getResults();
  return it;
}

// connected_component.cu:66-81
int64_t ref_cc(int nV, int nE, const int *srcs, const int *dsts, int *label) {
  for (int i = 0; i < nV; ++i) label[i] = i;
  GASEngineRef<RefCC> engine;
  engine.setGraph(nV, label, nE, 0, srcs, dsts);
  engine.setActive(0, nV);
  int64_t it = 0;
  while (engine.countActive()) {
    engine.gather();
    engine.apply();
    engine.scatterActivate();
    engine.nextIter();
    ++it;
  }
  engine.getResults();
  return it;
}

// pagerank.cu:85-101 with pagerank.cu:374-382 for numOutEdges
int64_t ref_pagerank(int nV, int nE, const int *srcs, const int *dsts,
                     float *rank) {
  std::vector<int> off(nV + 1);
  edgeListToCSR<int>(nV, nE, srcs, dsts, off.data(), 0, 0);
  std::vector<RefPR::VertexData> vd(nV);
  for (int i = 0; i < nV; ++i) {
    vd[i].numOutEdges = off[i + 1] - off[i];
    vd[i].rank = 0.15f;
  }
  GASEngineRef<RefPR> engine;
  engine.setGraph(nV, vd.data(), nE, 0, srcs, dsts);
  engine.setActive(0, nV);
  int64_t it = 0;
  while (engine.countActive()) {
    engine.gather();
    engine.apply();
    engine.scatterActivate();
    engine.nextIter();
    ++it;
  }
  engine.getResults();
  for (int i = 0; i < nV; ++i) rank[i] = vd[i].rank;
  return it;
}

// util.cuh:80-111
void ref_edge_list_to_csr(int nV, int nE, const int *srcs, const int *dsts,
                          int *offsets, int *out, int *perm) {
  edgeListToCSR<int>(nV, nE, srcs, dsts, offsets, out, perm);
}

// graphio.cpp:365-413
int ref_write_gr(const char *fname, int nV, int nE, const int *offsets,
                 const int *dsts, const int *weights) {
  writeGraph_binaryCSR(fname, nV, nE, offsets, dsts, weights);
  return 0;
}

// graphio.cpp:416-437
int ref_write_mtx(const char *fname, int nV, int nE, const int *srcs, const int *dsts,
                  const int *weights) {
  writeGraph_mtx(fname, nV, nE, srcs, dsts, weights);
  return 0;
}

// graphio.cpp:274-362 through loadGraph (graphio.cpp:441-473).  Returns the
// edge count; srcs/dsts/weights must hold cap entries.
int64_t ref_load_graph(const char *fname, int want_weights, int cap, int *nV,
                       int *srcs, int *dsts, int *weights) {
  std::vector<int> s, d, w;
  int n = 0;
  loadGraph(fname, n, s, d, want_weights ? &w : 0);
  *nV = n;
  if ((int64_t)s.size() > cap) return -1;
  for (size_t i = 0; i < s.size(); ++i) {
    srcs[i] = s[i];
    dsts[i] = d[i];
    if (want_weights) weights[i] = w[i];
  }
  return (int64_t)s.size();
}

}  // extern "C"
