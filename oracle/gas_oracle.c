/*
 * gas_oracle.c -- THE ORACLE (test infrastructure, not product code).
 *
 * A plain-C restatement of the reference's CPU Gather-Apply-Scatter engine
 * `GASEngineRef` (refgas.h:30-230) driving restatements of the reference's four
 * vertex programs (bfs.cu:31-80, sssp.cu:25-66, connected_component.cu:25-63,
 * pagerank.cu:27-73) exactly the way the reference apps drive them
 * (bfs.cu:93-134, sssp.cu:69-111 one run, connected_component.cu:66-81,
 * pagerank.cu:85-101), plus an FP64 power-iteration PageRank in the
 * normalised "precision form" (r = (1-d)/N + d * sum r_u/outdeg_u, stop when
 * the global L1 residual <= tol) used to judge the FP32 GPU PageRank.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, and only as the checker / the timed CPU baseline.  The GPU
 * engine never calls into it.
 *
 * Parity pin: tests/test_oracle.py checks every function here against golden
 * vectors that tests/golden/make_golden.py produced by running the reference's
 * own refgas.h (compiled by oracle/Makefile into oracle/_ref/libref.so).
 *
 * One deliberate difference from the reference: edgeListToCSR (util.cuh:80-111)
 * orders the edges of one vertex with an unstable std::sort (util.cuh:49-72);
 * this restatement uses a stable counting sort, so edges of one vertex keep
 * their edge-list order.  Integer programs (min / level) do not depend on that
 * order; PageRank sums can differ in the last ulp, which the tests allow for.
 *
 * Threads: the engine's per-vertex loops and the FP64 PageRank loops run on
 * OpenMP threads (orc_set_threads); results do not depend on the thread
 * count (per-vertex folds stay sequential in CSC order, residuals are summed
 * per fixed chunk of ORC_CHUNK vertices and then in chunk order).
 *
 * Synthetic inputs: orc_rmat, orc_append_grid_islands, orc_set_uniform_weights
 * and orc_sample_sources restate the seeded generators of the product library
 * (graphreduce_gb300/csrc/gas_host_graph.cpp; they have no reference
 * counterpart) so that the CPU baseline can build its workload without
 * loading the product library; tests/test_oracle.py checks that they give
 * the same edge lists, weights and sources.
 *
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off, so x86 and Arm agree).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <limits.h>

#include <omp.h>

#define ORC_EXPORT __attribute__((visibility("default")))
/* Vertices per chunk of the parallel loops whose partial results are joined
 * in a fixed order (next active list, residual sums). */
#define ORC_CHUNK 65536

ORC_EXPORT void orc_set_threads(int32_t n) { if (n > 0) omp_set_num_threads(n); }
ORC_EXPORT int32_t orc_get_threads(void) { return (int32_t)omp_get_max_threads(); }

/* ------------------------------------------------------------------------ */
/* CSR / CSC construction: util.cuh:80-121 (edgeListToCSR / edgeListToCSC).  */
/* ------------------------------------------------------------------------ */

static int cmp_eid(const void *a, const void *b)
{
  const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

/* offsets[nV+1]; out[nE] = vals[perm[i]]; perm[nE] = original edge index.
 * Keys outside [0,nV) are a caller error and return -1.  The result is that
 * of a stable counting sort by key (edges of one key keep their edge-list
 * order); it is computed in parallel by placing edge ids with atomic
 * cursors and then sorting each row's ids. */
ORC_EXPORT int orc_edge_list_to_csr(int32_t nV, int64_t nE,
                                    const int32_t *keys, const int32_t *vals,
                                    int64_t *offsets, int32_t *out,
                                    int32_t *perm)
{
  int64_t i;
  int32_t v;
  int64_t *cursor;
  int32_t *ids = perm;
  int bad = 0;
  for (v = 0; v <= nV; ++v) offsets[v] = 0;
#pragma omp parallel for schedule(static) reduction(|:bad)
  for (i = 0; i < nE; ++i) {
    if (keys[i] < 0 || keys[i] >= nV) { bad = 1; continue; }
    __atomic_fetch_add(&offsets[keys[i] + 1], 1, __ATOMIC_RELAXED);
  }
  if (bad) return -1;
  for (v = 0; v < nV; ++v) offsets[v + 1] += offsets[v];
  cursor = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nV > 0 ? nV : 1));
  if (!ids) ids = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nE > 0 ? nE : 1));
  if (!cursor || !ids) {
    free(cursor);
    if (ids != perm) free(ids);
    return -2;
  }
  memcpy(cursor, offsets, sizeof(int64_t) * (size_t)nV);
#pragma omp parallel for schedule(static)
  for (i = 0; i < nE; ++i)
    ids[__atomic_fetch_add(&cursor[keys[i]], 1, __ATOMIC_RELAXED)] = (int32_t)i;
#pragma omp parallel for schedule(dynamic, 1024)
  for (v = 0; v < nV; ++v) {
    int32_t *row = ids + offsets[v];
    int64_t n = offsets[v + 1] - offsets[v], a, b;
    if (n > 32) {
      qsort(row, (size_t)n, sizeof(int32_t), cmp_eid);
    } else {
      for (a = 1; a < n; ++a) {
        int32_t x = row[a];
        for (b = a; b > 0 && row[b - 1] > x; --b) row[b] = row[b - 1];
        row[b] = x;
      }
    }
  }
  if (out) {
#pragma omp parallel for schedule(static)
    for (i = 0; i < nE; ++i) out[i] = vals[ids[i]];
  }
  free(cursor);
  if (ids != perm) free(ids);
  return 0;
}

typedef struct {
  int32_t nV;
  int64_t nE;
  /* gather side (CSC): in-edges grouped by destination, refgas.h:43-46 */
  int64_t *csc_off;
  int32_t *csc_src;
  int32_t *csc_eid;
  /* scatter side (CSR): out-edges grouped by source, refgas.h:48-51 */
  int64_t *csr_off;
  int32_t *csr_dst;
  int32_t *csr_eid;
} orc_graph;

static void graph_free(orc_graph *g)
{
  free(g->csc_off); free(g->csc_src); free(g->csc_eid);
  free(g->csr_off); free(g->csr_dst); free(g->csr_eid);
}

/* refgas.h:81-113 (setGraph): CSR for scatter, CSC for gather. */
static int graph_init(orc_graph *g, int32_t nV, int64_t nE,
                      const int32_t *srcs, const int32_t *dsts)
{
  size_t ne = (size_t)(nE > 0 ? nE : 1);
  memset(g, 0, sizeof(*g));
  g->nV = nV;
  g->nE = nE;
  g->csc_off = (int64_t *)malloc(sizeof(int64_t) * ((size_t)nV + 1));
  g->csr_off = (int64_t *)malloc(sizeof(int64_t) * ((size_t)nV + 1));
  g->csc_src = (int32_t *)malloc(sizeof(int32_t) * ne);
  g->csc_eid = (int32_t *)malloc(sizeof(int32_t) * ne);
  g->csr_dst = (int32_t *)malloc(sizeof(int32_t) * ne);
  g->csr_eid = (int32_t *)malloc(sizeof(int32_t) * ne);
  if (!g->csc_off || !g->csr_off || !g->csc_src || !g->csc_eid ||
      !g->csr_dst || !g->csr_eid) {
    graph_free(g);
    return -2;
  }
  if (orc_edge_list_to_csr(nV, nE, srcs, dsts, g->csr_off, g->csr_dst,
                           g->csr_eid) ||
      orc_edge_list_to_csr(nV, nE, dsts, srcs, g->csc_off, g->csc_src,
                           g->csc_eid)) {
    graph_free(g);
    return -1;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* The engine, instantiated once per program through gas_oracle_engine.inc.  */
/* ------------------------------------------------------------------------ */

/* BFS::apply reads the level from a global (bfs.cu:27-28, 58-71). */
static int32_t g_bfs_level;

typedef struct { float rank; int32_t numOutEdges; } orc_pr_vertex;

/* BFS: bfs.cu:31-80 */
#define ENG bfs
#define VD int32_t
#define ED int32_t
#define GR int32_t
#define ZERO (INT_MAX - 1)
#define MAP(dst, src, e) ((void)(dst), (void)(src), (void)(e), 0)
#define REDUCE(a, b) ((void)(a), (void)(b), 0)
static inline int bfs_apply(int32_t *v, int32_t g)
{
  (void)g;
  if (*v == -1) { *v = g_bfs_level; return 1; }
  return 0;
}
#define APPLY(v, g) bfs_apply((v), (g))
#include "gas_oracle_engine.inc"

/* SSSP: sssp.cu:25-66 */
#define ENG sssp
#define VD int32_t
#define ED int32_t
#define GR int32_t
#define ZERO (INT_MAX - 100000)
#define MAP(dst, src, e) ((void)(dst), *(src) + *(e))
#define REDUCE(a, b) ((a) < (b) ? (a) : (b))
static inline int min_apply(int32_t *v, int32_t g)
{
  int changed = g < *v;
  if (g < *v) *v = g;
  return changed;
}
#define APPLY(v, g) min_apply((v), (g))
#include "gas_oracle_engine.inc"

/* CC: connected_component.cu:25-63 */
#define ENG cc
#define VD int32_t
#define ED int32_t
#define GR int32_t
#define ZERO INT_MAX
#define MAP(dst, src, e) ((void)(dst), (void)(e), *(src))
#define REDUCE(a, b) ((a) < (b) ? (a) : (b))
#define APPLY(v, g) min_apply((v), (g))
#include "gas_oracle_engine.inc"

/* PageRank, reference (unnormalised) form: pagerank.cu:27-73 */
#define ENG pr
#define VD orc_pr_vertex
#define ED int32_t
#define GR float
#define ZERO 0.0f
#define MAP(dst, src, e) ((void)(dst), (void)(e), (src)->rank / (float)(src)->numOutEdges)
#define REDUCE(a, b) ((a) + (b))
static inline int pr_apply(orc_pr_vertex *v, float g)
{
  const float pageConst = 0.15f, tol = 0.01f;
  float newRank = pageConst + (1.0f - pageConst) * g;
  int ret = fabsf(newRank - v->rank) >= tol;
  v->rank = newRank;
  return ret;
}
#define APPLY(v, g) pr_apply((v), (g))
#include "gas_oracle_engine.inc"

/* ------------------------------------------------------------------------ */
/* Drivers, each mirroring how the reference app runs the engine, on a      */
/* graph built once (orc_graph_new; refgas.h:81-113) so that many runs can  */
/* share it.  All return the number of GAS iterations, or a negative error  */
/* code.  The orc_<program> entry points below build the graph per call.    */
/* ------------------------------------------------------------------------ */

ORC_EXPORT orc_graph *orc_graph_new(int32_t nV, int64_t nE, const int32_t *srcs,
                                    const int32_t *dsts)
{
  orc_graph *g = (orc_graph *)malloc(sizeof(orc_graph));
  if (!g) return NULL;
  if (nV < 0 || nE < 0 || graph_init(g, nV, nE, srcs, dsts)) { free(g); return NULL; }
  return g;
}

ORC_EXPORT void orc_graph_delete(orc_graph *g)
{
  if (!g) return;
  graph_free(g);
  free(g);
}

ORC_EXPORT int64_t orc_graph_num_edges(const orc_graph *g) { return g ? g->nE : -1; }

/* bfs.cu:93-134: depth=-1, setActive(src,src+1), step loop with
 * gather(false)/apply/scatterActivate(false)/nextIter and ++level. */
ORC_EXPORT int64_t orc_g_bfs(const orc_graph *g, int32_t source, int32_t *depth)
{
  bfs_engine e;
  int64_t it = 0;
  int32_t v;
  if (g->nV > 0 && (source < 0 || source >= g->nV)) return -1;
  for (v = 0; v < g->nV; ++v) depth[v] = -1;
  if (bfs_engine_init(&e, g, depth, NULL)) return -2;
  if (g->nV > 0) bfs_set_active(&e, source, source + 1);
  g_bfs_level = 0;
  while (bfs_count_active(&e)) {
    bfs_gather(&e);
    bfs_apply_all(&e);
    bfs_scatter_activate(&e);
    bfs_next_iter(&e);
    g_bfs_level = (int32_t)(++it);
  }
  bfs_engine_free(&e);
  return it;
}

/* sssp.cu:69-111 (one of its ten identical runs): dist = gatherZero except
 * the source, setActive(0,n), step loop with gather/apply/scatter/nextIter.
 * weights: nE records in edge-list order. */
ORC_EXPORT int64_t orc_g_sssp(const orc_graph *g, const int32_t *weights,
                              int32_t source, int32_t *dist)
{
  sssp_engine e;
  int64_t it = 0;
  int32_t v;
  if (g->nV > 0 && (source < 0 || source >= g->nV)) return -1;
  for (v = 0; v < g->nV; ++v) dist[v] = INT_MAX - 100000;
  if (g->nV > 0) dist[source] = 0;
  if (sssp_engine_init(&e, g, dist, weights)) return -2;
  sssp_set_active(&e, 0, g->nV);
  while (sssp_count_active(&e)) {
    sssp_gather(&e);
    sssp_apply_all(&e);
    sssp_scatter_activate(&e);
    sssp_next_iter(&e);
    ++it;
  }
  sssp_engine_free(&e);
  return it;
}

/* connected_component.cu:66-81 and 386-389: label = id, setActive(0,n), run(). */
ORC_EXPORT int64_t orc_g_cc(const orc_graph *g, int32_t *label)
{
  cc_engine e;
  int64_t it;
  int32_t v;
  for (v = 0; v < g->nV; ++v) label[v] = v;
  if (cc_engine_init(&e, g, label, NULL)) return -2;
  cc_set_active(&e, 0, g->nV);
  it = cc_run(&e);
  cc_engine_free(&e);
  return it;
}

/* pagerank.cu:85-101 and 374-382: rank = 0.15, numOutEdges = out-degree,
 * setActive(0,n), run().  rank[] receives the final ranks. */
ORC_EXPORT int64_t orc_g_pagerank(const orc_graph *g, float *rank)
{
  pr_engine e;
  orc_pr_vertex *vd;
  int64_t it;
  int32_t v;
  vd = (orc_pr_vertex *)malloc(sizeof(orc_pr_vertex) * (size_t)(g->nV > 0 ? g->nV : 1));
  if (!vd) return -2;
  for (v = 0; v < g->nV; ++v) {
    vd[v].rank = 0.15f;
    vd[v].numOutEdges = (int32_t)(g->csr_off[v + 1] - g->csr_off[v]);
  }
  if (pr_engine_init(&e, g, vd, NULL)) { free(vd); return -2; }
  pr_set_active(&e, 0, g->nV);
  it = pr_run(&e);
  for (v = 0; v < g->nV; ++v) rank[v] = vd[v].rank;
  pr_engine_free(&e);
  free(vd);
  return it;
}

/* One FP64 power-iteration step shared by the PageRank oracles:
 * contrib[u] = r[u] / outdeg(u) (0 without out-edges), then
 * rn[v] = teleport(v) + d * sum_{u->v} contrib[u] folded in CSC order, with
 * teleport(v) = (1-d)/N for global PageRank (seed < 0) and (1-d)[v == seed]
 * for personalized PageRank.  Returns sum_v |rn[v] - r[v]|, summed per chunk
 * of ORC_CHUNK vertices and then over chunks in order (independent of the
 * thread count), or -1 if the chunk table cannot be allocated. */
static double fp64_step(const orc_graph *g, double damping, int32_t seed,
                        const double *r, double *rn, double *contrib)
{
  const int64_t nV = g->nV;
  const int64_t nchunk = (nV + ORC_CHUNK - 1) / ORC_CHUNK;
  double *part = (double *)malloc(sizeof(double) * (size_t)(nchunk > 0 ? nchunk : 1));
  double l1 = 0.0;
  int64_t c;
  if (!part) return -1.0;
#pragma omp parallel for schedule(static)
  for (c = 0; c < nV; ++c) {
    int64_t od = g->csr_off[c + 1] - g->csr_off[c];
    contrib[c] = od ? r[c] / (double)od : 0.0;
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (c = 0; c < nchunk; ++c) {
    int64_t v, hi = (c + 1) * ORC_CHUNK < nV ? (c + 1) * ORC_CHUNK : nV;
    double acc = 0.0;
    for (v = c * ORC_CHUNK; v < hi; ++v) {
      double s = 0.0;
      int64_t ie;
      for (ie = g->csc_off[v]; ie < g->csc_off[v + 1]; ++ie)
        s += contrib[g->csc_src[ie]];
      rn[v] = (seed < 0 ? (1.0 - damping) / (double)nV
                        : (v == seed ? 1.0 - damping : 0.0)) + damping * s;
      acc += fabs(rn[v] - r[v]);
    }
    part[c] = acc;
  }
  for (c = 0; c < nchunk; ++c) l1 += part[c];
  free(part);
  return l1;
}

/* Power iteration from r0 until the first step whose L1 residual <= tol;
 * -3 after max_iter steps.  seed < 0: precision-form PageRank from 1/N;
 * otherwise personalized PageRank of that seed from e_seed. */
static int64_t fp64_iterate(const orc_graph *g, int32_t seed, double damping,
                            double tol, int64_t max_iter, double *rank,
                            double *l1_out)
{
  const int32_t nV = g->nV;
  double *r, *rn, *contrib;
  int64_t it = 0;
  int32_t v;
  double l1 = 0.0;
  if (nV <= 0) { if (l1_out) *l1_out = 0.0; return seed < 0 ? 0 : -1; }
  if (seed >= nV) return -1;
  r = (double *)malloc(sizeof(double) * (size_t)nV);
  rn = (double *)malloc(sizeof(double) * (size_t)nV);
  contrib = (double *)malloc(sizeof(double) * (size_t)nV);
  if (!r || !rn || !contrib) { free(r); free(rn); free(contrib); return -2; }
  for (v = 0; v < nV; ++v)
    r[v] = seed < 0 ? 1.0 / (double)nV : (v == seed ? 1.0 : 0.0);
  for (;;) {
    if (it >= max_iter) { it = -3; break; }
    l1 = fp64_step(g, damping, seed, r, rn, contrib);
    if (l1 < 0) { it = -2; break; }
    { double *t = r; r = rn; rn = t; }
    ++it;
    if (l1 <= tol) break;
  }
  for (v = 0; v < nV; ++v) rank[v] = r[v];
  if (l1_out) *l1_out = l1;
  free(r); free(rn); free(contrib);
  return it;
}

/* Precision-form PageRank in FP64: r0 = 1/N; every vertex active every
 * iteration; r'_v = (1-d)/N + d * sum_{u->v} r_u / outdeg(u) (no dangling
 * redistribution); stop after the first iteration whose L1 residual
 * sum |r' - r| <= tol, or fail with -3 after max_iter iterations.
 * Returns iterations; *l1_out = last residual. */
ORC_EXPORT int64_t orc_g_pagerank_fp64(const orc_graph *g, double damping,
                                       double tol, int64_t max_iter,
                                       double *rank, double *l1_out)
{
  return fp64_iterate(g, -1, damping, tol, max_iter, rank, l1_out);
}

/* Personalized PageRank in FP64 (no reference counterpart; the formula of
 * orc_g_pagerank_fp64 with the teleport term on one seed): r0 = e_seed;
 * r'_v = (1-d) [v == seed] + d * sum_{u->v} r_u / outdeg(u); stop after the
 * first iteration whose L1 residual <= tol, or fail with -3 after max_iter
 * iterations.  Returns iterations; *l1_out = last residual. */
ORC_EXPORT int64_t orc_g_ppr_fp64(const orc_graph *g, int32_t seed,
                                  double damping, double tol, int64_t max_iter,
                                  double *rank, double *l1_out)
{
  if (seed < 0) return -1;
  return fp64_iterate(g, seed, damping, tol, max_iter, rank, l1_out);
}

/* The same drivers on an edge list (graph built and freed per call). */
#define ORC_ON_EDGES(call)                                      \
  do {                                                          \
    orc_graph *g_ = orc_graph_new(nV, nE, srcs, dsts);          \
    int64_t r_;                                                 \
    if (!g_) return -2;                                         \
    r_ = (call);                                                \
    orc_graph_delete(g_);                                       \
    return r_;                                                  \
  } while (0)

ORC_EXPORT int64_t orc_bfs(int32_t nV, int64_t nE, const int32_t *srcs,
                           const int32_t *dsts, int32_t source,
                           int32_t *depth)
{
  if (nV > 0 && (source < 0 || source >= nV)) return -1;
  ORC_ON_EDGES(orc_g_bfs(g_, source, depth));
}

ORC_EXPORT int64_t orc_sssp(int32_t nV, int64_t nE, const int32_t *srcs,
                            const int32_t *dsts, const int32_t *weights,
                            int32_t source, int32_t *dist)
{
  if (nV > 0 && (source < 0 || source >= nV)) return -1;
  ORC_ON_EDGES(orc_g_sssp(g_, weights, source, dist));
}

ORC_EXPORT int64_t orc_cc(int32_t nV, int64_t nE, const int32_t *srcs,
                          const int32_t *dsts, int32_t *label)
{
  ORC_ON_EDGES(orc_g_cc(g_, label));
}

ORC_EXPORT int64_t orc_pagerank(int32_t nV, int64_t nE, const int32_t *srcs,
                                const int32_t *dsts, float *rank)
{
  ORC_ON_EDGES(orc_g_pagerank(g_, rank));
}

ORC_EXPORT int64_t orc_pagerank_fp64(int32_t nV, int64_t nE,
                                     const int32_t *srcs, const int32_t *dsts,
                                     double damping, double tol,
                                     int64_t max_iter, double *rank,
                                     double *l1_out)
{
  if (nV <= 0) { if (l1_out) *l1_out = 0.0; return 0; }
  ORC_ON_EDGES(orc_g_pagerank_fp64(g_, damping, tol, max_iter, rank, l1_out));
}

ORC_EXPORT int64_t orc_ppr_fp64(int32_t nV, int64_t nE, const int32_t *srcs,
                                const int32_t *dsts, int32_t seed, double damping,
                                double tol, int64_t max_iter, double *rank,
                                double *l1_out)
{
  if (nV <= 0 || seed < 0 || seed >= nV) return -1;
  ORC_ON_EDGES(orc_g_ppr_fp64(g_, seed, damping, tol, max_iter, rank, l1_out));
}

/* One precision-form step on given ranks (FP64), for per-iteration checks
 * of a GPU step: out[v] = (1-d)/N + d * sum r_u/outdeg(u); returns L1. */
ORC_EXPORT double orc_pagerank_fp64_step(int32_t nV, int64_t nE,
                                         const int32_t *srcs,
                                         const int32_t *dsts, double damping,
                                         const double *r, double *out)
{
  orc_graph g;
  double l1 = 0.0;
  int32_t v;
  if (graph_init(&g, nV, nE, srcs, dsts)) return -1.0;
  for (v = 0; v < nV; ++v) {
    double s = 0.0;
    int64_t ie;
    for (ie = g.csc_off[v]; ie < g.csc_off[v + 1]; ++ie) {
      int32_t u = g.csc_src[ie];
      s += r[u] / (double)(g.csr_off[u + 1] - g.csr_off[u]);
    }
    out[v] = (1.0 - damping) / (double)nV + damping * s;
    l1 += fabs(out[v] - r[v]);
  }
  graph_free(&g);
  return l1;
}
