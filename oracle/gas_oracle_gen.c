/*
 * gas_oracle_gen.c -- part of THE ORACLE (test infrastructure, not product
 * code).
 *
 * Seeded synthetic inputs for the CPU baseline and the tests, restated from
 * the product library's generators (graphreduce_gb300/csrc/gas_host_graph.cpp:
 * gas_rmat, gas_edge_list_append_grid_islands,
 * gas_edge_list_set_uniform_weights, gas_edge_list_sample_sources), so that
 * bench.py's CPU arm builds the very same graphs without loading the product
 * library.  The reference has no generators (it reads files, graphio.cpp:
 * 441-473); these follow the workload definitions:
 *   R-MAT: 2^scale vertices, edge_factor * 2^scale samples, quadrant
 *     probabilities (a, b, c, 1-a-b-c) per level, no vertex permutation;
 *     symmetrize adds every reversed sample; self loops and duplicates are
 *     removed and the result is sorted by (src, dst).
 *   Random draws: splitmix64's output function (Steele, Lea & Flood, OOPSLA
 *     2014) applied to (seed key, stream, index), so every draw is a pure
 *     function of its index and nothing depends on the thread count.
 *   Grid islands: side x side 4-neighbour grids after the existing vertices,
 *     each vertex's edges in ascending neighbour order (up, left, right, down)
 *     -- the concatenation at vertex offsets of createCCGraph.cpp:36-44.
 *   Weights: uniform in [lo, hi] from the unordered pair {u, v}, so both
 *     directions of an undirected edge weigh the same.
 *   Sources: k distinct vertices drawn uniformly from the largest weakly
 *     connected component (ties: the component found first by vertex id).
 * tests/test_oracle.py checks each against the product library's output.
 *
 * Arrays returned through pointer arguments are malloc'd here; release them
 * with orc_free.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

#define ORC_EXPORT __attribute__((visibility("default")))

ORC_EXPORT void orc_free(void *p) { free(p); }

static inline uint64_t sm64(uint64_t z)
{
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static inline uint64_t draw_at(uint64_t key, uint64_t stream, uint64_t i)
{
  return sm64(key ^ sm64(stream * 0xD1B54A32D192ED03ull + i));
}

static int cmp_i32(const void *a, const void *b)
{
  const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

static void sort_row(int32_t *p, int64_t n)
{
  if (n <= 24) {
    int64_t i, j;
    for (i = 1; i < n; ++i) {
      int32_t x = p[i];
      for (j = i; j > 0 && p[j - 1] > x; --j) p[j] = p[j - 1];
      p[j] = x;
    }
  } else {
    qsort(p, (size_t)n, sizeof(int32_t), cmp_i32);
  }
}

/* Samples (ku[i], kv[i]) over nV vertices -> edges sorted by (src, dst)
 * without self loops and duplicates.  Bucketed by source (row counts, then
 * each row sorted and deduplicated on its own), which gives the order of a
 * sort by the 64-bit key (src << 32 | dst). */
static int64_t finish_samples(int64_t nV, int64_t nk, const int32_t *ku,
                              const int32_t *kv, int32_t **src_out,
                              int32_t **dst_out)
{
  int64_t *off = (int64_t *)calloc((size_t)nV + 1, sizeof(int64_t));
  int64_t *cur = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nV > 0 ? nV : 1));
  int32_t *col = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nk > 0 ? nk : 1));
  int64_t *keep = (int64_t *)calloc((size_t)nV + 1, sizeof(int64_t));
  int32_t *so = NULL, *dO = NULL;
  int64_t i, v, n;
  if (!off || !cur || !col || !keep) goto fail;
#pragma omp parallel for schedule(static)
  for (i = 0; i < nk; ++i) __atomic_fetch_add(&off[ku[i] + 1], 1, __ATOMIC_RELAXED);
  for (v = 0; v < nV; ++v) off[v + 1] += off[v];
  memcpy(cur, off, sizeof(int64_t) * (size_t)nV);
#pragma omp parallel for schedule(static)
  for (i = 0; i < nk; ++i) {
    int64_t p = __atomic_fetch_add(&cur[ku[i]], 1, __ATOMIC_RELAXED);
    col[p] = kv[i];
  }
#pragma omp parallel for schedule(dynamic, 1024)
  for (v = 0; v < nV; ++v) {
    int32_t *row = col + off[v];
    int64_t len = off[v + 1] - off[v], j, m = 0;
    sort_row(row, len);
    for (j = 0; j < len; ++j) {
      if (row[j] == (int32_t)v) continue;           /* self loop */
      if (m > 0 && row[m - 1] == row[j]) continue;  /* duplicate */
      row[m++] = row[j];
    }
    keep[v + 1] = m;
  }
  for (v = 0; v < nV; ++v) keep[v + 1] += keep[v];
  n = keep[nV];
  so = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  dO = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  if (!so || !dO) goto fail;
#pragma omp parallel for schedule(dynamic, 1024)
  for (v = 0; v < nV; ++v) {
    int64_t j, m = keep[v + 1] - keep[v];
    for (j = 0; j < m; ++j) {
      so[keep[v] + j] = (int32_t)v;
      dO[keep[v] + j] = col[off[v] + j];
    }
  }
  free(off); free(cur); free(col); free(keep);
  *src_out = so;
  *dst_out = dO;
  return n;
fail:
  free(off); free(cur); free(col); free(keep); free(so); free(dO);
  return -2;
}

/* gas_rmat: returns the edge count (or < 0), *src_out / *dst_out malloc'd. */
ORC_EXPORT int64_t orc_rmat(int32_t scale, int32_t edge_factor, double a,
                            double b, double c, uint64_t seed,
                            int32_t symmetrize, int32_t **src_out,
                            int32_t **dst_out)
{
  const double two32 = 4294967296.0;
  int64_t nV, ns, nk, i, n;
  uint64_t ta, tb, tc, key;
  int nwords;
  int32_t *ku, *kv;
  if (!src_out || !dst_out || scale < 1 || scale > 30 || edge_factor < 1 ||
      a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
    return -1;
  nV = (int64_t)1 << scale;
  ns = nV * edge_factor;
  nk = symmetrize ? 2 * ns : ns;
  ku = (int32_t *)malloc(sizeof(int32_t) * (size_t)nk);
  kv = (int32_t *)malloc(sizeof(int32_t) * (size_t)nk);
  if (!ku || !kv) { free(ku); free(kv); return -2; }
  /* quadrant thresholds on 32-bit halves of each 64-bit draw */
  ta = (uint64_t)(a * two32);
  tb = (uint64_t)((a + b) * two32);
  tc = (uint64_t)((a + b + c) * two32);
  key = sm64(seed ^ 0x52D4A7A1F00DULL);
  nwords = (scale + 1) / 2;
#pragma omp parallel for schedule(static)
  for (i = 0; i < ns; ++i) {
    uint64_t u = 0, v = 0;
    int level;
    for (level = 0; level < scale; ++level) {
      const uint64_t r = draw_at(key, 1, (uint64_t)i * (uint64_t)nwords + (uint64_t)(level / 2));
      const uint64_t x = (r >> (32 * (level & 1))) & 0xffffffffull;
      const uint64_t bit = (uint64_t)1 << (scale - 1 - level);
      if (x >= tc) { u |= bit; v |= bit; }
      else if (x >= tb) u |= bit;
      else if (x >= ta) v |= bit;
    }
    ku[i] = (int32_t)u;
    kv[i] = (int32_t)v;
    if (symmetrize) { ku[ns + i] = (int32_t)v; kv[ns + i] = (int32_t)u; }
  }
  n = finish_samples(nV, nk, ku, kv, src_out, dst_out);
  free(ku);
  free(kv);
  return n;
}

/* The edges gas_edge_list_append_grid_islands appends after nV0 vertices:
 * n_islands * 4 * side * (side - 1) of them, written to src / dst (caller
 * arrays).  Returns the edge count, or < 0 on bad arguments. */
ORC_EXPORT int64_t orc_grid_islands(int32_t nV0, int32_t n_islands,
                                    int32_t side, int32_t *src, int32_t *dst)
{
  const int64_t per = (int64_t)side * side;
  const int64_t perE = 4LL * side * (side - 1);
  int32_t k;
  if (nV0 < 0 || n_islands < 0 || side < 1 ||
      (int64_t)nV0 + per * n_islands > INT32_MAX)
    return -1;
#pragma omp parallel for schedule(static)
  for (k = 0; k < n_islands; ++k) {
    const int64_t v0 = (int64_t)nV0 + per * k;
    int64_t p = perE * k;
    int32_t r, cc;
    for (r = 0; r < side; ++r)
      for (cc = 0; cc < side; ++cc) {
        const int32_t v = (int32_t)(v0 + (int64_t)r * side + cc);
        if (r > 0) { src[p] = v; dst[p++] = v - side; }
        if (cc > 0) { src[p] = v; dst[p++] = v - 1; }
        if (cc + 1 < side) { src[p] = v; dst[p++] = v + 1; }
        if (r + 1 < side) { src[p] = v; dst[p++] = v + side; }
      }
  }
  return perE * n_islands;
}

/* gas_edge_list_set_uniform_weights: w[i] uniform in [lo, hi] from the
 * unordered pair {src[i], dst[i]}. */
ORC_EXPORT int orc_uniform_weights(int64_t nE, const int32_t *src,
                                   const int32_t *dst, int32_t lo, int32_t hi,
                                   uint64_t seed, int32_t *w)
{
  const uint64_t key = sm64(seed ^ 0x3E16ull);
  const uint64_t range = (uint64_t)((int64_t)hi - lo + 1);
  int64_t i;
  if (hi < lo) return -1;
#pragma omp parallel for schedule(static)
  for (i = 0; i < nE; ++i) {
    const uint32_t u = (uint32_t)src[i], v = (uint32_t)dst[i];
    const uint64_t pair = u < v ? ((uint64_t)u << 32 | v) : ((uint64_t)v << 32 | u);
    const uint64_t r = draw_at(key, 3, pair);
    w[i] = (int32_t)(lo + (int64_t)(((r >> 32) * range) >> 32));
  }
  return 0;
}

static int32_t uf_find(int32_t *p, int32_t x)
{
  while (p[x] != x) {
    p[x] = p[p[x]];
    x = p[x];
  }
  return x;
}

/* gas_edge_list_sample_sources: k distinct vertices, uniform draws kept only
 * inside the largest weakly connected component (union by smaller root id;
 * the first root of maximum size wins). */
ORC_EXPORT int orc_sample_sources(int32_t nV, int64_t nE, const int32_t *src,
                                  const int32_t *dst, int32_t k, uint64_t seed,
                                  int32_t *out)
{
  int32_t *p, *size, root = 0, got = 0, v;
  int64_t i;
  uint64_t key, j;
  if (nV < 1 || k < 0) return -1;
  p = (int32_t *)malloc(sizeof(int32_t) * (size_t)nV);
  size = (int32_t *)calloc((size_t)nV, sizeof(int32_t));
  if (!p || !size) { free(p); free(size); return -2; }
  for (v = 0; v < nV; ++v) p[v] = v;
  for (i = 0; i < nE; ++i) {
    int32_t a = uf_find(p, src[i]), b = uf_find(p, dst[i]);
    if (a == b) continue;
    if (a < b) p[b] = a; else p[a] = b;
  }
  for (v = 0; v < nV; ++v) ++size[uf_find(p, v)];
  for (v = 0; v < nV; ++v)
    if (size[v] > size[root]) root = v;
  if (k > size[root]) { free(p); free(size); return -1; }
  key = sm64(seed ^ 0x50C5ull);
  for (j = 0; got < k; ++j) {
    const uint64_t r = draw_at(key, 4, j);
    const int32_t x = (int32_t)(((r >> 32) * (uint64_t)nV) >> 32);
    int32_t q, dup = 0;
    if (uf_find(p, x) != root) continue;
    for (q = 0; q < got; ++q) dup |= out[q] == x;
    if (!dup) out[got++] = x;
  }
  free(p);
  free(size);
  return 0;
}
