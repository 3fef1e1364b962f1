// gas_host_graph.cpp -- host-side graph I/O and synthetic graph generators
// of libgas (the reference's graphio.cpp / util.cuh layer, plus the R-MAT,
// Erdos-Renyi and grid-island generators the reference does not have).
#include <omp.h>
#include <parallel/algorithm>

#include <algorithm>
#include <cctype>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "gas.h"
#include "gas_internal.h"

struct gas_edge_list {
  int32_t nV = 0;
  std::vector<int32_t> src, dst, w;
  bool has_w = false;
};

namespace {

// splitmix64 finaliser: a counter-based generator, so every draw is a pure
// function of (seed, index) and the graphs do not depend on thread count.
inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

inline uint64_t draw(uint64_t seed_key, uint64_t stream, uint64_t i) {
  return mix64(seed_key ^ mix64(stream * 0xD1B54A32D192ED03ull + i));
}

// Sort keys (src << 32 | dst), drop self loops and duplicates, split.
gas_status_t finish_keys(std::vector<uint64_t> &keys, int32_t nV,
                         gas_edge_list **out) {
  __gnu_parallel::sort(keys.begin(), keys.end());
  size_t n = 0;
  const size_t m = keys.size();
  for (size_t i = 0; i < m; ++i) {
    const uint64_t k = keys[i];
    if ((uint32_t)(k >> 32) == (uint32_t)k) continue;  // self loop
    if (n > 0 && keys[n - 1] == k) continue;           // duplicate
    keys[n++] = k;
  }
  if (n > (size_t)INT32_MAX)
    return gas::fail(GAS_ERR_TOO_LARGE, "edge count %zu exceeds int32", n);
  gas_edge_list *el = new (std::nothrow) gas_edge_list;
  if (!el) return gas::fail(GAS_ERR_NOMEM, "edge list allocation");
  try {
    el->nV = nV;
    el->src.resize(n);
    el->dst.resize(n);
  } catch (...) {
    delete el;
    return gas::fail(GAS_ERR_NOMEM, "edge list of %zu edges", n);
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    el->src[i] = (int32_t)(keys[i] >> 32);
    el->dst[i] = (int32_t)(uint32_t)keys[i];
  }
  *out = el;
  return GAS_OK;
}

struct UnionFind {
  std::vector<int32_t> p;
  explicit UnionFind(int32_t n) : p(n) {
    for (int32_t i = 0; i < n; ++i) p[i] = i;
  }
  int32_t find(int32_t x) {
    while (p[x] != x) {
      p[x] = p[p[x]];
      x = p[x];
    }
    return x;
  }
  void unite(int32_t a, int32_t b) {
    a = find(a);
    b = find(b);
    if (a == b) return;
    if (a < b)
      p[b] = a;
    else
      p[a] = b;
  }
};

}  // namespace

extern "C" {

gas_status_t gas_edge_list_create(int32_t nV, int64_t nE, const int32_t *srcs,
                                  const int32_t *dsts, const int32_t *weights,
                                  gas_edge_list **out) {
  if (!out || nV < 0 || nE < 0 || (nE > 0 && (!srcs || !dsts)))
    return gas::fail(GAS_ERR_INVALID, "gas_edge_list_create: bad arguments");
  if (nE > INT32_MAX) return gas::fail(GAS_ERR_TOO_LARGE, "nE > INT32_MAX");
  for (int64_t i = 0; i < nE; ++i)
    if (srcs[i] < 0 || srcs[i] >= nV || dsts[i] < 0 || dsts[i] >= nV)
      return gas::fail(GAS_ERR_INVALID, "edge %lld has an endpoint outside [0,%d)",
                       (long long)i, nV);
  gas_edge_list *el = new (std::nothrow) gas_edge_list;
  if (!el) return gas::fail(GAS_ERR_NOMEM, "edge list allocation");
  try {
    el->nV = nV;
    el->src.assign(srcs, srcs + nE);
    el->dst.assign(dsts, dsts + nE);
    if (weights) {
      el->w.assign(weights, weights + nE);
      el->has_w = true;
    }
  } catch (...) {
    delete el;
    return gas::fail(GAS_ERR_NOMEM, "edge list copy");
  }
  *out = el;
  return GAS_OK;
}

void gas_edge_list_destroy(gas_edge_list *el) { delete el; }
int32_t gas_edge_list_num_vertices(const gas_edge_list *el) {
  return el ? el->nV : 0;
}
int64_t gas_edge_list_num_edges(const gas_edge_list *el) {
  return el ? (int64_t)el->src.size() : 0;
}
const int32_t *gas_edge_list_srcs(const gas_edge_list *el) {
  return el && !el->src.empty() ? el->src.data() : nullptr;
}
const int32_t *gas_edge_list_dsts(const gas_edge_list *el) {
  return el && !el->dst.empty() ? el->dst.data() : nullptr;
}
const int32_t *gas_edge_list_weights(const gas_edge_list *el) {
  return el && el->has_w && !el->w.empty() ? el->w.data() : nullptr;
}

gas_status_t gas_rmat(int32_t scale, int32_t edge_factor, double a, double b,
                      double c, uint64_t seed, int32_t symmetrize,
                      gas_edge_list **out) {
  if (!out || scale < 1 || scale > 30 || edge_factor < 1 || a < 0 || b < 0 ||
      c < 0 || a + b + c > 1.0)
    return gas::fail(GAS_ERR_INVALID, "gas_rmat: bad arguments");
  const int64_t nV = (int64_t)1 << scale;
  const int64_t ns = nV * edge_factor;
  const int64_t nk = symmetrize ? 2 * ns : ns;
  std::vector<uint64_t> keys;
  try {
    keys.resize((size_t)nk);
  } catch (...) {
    return gas::fail(GAS_ERR_NOMEM, "gas_rmat: %lld keys", (long long)nk);
  }
  // Quadrant thresholds on 32-bit draws; two levels per 64-bit draw.
  const double two32 = 4294967296.0;
  const uint64_t ta = (uint64_t)(a * two32);
  const uint64_t tb = (uint64_t)((a + b) * two32);
  const uint64_t tc = (uint64_t)((a + b + c) * two32);
  const uint64_t key = mix64(seed ^ 0x52D4A7A1F00DULL);
  const int nwords = (scale + 1) / 2;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < ns; ++i) {
    uint64_t u = 0, v = 0;
    for (int wi = 0; wi < nwords; ++wi) {
      const uint64_t r = draw(key, 1, (uint64_t)i * (uint64_t)nwords + wi);
      for (int h = 0; h < 2; ++h) {
        const int level = 2 * wi + h;
        if (level >= scale) break;
        const uint64_t x = (r >> (32 * h)) & 0xffffffffull;
        const uint64_t bit = (uint64_t)1 << (scale - 1 - level);
        if (x < ta) {
        } else if (x < tb) {
          v |= bit;
        } else if (x < tc) {
          u |= bit;
        } else {
          u |= bit;
          v |= bit;
        }
      }
    }
    keys[(size_t)i] = (u << 32) | v;
    if (symmetrize) keys[(size_t)(ns + i)] = (v << 32) | u;
  }
  return finish_keys(keys, (int32_t)nV, out);
}

gas_status_t gas_erdos_renyi(int32_t nV, int64_t n_samples, uint64_t seed,
                             int32_t symmetrize, gas_edge_list **out) {
  if (!out || nV < 1 || n_samples < 0)
    return gas::fail(GAS_ERR_INVALID, "gas_erdos_renyi: bad arguments");
  const int64_t nk = symmetrize ? 2 * n_samples : n_samples;
  std::vector<uint64_t> keys;
  try {
    keys.resize((size_t)nk);
  } catch (...) {
    return gas::fail(GAS_ERR_NOMEM, "gas_erdos_renyi: %lld keys",
                     (long long)nk);
  }
  const uint64_t key = mix64(seed ^ 0xE2D05ull);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n_samples; ++i) {
    const uint64_t r = draw(key, 2, (uint64_t)i);
    const uint64_t u = ((r & 0xffffffffull) * (uint64_t)nV) >> 32;
    const uint64_t v = ((r >> 32) * (uint64_t)nV) >> 32;
    keys[(size_t)i] = (u << 32) | v;
    if (symmetrize) keys[(size_t)(n_samples + i)] = (v << 32) | u;
  }
  return finish_keys(keys, nV, out);
}

gas_status_t gas_edge_list_append_grid_islands(gas_edge_list *el,
                                               int32_t n_islands,
                                               int32_t side) {
  if (!el || n_islands < 0 || side < 1)
    return gas::fail(GAS_ERR_INVALID, "grid islands: bad arguments");
  const int64_t per = (int64_t)side * side;
  const int64_t addV = per * n_islands;
  const int64_t perE = 4LL * side * (side - 1);
  if ((int64_t)el->nV + addV > INT32_MAX ||
      (int64_t)el->src.size() + perE * n_islands > INT32_MAX)
    return gas::fail(GAS_ERR_TOO_LARGE, "grid islands overflow int32");
  const size_t base = el->src.size();
  try {
    el->src.resize(base + (size_t)(perE * n_islands));
    el->dst.resize(base + (size_t)(perE * n_islands));
    if (el->has_w) el->w.resize(base + (size_t)(perE * n_islands), 0);
  } catch (...) {
    return gas::fail(GAS_ERR_NOMEM, "grid islands");
  }
#pragma omp parallel for schedule(static)
  for (int32_t k = 0; k < n_islands; ++k) {
    const int64_t v0 = (int64_t)el->nV + per * k;
    size_t p = base + (size_t)(perE * k);
    for (int32_t r = 0; r < side; ++r)
      for (int32_t c = 0; c < side; ++c) {
        const int32_t v = (int32_t)(v0 + (int64_t)r * side + c);
        // neighbours in ascending id order: up, left, right, down
        if (r > 0) { el->src[p] = v; el->dst[p++] = v - side; }
        if (c > 0) { el->src[p] = v; el->dst[p++] = v - 1; }
        if (c + 1 < side) { el->src[p] = v; el->dst[p++] = v + 1; }
        if (r + 1 < side) { el->src[p] = v; el->dst[p++] = v + side; }
      }
  }
  el->nV = (int32_t)(el->nV + addV);
  return GAS_OK;
}

gas_status_t gas_edge_list_set_uniform_weights(gas_edge_list *el, int32_t lo,
                                               int32_t hi, uint64_t seed) {
  if (!el || hi < lo) return gas::fail(GAS_ERR_INVALID, "weights: bad range");
  const size_t n = el->src.size();
  try {
    el->w.resize(n);
  } catch (...) {
    return gas::fail(GAS_ERR_NOMEM, "weights");
  }
  el->has_w = true;
  const uint64_t key = mix64(seed ^ 0x3E16ull);
  const uint64_t range = (uint64_t)((int64_t)hi - lo + 1);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const uint32_t u = (uint32_t)el->src[i], v = (uint32_t)el->dst[i];
    const uint64_t pair = u < v ? ((uint64_t)u << 32 | v) : ((uint64_t)v << 32 | u);
    const uint64_t r = draw(key, 3, pair);
    el->w[i] = (int32_t)(lo + (int64_t)(((r >> 32) * range) >> 32));
  }
  return GAS_OK;
}

gas_status_t gas_edge_list_max_out_degree_vertex(const gas_edge_list *el,
                                                 int32_t *vertex,
                                                 int32_t *degree) {
  if (!el || !vertex) return gas::fail(GAS_ERR_INVALID, "null argument");
  std::vector<int32_t> deg(el->nV, 0);
  for (int32_t s : el->src) ++deg[s];
  int32_t best = -1, bestd = -1;
  for (int32_t v = 0; v < el->nV; ++v)
    if (deg[v] > bestd) {
      bestd = deg[v];
      best = v;
    }
  *vertex = best;
  if (degree) *degree = bestd;
  return GAS_OK;
}

gas_status_t gas_edge_list_sample_sources(const gas_edge_list *el, int32_t k,
                                          uint64_t seed, int32_t *out) {
  if (!el || !out || k < 0 || el->nV < 1)
    return gas::fail(GAS_ERR_INVALID, "sample_sources: bad arguments");
  UnionFind uf(el->nV);
  for (size_t i = 0; i < el->src.size(); ++i) uf.unite(el->src[i], el->dst[i]);
  std::vector<int32_t> size(el->nV, 0);
  for (int32_t v = 0; v < el->nV; ++v) ++size[uf.find(v)];
  int32_t root = 0;
  for (int32_t v = 0; v < el->nV; ++v)
    if (size[v] > size[root]) root = v;
  if (k > size[root])
    return gas::fail(GAS_ERR_INVALID, "largest component has %d < %d vertices",
                     size[root], k);
  const uint64_t key = mix64(seed ^ 0x50C5ull);
  int32_t got = 0;
  for (uint64_t i = 0; got < k; ++i) {
    const uint64_t r = draw(key, 4, i);
    const int32_t v = (int32_t)(((r >> 32) * (uint64_t)el->nV) >> 32);
    if (uf.find(v) != root) continue;
    bool dup = false;
    for (int32_t j = 0; j < got; ++j) dup |= out[j] == v;
    if (!dup) out[got++] = v;
  }
  return GAS_OK;
}

gas_status_t gas_edge_list_to_csr(int32_t nV, int64_t nE, const int32_t *keys,
                                  const int32_t *vals, int32_t *offsets,
                                  int32_t *out, int32_t *perm) {
  if (nV < 0 || nE < 0 || !offsets || (nE > 0 && !keys) || (out && !vals))
    return gas::fail(GAS_ERR_INVALID, "edge_list_to_csr: bad arguments");
  if (nE > INT32_MAX) return gas::fail(GAS_ERR_TOO_LARGE, "nE > INT32_MAX");
  return gas::build_csr_host(nV, nE, keys, vals, offsets, out, perm);
}

// Lonestar ".gr": u64 version, u64 edge-data size, u64 nV, u64 nE,
// u64 end-offset[nV], u32 dst[nE] (+ u32 pad when nE is odd),
// u32 edge data[nE]  (graphio.cpp:265-272).
gas_status_t gas_gr_write(const char *path, const gas_edge_list *el) {
  if (!path || !el) return gas::fail(GAS_ERR_INVALID, "gr_write: null argument");
  const int64_t nE = (int64_t)el->src.size();
  std::vector<int32_t> off(el->nV + 1), dst(nE), perm(nE);
  gas_status_t st = gas::build_csr_host(el->nV, nE, el->src.data(),
                                        el->dst.data(), off.data(), dst.data(),
                                        perm.data());
  if (st != GAS_OK) return st;
  FILE *f = fopen(path, "wb");
  if (!f) return gas::fail(GAS_ERR_IO, "cannot open %s for writing", path);
  uint64_t hdr[4] = {1, 4, (uint64_t)el->nV, (uint64_t)nE};
  bool ok = fwrite(hdr, 8, 4, f) == 4;
  std::vector<uint64_t> ends(el->nV);
  for (int32_t v = 0; v < el->nV; ++v) ends[v] = (uint64_t)off[v + 1];
  ok = ok && fwrite(ends.data(), 8, ends.size(), f) == ends.size();
  ok = ok && fwrite(dst.data(), 4, (size_t)nE, f) == (size_t)nE;
  if (nE % 2) {
    uint32_t pad = 0;
    ok = ok && fwrite(&pad, 4, 1, f) == 1;
  }
  std::vector<int32_t> w(nE, 0);
  if (el->has_w)
    for (int64_t i = 0; i < nE; ++i) w[i] = el->w[perm[i]];
  ok = ok && fwrite(w.data(), 4, (size_t)nE, f) == (size_t)nE;
  ok = (fclose(f) == 0) && ok;
  if (!ok) return gas::fail(GAS_ERR_IO, "short write to %s", path);
  return GAS_OK;
}

gas_status_t gas_gr_read(const char *path, gas_edge_list **out) {
  if (!path || !out) return gas::fail(GAS_ERR_INVALID, "gr_read: null argument");
  FILE *f = fopen(path, "rb");
  if (!f) return gas::fail(GAS_ERR_IO, "cannot open %s", path);
  uint64_t hdr[4];
  if (fread(hdr, 8, 4, f) != 4) {
    fclose(f);
    return gas::fail(GAS_ERR_IO, "%s: truncated header", path);
  }
  const uint64_t esz = hdr[1], nV = hdr[2], nE = hdr[3];
  if ((esz != 0 && esz != 4) || nV > (uint64_t)INT32_MAX ||
      nE > (uint64_t)INT32_MAX) {
    fclose(f);
    return gas::fail(GAS_ERR_IO, "%s: unsupported header (edge size %llu)",
                     path, (unsigned long long)esz);
  }
  gas_edge_list *el = new (std::nothrow) gas_edge_list;
  if (!el) {
    fclose(f);
    return gas::fail(GAS_ERR_NOMEM, "gr_read");
  }
  std::vector<uint64_t> ends;
  bool ok = true;
  try {
    el->nV = (int32_t)nV;
    ends.resize(nV);
    el->src.resize(nE);
    el->dst.resize(nE);
  } catch (...) {
    fclose(f);
    delete el;
    return gas::fail(GAS_ERR_NOMEM, "gr_read: %llu edges", (unsigned long long)nE);
  }
  ok = fread(ends.data(), 8, nV, f) == nV;
  ok = ok && fread(el->dst.data(), 4, nE, f) == nE;
  if (ok && (nE % 2)) {
    uint32_t pad;
    ok = fread(&pad, 4, 1, f) == 1;
  }
  if (ok && esz == 4) {
    try {
      el->w.resize(nE);
    } catch (...) {
      ok = false;
    }
    ok = ok && fread(el->w.data(), 4, nE, f) == nE;
    el->has_w = ok;
  }
  fclose(f);
  uint64_t prev = 0;
  for (uint64_t v = 0; ok && v < nV; ++v) {
    if (ends[v] < prev || ends[v] > nE) ok = false;
    for (uint64_t j = prev; ok && j < ends[v]; ++j) el->src[j] = (int32_t)v;
    prev = ends[v];
  }
  ok = ok && (nV == 0 ? nE == 0 : ends[nV - 1] == nE);
  for (uint64_t j = 0; ok && j < nE; ++j)
    if ((uint32_t)el->dst[j] >= nV) ok = false;
  if (!ok) {
    delete el;
    return gas::fail(GAS_ERR_IO, "%s: truncated or inconsistent file", path);
  }
  *out = el;
  return GAS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Text formats: MatrixMarket coordinate and GraphLab / SNAP edge lists.
// ---------------------------------------------------------------------------
namespace {

enum Sym { kSymNone, kSymSym, kSymSkew, kSymHerm };

bool blank_line(const char *p) {
  for (; *p; ++p)
    if (!isspace((unsigned char)*p)) return false;
  return true;
}

// The line loop shared by both formats (loadGraph_common semantics).
gas_status_t read_lines(FILE *f, const char *path, char comment, bool skip_size_line,
                        bool one_based, Sym sym, bool values, gas_edge_list *el) {
  char buf[1024];
  int64_t line = 0;
  int64_t max_v = 0;
  bool size_line = skip_size_line;
  while (fgets(buf, sizeof buf, f)) {
    ++line;
    if (buf[0] == 0 || buf[0] == comment || blank_line(buf)) continue;
    if (size_line) {
      size_line = false;
      continue;
    }
    long long a, b;
    int used = 0;
    if (sscanf(buf, "%lld%lld%n", &a, &b, &used) != 2)
      return gas::fail(GAS_ERR_IO, "%s:%lld: cannot parse src/dst", path, (long long)line);
    if (one_based) {
      --a;
      --b;
    }
    if (a < 0 || b < 0 || a >= INT32_MAX || b >= INT32_MAX)
      return gas::fail(GAS_ERR_IO, "%s:%lld: vertex id out of range", path, (long long)line);
    float val = 0.f;
    if (values && sscanf(buf + used, "%f", &val) != 1)
      return gas::fail(GAS_ERR_IO, "%s:%lld: missing edge value", path, (long long)line);
    if (a == b) {
      if (values) continue;  // dropped before the largest id is updated
    } else {
      el->src.push_back((int32_t)a);
      el->dst.push_back((int32_t)b);
      if (sym != kSymNone) {
        el->src.push_back((int32_t)b);
        el->dst.push_back((int32_t)a);
      }
      if (values) {
        el->w.push_back((int32_t)val);
        if (sym == kSymSym) el->w.push_back((int32_t)val);
        if (sym == kSymSkew) el->w.push_back((int32_t)(-val));
      }
    }
    max_v = std::max<int64_t>(max_v, std::max(a, b));
  }
  if (ferror(f)) return gas::fail(GAS_ERR_IO, "%s: read error", path);
  el->nV = (int32_t)(max_v + 1);
  el->has_w = values;
  return GAS_OK;
}

gas_status_t read_text(const char *path, bool mtx, gas_edge_list **out) {
  if (!path || !out) return gas::fail(GAS_ERR_INVALID, "null argument");
  FILE *f = fopen(path, "r");
  if (!f) return gas::fail(GAS_ERR_IO, "cannot open %s", path);
  Sym sym = kSymNone;
  bool values = false;
  if (mtx) {
    char hdr[1024];
    char t[5][64] = {};
    if (!fgets(hdr, sizeof hdr, f) ||
        sscanf(hdr, "%63s %63s %63s %63s %63s", t[0], t[1], t[2], t[3], t[4]) != 5) {
      fclose(f);
      return gas::fail(GAS_ERR_IO, "%s: bad MatrixMarket header", path);
    }
    if (strcmp(t[1], "matrix") != 0 || strcmp(t[2], "coordinate") != 0) {
      fclose(f);
      return gas::fail(GAS_ERR_IO, "%s: only 'matrix coordinate' files are read", path);
    }
    if (strcmp(t[3], "complex") == 0) {
      fclose(f);
      return gas::fail(GAS_ERR_UNSUPPORTED, "%s: complex edge values", path);
    }
    values = strcmp(t[3], "pattern") != 0;
    if (strcmp(t[4], "general") == 0) sym = kSymNone;
    else if (strcmp(t[4], "symmetric") == 0) sym = kSymSym;
    else if (strcmp(t[4], "skew-symmetric") == 0) sym = kSymSkew;
    else if (strcmp(t[4], "hermitian") == 0) sym = kSymHerm;
    else {
      fclose(f);
      return gas::fail(GAS_ERR_IO, "%s: unrecognised symmetry '%s'", path, t[4]);
    }
    if (sym == kSymHerm && values) {
      fclose(f);
      return gas::fail(GAS_ERR_UNSUPPORTED, "%s: hermitian files with values", path);
    }
  }
  gas_edge_list *el = new (std::nothrow) gas_edge_list;
  if (!el) {
    fclose(f);
    return gas::fail(GAS_ERR_NOMEM, "text graph");
  }
  gas_status_t st;
  try {
    st = read_lines(f, path, mtx ? '%' : '#', mtx, mtx, sym, values, el);
  } catch (...) {
    st = gas::fail(GAS_ERR_NOMEM, "%s: edge list", path);
  }
  fclose(f);
  if (st != GAS_OK) {
    delete el;
    return st;
  }
  *out = el;
  return GAS_OK;
}

}  // namespace

extern "C" {

gas_status_t gas_mtx_read(const char *path, gas_edge_list **out) {
  return read_text(path, true, out);
}

gas_status_t gas_snap_read(const char *path, gas_edge_list **out) {
  return read_text(path, false, out);
}

gas_status_t gas_mtx_write(const char *path, const gas_edge_list *el) {
  if (!path || !el) return gas::fail(GAS_ERR_INVALID, "mtx_write: null argument");
  FILE *f = fopen(path, "w");
  if (!f) return gas::fail(GAS_ERR_IO, "cannot open %s for writing", path);
  const size_t nE = el->src.size();
  bool ok = fprintf(f, "%%%%MatrixMarket matrix coordinate Integer general\n") > 0;
  ok = ok && fprintf(f, "%d %d %zu\n", el->nV, el->nV, nE) > 0;
  for (size_t i = 0; ok && i < nE; ++i) {
    if (el->has_w)
      ok = fprintf(f, "%d %d %d\n", el->src[i] + 1, el->dst[i] + 1, el->w[i]) > 0;
    else
      ok = fprintf(f, "%d %d\n", el->src[i] + 1, el->dst[i] + 1) > 0;
  }
  ok = (fclose(f) == 0) && ok;
  if (!ok) return gas::fail(GAS_ERR_IO, "short write to %s", path);
  return GAS_OK;
}

gas_status_t gas_graph_read(const char *path, gas_edge_list **out) {
  if (!path || !out) return gas::fail(GAS_ERR_INVALID, "null argument");
  const char *dot = strrchr(path, '.');
  if (dot && strcmp(dot, ".gz") == 0)
    return gas::fail(GAS_ERR_UNSUPPORTED, "%s: gzip input is not read; decompress it", path);
  if (dot && strncmp(dot, ".edge", 5) == 0) return gas_snap_read(path, out);
  if (dot && strncmp(dot, ".mtx", 4) == 0) return gas_mtx_read(path, out);
  if (dot && strncmp(dot, ".gr", 3) == 0) return gas_gr_read(path, out);
  return gas::fail(GAS_ERR_UNSUPPORTED, "%s: unrecognised file extension", path);
}

}  // extern "C"

namespace gas {

// Stable counting sort of edges by key: util.cuh:80-111 semantics with the
// edges of one key kept in edge-list order.  Parallel histogram and scatter
// over fixed per-thread edge ranges keep the result independent of timing.
gas_status_t build_csr_host(int32_t nV, int64_t nE, const int32_t *keys,
                            const int32_t *vals, int32_t *offsets,
                            int32_t *out, int32_t *perm) {
  for (int64_t i = 0; i < nE; ++i)
    if (keys[i] < 0 || keys[i] >= nV)
      return fail(GAS_ERR_INVALID, "edge %lld: key %d outside [0,%d)",
                  (long long)i, keys[i], nV);
  // One histogram row per thread: cap the thread count so that the rows
  // stay small next to the edge arrays.
  int64_t nt64 = nV > 0 ? nE / (2 * (int64_t)nV) : 1;
  nt64 = std::min<int64_t>(nt64, std::min(omp_get_max_threads(), 16));
  const int nt = nE >= (1 << 22) && nt64 > 1 ? (int)nt64 : 1;
  std::vector<int32_t> cnt;
  try {
    cnt.assign((size_t)nt * ((size_t)nV + 1), 0);
  } catch (...) {
    return fail(GAS_ERR_NOMEM, "csr histogram");
  }
  const int64_t chunk = (nE + nt - 1) / nt;
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    int32_t *c = cnt.data() + (size_t)t * (nV + 1);
    const int64_t lo = t * chunk, hi = std::min(nE, lo + chunk);
    for (int64_t i = lo; i < hi; ++i) ++c[keys[i]];
  }
  // offsets and per-thread cursors: for key k, thread t starts after all
  // entries of keys < k and of threads < t with key k.
  int64_t run = 0;
  for (int32_t k = 0; k < nV; ++k) {
    offsets[k] = (int32_t)run;
    for (int t = 0; t < nt; ++t) {
      int32_t *c = cnt.data() + (size_t)t * (nV + 1) + k;
      const int64_t n = *c;
      *c = (int32_t)run;
      run += n;
    }
  }
  offsets[nV] = (int32_t)run;
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    int32_t *c = cnt.data() + (size_t)t * (nV + 1);
    const int64_t lo = t * chunk, hi = std::min(nE, lo + chunk);
    for (int64_t i = lo; i < hi; ++i) {
      const int64_t p = c[keys[i]]++;
      if (out) out[p] = vals[i];
      if (perm) perm[p] = (int32_t)i;
    }
  }
  return GAS_OK;
}

}  // namespace gas
