// gas_engine.cu -- libgas: the GASEngineGPU engine behind the C ABI of
// include/gas.h, for sm_103a.
//
// Layout in HBM per graph (all int32, device resident for the engine's life):
//   csc_off[V+1], csc_src[E], csc_ed[E]    gather side, edge data in CSC order
//   csr_off[V+1], csr_dst[E], csr_ed[E]    scatter side
// Frontier state (V-sized, reused every iteration):
//   active[V] ascending ids, active_scan[V+1] in-degree scan, apply_ret[V],
//   slot[V] new vertex data per active slot, gather_tmp[V], next-frontier
//   bitmap bits[V/32], scatter scan sscan[V+1], per-tile carries.
// Counters live in one device line (gas_counters); the step API reads them
// back once per nextIter()/countActive(), the fast runs never do until the
// end (the loop is a CUDA graph with a device-side WHILE condition).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "gas.h"
#include "gas_device.cuh"
#include "gas_internal.h"
#include "gas_engine_impl.h"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
namespace gas {
namespace {
thread_local char g_err[512];
}
gas_status_t fail(gas_status_t s, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return s;
}
void clear_error() { g_err[0] = 0; }
const char *g_err_ptr() { return g_err; }
}  // namespace gas

using gasdev::kNT;
using gasdev::SegSource;

// ---------------------------------------------------------------------------
// Built-in vertex programs (device restatements of the reference's four).
// ---------------------------------------------------------------------------
namespace progs {

// sssp.cu:25-66
struct Sssp {
  typedef int32_t VertexData;
  typedef int32_t EdgeData;
  typedef int32_t GatherResult;
  static constexpr int32_t gatherZero = INT_MAX - 100000;
  __device__ static int32_t gatherReduce(const int32_t &a, const int32_t &b) {
    return a < b ? a : b;
  }
  __device__ static int32_t gatherMap(const int32_t *, const int32_t *s,
                                      const int32_t *e) {
    return *s + *e;
  }
  __device__ static bool apply(int32_t *c, const int32_t &d) {
    const bool ch = d < *c;
    if (ch) *c = d;
    return ch;
  }
};

// connected_component.cu:25-63
struct Cc {
  typedef int32_t VertexData;
  typedef int32_t EdgeData;
  typedef int32_t GatherResult;
  static constexpr int32_t gatherZero = INT_MAX;
  __device__ static int32_t gatherReduce(const int32_t &a, const int32_t &b) {
    return a < b ? a : b;
  }
  __device__ static int32_t gatherMap(const int32_t *, const int32_t *s,
                                      const int32_t *) {
    return *s;
  }
  __device__ static bool apply(int32_t *c, const int32_t &l) {
    const bool ch = l < *c;
    if (ch) *c = l;
    return ch;
  }
};

struct PrVertex {
  float rank;
  int32_t numOutEdges;
};

// pagerank.cu:27-73, with explicitly rounded operations so that no FMA
// contraction changes the result relative to the reference's CPU engine.
struct PageRank {
  typedef PrVertex VertexData;
  typedef int32_t EdgeData;
  typedef float GatherResult;
  static constexpr float gatherZero = 0.0f;
  __device__ static float gatherReduce(const float &a, const float &b) {
    return __fadd_rn(a, b);
  }
  __device__ static float gatherMap(const PrVertex *, const PrVertex *s,
                                    const int32_t *) {
    return __fdiv_rn(s->rank, (float)s->numOutEdges);
  }
  __device__ static bool apply(PrVertex *v, const float &g) {
    const float pageConst = 0.15f, tol = 0.01f;
    const float nr = __fadd_rn(pageConst, __fmul_rn(__fsub_rn(1.0f, pageConst), g));
    const bool ret = fabsf(__fsub_rn(nr, v->rank)) >= tol;
    v->rank = nr;
    return ret;
  }
};

}  // namespace progs

// ---------------------------------------------------------------------------
// Program-independent kernels.
// ---------------------------------------------------------------------------
namespace {

constexpr int kScanItems = 16;                   // items per thread in scans
constexpr int kScanBlock = kNT * kScanItems;     // 4096 slots per block
constexpr int kWordsPerThread = 4;               // bitmap words per thread
constexpr int kCompactBlock = kNT * kWordsPerThread;  // 1024 words per block

__device__ __forceinline__ int warp_incl_sum(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int o = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += o;
  }
  return v;
}

// Exclusive prefix sum over the CTA (kNT threads); *total gets the sum.
__device__ __forceinline__ int block_excl_sum(int v, int *total) {
  __shared__ int s_w[kNT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int incl = warp_incl_sum(v);
  if (lane == 31) s_w[warp] = incl;
  __syncthreads();
  int pre = 0, tot = 0;
  for (int w = 0; w < kNT / 32; ++w) {
    if (w < warp) pre += s_w[w];
    tot += s_w[w];
  }
  __syncthreads();
  *total = tot;
  return pre + incl - v;
}

__global__ void k_set_range(int32_t start, int32_t n, const int32_t *csc_off,
                            int32_t *act, int32_t *scan, gas_counters *cnt) {
  const int32_t base = csc_off[start];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n;
       i += gridDim.x * blockDim.x) {
    if (i < n) act[i] = start + i;
    scan[i] = csc_off[start + i] - base;
    if (i == n) {
      cnt->n_active = n;
      cnt->n_edges = csc_off[start + n] - base;
      cnt->n_scatter_edges = 0;
    }
  }
}

// vd[act[i]] = slot[i]: makes the applied vertex data visible after every
// gather of the iteration has read the old values (bulk-synchronous apply).
__global__ void k_commit(const int32_t *act, const gas_counters *cnt,
                         const uint8_t *slot, uint8_t *vd, int vbytes) {
  const int n = cnt->n_active;
  if ((vbytes & 3) == 0) {
    const int w = vbytes >> 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
      const uint32_t *s = reinterpret_cast<const uint32_t *>(slot) + (size_t)i * w;
      uint32_t *d = reinterpret_cast<uint32_t *>(vd) + (size_t)act[i] * w;
      for (int k = 0; k < w; ++k) d[k] = s[k];
    }
  } else {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
      const uint8_t *s = slot + (size_t)i * vbytes;
      uint8_t *d = vd + (size_t)act[i] * vbytes;
      for (int k = 0; k < vbytes; ++k) d[k] = s[k];
    }
  }
}

// Scan of out-degree over apply()==true slots -> sscan (three passes:
// per-block totals, spine, per-block scan).
__device__ __forceinline__ int pred_outdeg(const int32_t *act,
                                           const uint8_t *ret,
                                           const int32_t *csr_off, int i,
                                           int n) {
  if (i >= n || !ret[i]) return 0;
  const int v = act[i];
  return csr_off[v + 1] - csr_off[v];
}

__global__ void __launch_bounds__(kNT)
    k_pscan_reduce(const int32_t *act, const uint8_t *ret,
                   const int32_t *csr_off, const gas_counters *cnt,
                   int32_t *part) {
  const int n = cnt->n_active;
  const int nb = (n + kScanBlock - 1) / kScanBlock;
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    int s = 0;
    const int base = b * kScanBlock + threadIdx.x;
#pragma unroll 4
    for (int k = 0; k < kScanItems; ++k)
      s += pred_outdeg(act, ret, csr_off, base + k * kNT, n);
    int tot;
    block_excl_sum(s, &tot);
    if (threadIdx.x == 0) part[b] = tot;
  }
}

// Single CTA: exclusive scan of part[0..nb) in place; total to *total.
__device__ void spine_scan(int32_t *part, int nb, int32_t *total) {
  __shared__ int s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += kNT) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? part[i] : 0;
    int tot;
    const int ex = block_excl_sum(v, &tot);
    const int carry = s_carry;
    if (i < nb) part[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) s_carry = carry + tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = s_carry;
}

__global__ void __launch_bounds__(kNT)
    k_pscan_spine(int32_t *part, gas_counters *cnt) {
  const int n = cnt->n_active;
  const int nb = (n + kScanBlock - 1) / kScanBlock;
  spine_scan(part, nb, &cnt->n_scatter_edges);
}

__global__ void __launch_bounds__(kNT)
    k_pscan_down(const int32_t *act, const uint8_t *ret,
                 const int32_t *csr_off, const gas_counters *cnt,
                 const int32_t *part, int32_t *sscan) {
  const int n = cnt->n_active;
  const int nb = (n + kScanBlock - 1) / kScanBlock;
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    // each thread owns kScanItems consecutive slots
    const int base = b * kScanBlock + threadIdx.x * kScanItems;
    int vals[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      vals[k] = pred_outdeg(act, ret, csr_off, base + k, n);
      s += vals[k];
    }
    int tot;
    int run = block_excl_sum(s, &tot) + part[b];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      if (base + k < n) sscan[base + k] = run;
      run += vals[k];
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) sscan[n] = cnt->n_scatter_edges;
}

// Expansion: set the next-frontier bit of every out-neighbour of every
// apply()==true vertex.
struct ExpandPol {
  typedef int32_t Val;
  const int32_t *csr_dst;
  uint32_t *bits;
  __device__ Val zero() const { return 0; }
  __device__ Val reduce(Val a, Val) const { return a; }
  __device__ Val map(int, int, int) const { return 0; }
  __device__ void emit(int, int, Val) const {}
  __device__ __forceinline__ void visit(int, int, int pos) const {
    const uint32_t w = (uint32_t)__ldg(csr_dst + pos);
    atomicOr(bits + (w >> 5), 1u << (w & 31));
  }
};

__global__ void __launch_bounds__(kNT)
    k_expand(ExpandPol pol, SegSource src) {
  gasdev::tile_loop<ExpandPol, false, false>(pol, src, nullptr, nullptr, nullptr);
}

// Compaction of the next-frontier bitmap into the ascending active list with
// its in-degree scan (scatter_if_mgpu.h:130-157 + the gather's degree scan),
// clearing the bitmap for the following iteration.
__device__ __forceinline__ void word_stats(const uint32_t *bits,
                                           const int32_t *off, int nW, int w,
                                           int *c, int *d) {
  *c = 0;
  *d = 0;
  if (w >= nW) return;
  uint32_t m = bits[w];
  *c = __popc(m);
  while (m) {
    const int b = __ffs(m) - 1;
    m &= m - 1;
    const int v = w * 32 + b;
    *d += off[v + 1] - off[v];
  }
}

__global__ void __launch_bounds__(kNT)
    k_compact_count(const uint32_t *bits, const int32_t *csc_off, int nW,
                    int32_t *part) {
  const int b = blockIdx.x;
  int c = 0, d = 0;
  for (int k = 0; k < kWordsPerThread; ++k) {
    int cc, dd;
    word_stats(bits, csc_off, nW, b * kCompactBlock + threadIdx.x * kWordsPerThread + k,
               &cc, &dd);
    c += cc;
    d += dd;
  }
  int tc, td;
  block_excl_sum(c, &tc);
  block_excl_sum(d, &td);
  if (threadIdx.x == 0) {
    part[2 * b] = tc;
    part[2 * b + 1] = td;
  }
}

__global__ void __launch_bounds__(kNT)
    k_compact_spine(int32_t *part, int nb, gas_counters *cnt) {
  // de-interleave in place is awkward; scan the two series one after the
  // other with a stride-2 view.
  __shared__ int s_carry[2];
  if (threadIdx.x < 2) s_carry[threadIdx.x] = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += kNT) {
    const int i = base + threadIdx.x;
    const int vc = i < nb ? part[2 * i] : 0;
    const int vd = i < nb ? part[2 * i + 1] : 0;
    int tc, td;
    const int ec = block_excl_sum(vc, &tc);
    const int ed = block_excl_sum(vd, &td);
    const int cc = s_carry[0], cd = s_carry[1];
    if (i < nb) {
      part[2 * i] = cc + ec;
      part[2 * i + 1] = cd + ed;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      s_carry[0] = cc + tc;
      s_carry[1] = cd + td;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    cnt->n_active = s_carry[0];
    cnt->n_edges = s_carry[1];
  }
}

__global__ void __launch_bounds__(kNT)
    k_compact_write(uint32_t *bits, const int32_t *csc_off, int nW,
                    const int32_t *part, int32_t *act, int32_t *scan,
                    const gas_counters *cnt) {
  const int b = blockIdx.x;
  const int w0 = b * kCompactBlock + threadIdx.x * kWordsPerThread;
  int c = 0, d = 0;
  for (int k = 0; k < kWordsPerThread; ++k) {
    int cc, dd;
    word_stats(bits, csc_off, nW, w0 + k, &cc, &dd);
    c += cc;
    d += dd;
  }
  int tc, td;
  int pc = block_excl_sum(c, &tc) + part[2 * b];
  int pd = block_excl_sum(d, &td) + part[2 * b + 1];
  for (int k = 0; k < kWordsPerThread; ++k) {
    const int w = w0 + k;
    if (w >= nW) break;
    uint32_t m = bits[w];
    if (!m) continue;
    bits[w] = 0;
    while (m) {
      const int bit = __ffs(m) - 1;
      m &= m - 1;
      const int v = w * 32 + bit;
      act[pc] = v;
      scan[pc] = pd;
      ++pc;
      pd += csc_off[v + 1] - csc_off[v];
    }
  }
  if (b == 0 && threadIdx.x == 0) scan[cnt->n_active] = cnt->n_edges;
}

// BFS apply without gather (bfs.cu:58-71): level from the engine.
__global__ void k_bfs_apply(const int32_t *act, const gas_counters *cnt,
                            int32_t *depth, uint8_t *ret, int32_t level,
                            int32_t level_from_counters) {
  const int n = cnt->n_active;
  if (level_from_counters) level = cnt->iteration;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    int32_t *d = depth + act[i];
    const bool r = *d == -1;
    if (r) *d = level;
    ret[i] = r ? 1 : 0;
  }
}

}  // namespace

namespace {

template <class T>
gas_status_t dalloc(T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    return gas::fail(GAS_ERR_NOMEM, "cudaMalloc of %zu bytes: %s",
                     n * sizeof(T), cudaGetErrorString(e));
  }
  return GAS_OK;
}

template <class T>
void dfree(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

// Edge arrays in pinned, mapped host memory (GAS_EDGES_HOST): kernels read
// them over NVLink-C2C through their device address.
template <class T>
gas_status_t halloc(T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  void *h = nullptr;
  cudaError_t e = cudaHostAlloc(&h, n * sizeof(T), cudaHostAllocMapped);
  void *d = nullptr;
  if (e == cudaSuccess) e = cudaHostGetDevicePointer(&d, h, 0);
  if (e != cudaSuccess) {
    if (h) cudaFreeHost(h);
    return gas::fail(GAS_ERR_NOMEM, "cudaHostAlloc of %zu bytes: %s", n * sizeof(T),
                     cudaGetErrorString(e));
  }
  if (d != h) {  // kernels and the host must see one address (UVA)
    cudaFreeHost(h);
    return gas::fail(GAS_ERR_UNSUPPORTED, "host edge arrays need unified addressing");
  }
  *p = static_cast<T *>(h);
  return GAS_OK;
}

template <class T>
void hfree(T *&p) {
  if (p) cudaFreeHost((void *)p);
  p = nullptr;
}

void free_graph(gas_engine *e) {
  dfree(e->csc_off); dfree(e->csr_off);
  if (e->edges_on_host) {
    hfree(e->csc_src); hfree(e->csr_dst); hfree(e->csc_ed); hfree(e->csr_ed);
  } else {
    dfree(e->csc_src); dfree(e->csr_dst); dfree(e->csc_ed); dfree(e->csr_ed);
  }
  e->edges_on_host = false;
  dfree(e->vd); dfree(e->act); dfree(e->scan); dfree(e->sscan); dfree(e->ret);
  dfree(e->slot); dfree(e->gres); dfree(e->bits);
  dfree(e->tile_first); dfree(e->tile_carry); dfree(e->tile_a0);
  dfree(e->tpart); dfree(e->dpart);
  dfree(e->ppart); dfree(e->cpart); dfree(e->cnt);
  for (int i = 0; i < 2; ++i) { dfree(e->pr_rank[i]); dfree(e->pr_contrib[i]); }
  dfree(e->pr_seed); dfree(e->pr_inv_deg); dfree(e->pr_l1); dfree(e->csr_to_csc);
  dfree(e->pr_tile_row); dfree(e->pr_head); dfree(e->pr_tail);
  dfree(e->sb_bits); dfree(e->sb_ctl); dfree(e->sb_heavy);
  e->sb_clean = false;
  e->pr_tile_cap = 0;
  e->h_csr_perm.clear();
  e->h_csr_to_csc.clear();
  e->host_ed = nullptr;
  e->edges_dirty = false;
  dfree(e->q_ids); dfree(e->q_vals); dfree(e->q_end); dfree(e->q_delta); dfree(e->snap);
  dfree(e->qpart); dfree(e->cbits);
  dfree(e->ne_vid); dfree(e->ne_end);
  dfree(e->slab_dpart); dfree(e->slab_qpart); dfree(e->slab_a0);
  dfree(e->slab_first); dfree(e->slab_carry); dfree(e->slab_fix); dfree(e->slab_fix_n);
  dfree(e->trace); dfree(e->hist);
  e->n_ne = e->slab_cap = 0;
  for (int i = 0; i < kGraphSlots; ++i) {
    if (e->graphs[i]) cudaGraphExecDestroy(e->graphs[i]);
    e->graphs[i] = nullptr;
  }
  e->has_graph = false;
}

size_t program_vbytes(gas_program_t p) {
  switch (p) {
    case GAS_PROG_BFS: case GAS_PROG_SSSP: case GAS_PROG_CC: return 4;
    case GAS_PROG_PAGERANK: return 8;
    default: return 0;
  }
}

inline cudaStream_t S(void *s) { return (cudaStream_t)s; }

int grid_for(int64_t work_items, int per_block, int cap) {
  int64_t g = (work_items + per_block - 1) / per_block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

template <class K>
int occupancy_grid(gas_engine *e, K kernel, size_t smem = 0) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kNT, smem);
  if (per_sm < 1) per_sm = 1;
  return e->num_sms * per_sm;
}

gas_status_t sync_counts(gas_engine *e, void *stream) {
  CUDA_TRY(cudaMemcpyAsync(e->h_cnt, e->cnt, sizeof(gas_counters),
                           cudaMemcpyDeviceToHost, S(stream)));
  CUDA_TRY(cudaStreamSynchronize(S(stream)));
  e->n_active = e->h_cnt->n_active;
  e->n_edges = e->h_cnt->n_edges;
  e->counts_dirty = false;
  return GAS_OK;
}

// Launch the generic gather (fused with apply or not) for program P.
template <class P>
gas_status_t launch_generic_gather(gas_engine *e, bool fuse, bool ordered,
                                   void *stream) {
  using GR = typename P::GatherResult;
  gasdev::GenericGather<P> pol;
  pol.csc_src = e->csc_src;
  pol.csc_ed = static_cast<const typename P::EdgeData *>(e->csc_ed);
  pol.vd = static_cast<const typename P::VertexData *>(e->vd);
  pol.slot = static_cast<typename P::VertexData *>(e->slot);
  pol.ret = e->ret;
  pol.gres = static_cast<GR *>(e->gres);
  pol.fuse = fuse ? 1 : 0;
  if (ordered) {
    const int g = e->capturing ? 8 * e->num_sms : grid_for(e->n_active, kNT, 65535);
    gasdev::k_gather_ordered<P><<<g, kNT, 0, S(stream)>>>(pol, e->act,
                                                          e->csc_off, e->cnt);
    CUDA_TRY(cudaGetLastError());
    return GAS_OK;
  }
  const SegSource src = gasdev::frontier_source(
      e->act, e->scan, e->csc_off, &e->cnt->n_active, &e->cnt->n_edges, e->tpart);
  constexpr int kTile = gasdev::TileShape<sizeof(GR)>::kTile;
  const int64_t items = (int64_t)e->n_active + e->n_edges;
  gasdev::k_partition<kTile, false>
      <<<gas::engine_partition_grid(e, items, kTile), 256, 0, S(stream)>>>(src, e->tpart);
  const int cap = occupancy_grid(e, gasdev::k_gather_tiles<P>);
  const int grid = e->capturing ? cap : grid_for(items, kTile, cap);
  gasdev::k_gather_tiles<P><<<grid, kNT, 0, S(stream)>>>(
      pol, src, static_cast<GR *>(e->tile_first),
      static_cast<GR *>(e->tile_carry), e->tile_a0);
  CUDA_TRY(cudaGetLastError());
  const int64_t ntiles = (items + kTile - 1) / kTile;
  const int fgrid = e->capturing ? 4 * e->num_sms
                                  : grid_for(ntiles, kNT / 32, 4 * e->num_sms);
  gasdev::k_gather_fixup<P><<<fgrid, kNT, 0, S(stream)>>>(
      pol, src, static_cast<GR *>(e->tile_first),
      static_cast<GR *>(e->tile_carry), e->tile_a0);
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

gas_status_t builtin_gather(gas_engine *e, bool fuse, bool ordered,
                            void *stream) {
  switch (e->prog) {
    case GAS_PROG_SSSP: return launch_generic_gather<progs::Sssp>(e, fuse, ordered, stream);
    case GAS_PROG_CC: return launch_generic_gather<progs::Cc>(e, fuse, ordered, stream);
    case GAS_PROG_PAGERANK: return launch_generic_gather<progs::PageRank>(e, fuse, ordered, stream);
    default: return GAS_OK;  // BFS: gatherMap/gatherReduce are no-ops
  }
}

gas_status_t builtin_apply_only(gas_engine *e, void *stream) {
  const int grid = e->capturing ? 8 * e->num_sms
                                : grid_for(e->n_active, kNT, 8 * e->num_sms);
  switch (e->prog) {
    case GAS_PROG_BFS:
      k_bfs_apply<<<grid, kNT, 0, S(stream)>>>(e->act, e->cnt,
                                                (int32_t *)e->vd, e->ret, e->level,
                                                e->level_from_counters ? 1 : 0);
      break;
    case GAS_PROG_SSSP:
      gasdev::k_apply_only<progs::Sssp><<<grid, kNT, 0, S(stream)>>>(
          e->act, e->cnt, (int32_t *)e->vd,
          e->have_gres ? (const int32_t *)e->gres : nullptr, e->ret);
      break;
    case GAS_PROG_CC:
      gasdev::k_apply_only<progs::Cc><<<grid, kNT, 0, S(stream)>>>(
          e->act, e->cnt, (int32_t *)e->vd,
          e->have_gres ? (const int32_t *)e->gres : nullptr, e->ret);
      break;
    case GAS_PROG_PAGERANK:
      gasdev::k_apply_only<progs::PageRank><<<grid, kNT, 0, S(stream)>>>(
          e->act, e->cnt, (progs::PrVertex *)e->vd,
          e->have_gres ? (const float *)e->gres : nullptr, e->ret);
      break;
    default:
      return gas::fail(GAS_ERR_UNSUPPORTED, "apply: not a built-in program");
  }
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

// commit pending slots, expand, compact.
gas_status_t scatter_common(gas_engine *e, void *stream) {
  if (e->slots_pending) {
    const int g = e->capturing ? 8 * e->num_sms
                               : grid_for(e->n_active, kNT, 8 * e->num_sms);
    k_commit<<<g, kNT, 0, S(stream)>>>(
        e->act, e->cnt, (const uint8_t *)e->slot, (uint8_t *)e->vd,
        (int)e->vbytes);
    CUDA_TRY(cudaGetLastError());
    e->slots_pending = false;
  }
  const int nblk = grid_for(e->nV, kScanBlock, INT_MAX);
  k_pscan_reduce<<<nblk, kNT, 0, S(stream)>>>(e->act, e->ret, e->csr_off,
                                               e->cnt, e->ppart);
  k_pscan_spine<<<1, kNT, 0, S(stream)>>>(e->ppart, e->cnt);
  k_pscan_down<<<nblk, kNT, 0, S(stream)>>>(e->act, e->ret, e->csr_off, e->cnt,
                                             e->ppart, e->sscan);
  CUDA_TRY(cudaGetLastError());
  ExpandPol pol{e->csr_dst, e->bits};
  const SegSource src = gasdev::frontier_source(
      e->act, e->sscan, e->csr_off, &e->cnt->n_active, &e->cnt->n_scatter_edges,
      e->tpart);
  constexpr int kTile = gasdev::TileShape<sizeof(int32_t)>::kTile;
  // the scatter edge count is only known on the device: fixed grids
  gasdev::k_partition<kTile, false>
      <<<gas::engine_partition_grid(e, -1, kTile), 256, 0, S(stream)>>>(src, e->tpart);
  k_expand<<<occupancy_grid(e, k_expand), kNT, 0, S(stream)>>>(pol, src);
  CUDA_TRY(cudaGetLastError());
  const int nW = (e->nV + 31) / 32;
  k_compact_count<<<e->n_cblocks, kNT, 0, S(stream)>>>(e->bits, e->csc_off, nW,
                                                        e->cpart);
  k_compact_spine<<<1, kNT, 0, S(stream)>>>(e->cpart, e->n_cblocks, e->cnt);
  k_compact_write<<<e->n_cblocks, kNT, 0, S(stream)>>>(
      e->bits, e->csc_off, nW, e->cpart, e->act, e->scan, e->cnt);
  CUDA_TRY(cudaGetLastError());
  e->counts_dirty = true;
  e->have_gres = false;
  e->active_full = false;
  return GAS_OK;
}

gas_status_t flush_pending_gather(gas_engine *e, void *stream) {
  if (!e->pending_gather) return GAS_OK;
  e->pending_gather = false;
  if (e->prog == GAS_PROG_USER)
    return gas::fail(GAS_ERR_STATE, "user engine: gather must be launched by the header");
  GAS_TRY(builtin_gather(e, /*fuse=*/false, false, stream));
  e->have_gres = true;
  return GAS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char *gas_status_string(gas_status_t s) {
  switch (s) {
    case GAS_OK: return "ok";
    case GAS_ERR_INVALID: return "invalid argument";
    case GAS_ERR_NOMEM: return "out of memory";
    case GAS_ERR_CUDA: return "CUDA error";
    case GAS_ERR_ITER_CAP: return "iteration cap reached";
    case GAS_ERR_IO: return "I/O error";
    case GAS_ERR_STATE: return "call out of order";
    case GAS_ERR_UNSUPPORTED: return "unsupported";
    case GAS_ERR_DEVICE: return "device-side error";
    case GAS_ERR_TOO_LARGE: return "too large";
  }
  return "unknown status";
}

const char *gas_last_error(void) { return gas::g_err_ptr(); }

const char *gas_version(void) { return "libgas 0.1 (sm_103a)"; }

gas_status_t gas_engine_create(gas_program_t program, gas_engine **out) {
  if (!out) return gas::fail(GAS_ERR_INVALID, "null out");
  if (program < GAS_PROG_BFS || program > GAS_PROG_PAGERANK)
    return gas::fail(GAS_ERR_INVALID, "unknown program %d", (int)program);
  gas_engine *e = new (std::nothrow) gas_engine;
  if (!e) return gas::fail(GAS_ERR_NOMEM, "engine");
  e->prog = program;
  e->vbytes = program_vbytes(program);
  e->gbytes = 4;
  e->ebytes = 4;
  if (const char *pd = getenv("GAS_PULL_DIV")) {
    const int v = atoi(pd);
    if (v > 0) e->pull_div = v;
  }
  *out = e;  // CUDA is first touched by set_graph
  return GAS_OK;
}

gas_status_t gas_engine_create_user(size_t vertex_bytes, size_t gather_bytes,
                                    size_t edge_bytes, gas_engine **out) {
  if (!out || vertex_bytes == 0 || gather_bytes == 0)
    return gas::fail(GAS_ERR_INVALID, "create_user: bad sizes");
  gas_status_t s = gas_engine_create(GAS_PROG_BFS, out);
  if (s != GAS_OK) return s;
  (*out)->prog = GAS_PROG_USER;
  (*out)->vbytes = vertex_bytes;
  (*out)->gbytes = gather_bytes;
  (*out)->ebytes = edge_bytes;
  return GAS_OK;
}

void gas_engine_destroy(gas_engine *e) {
  if (!e) return;
  free_graph(e);
  for (int i = 0; i < 2; ++i)
    if (e->prof_ev[i]) cudaEventDestroy(e->prof_ev[i]);
  if (e->h_cnt) cudaFreeHost(e->h_cnt);
  delete e;
}

gas_status_t gas_engine_set_graph(gas_engine *e, int32_t nV, void *vertex_data,
                                  int64_t nE, const void *edge_data,
                                  const int32_t *srcs, const int32_t *dsts,
                                  void *stream) {
  if (!e || nV < 0 || nE < 0 || (nE > 0 && (!srcs || !dsts)) ||
      (nV > 0 && !vertex_data))
    return gas::fail(GAS_ERR_INVALID, "set_graph: bad arguments");
  if (nE > INT32_MAX || (int64_t)nV + nE + 1 > INT32_MAX)
    return gas::fail(GAS_ERR_TOO_LARGE, "set_graph: V + E must stay below 2^31");
  if (e->prog == GAS_PROG_SSSP && nE > 0 && !edge_data)
    return gas::fail(GAS_ERR_INVALID, "SSSP needs edge weights");
  if (e->prog == GAS_PROG_SSSP) {
    // The SSSP Program's margin (sssp.cu:32-33): gatherZero = INT_MAX - 100000,
    // so dist + w stays below INT_MAX only for weights up to 100000.
    const int32_t *w = static_cast<const int32_t *>(edge_data);
    for (int64_t i = 0; i < nE; ++i)
      if (w[i] < 0 || w[i] > 100000)
        return gas::fail(GAS_ERR_INVALID,
                         "set_graph: SSSP weight %d of edge %lld outside [0, 100000]", w[i],
                         (long long)i);
  }
  free_graph(e);
  if (!e->h_cnt) {
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce == cudaSuccess)
      ce = cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (ce == cudaSuccess)
      ce = cudaMallocHost((void **)&e->h_cnt, sizeof(gas_counters));
    if (ce != cudaSuccess) {
      e->h_cnt = nullptr;
      return gas::fail(GAS_ERR_CUDA, "set_graph: %s", cudaGetErrorString(ce));
    }
  }
  e->nV = nV;
  e->nE = (int32_t)nE;
  e->host_vd = vertex_data;

  // CSC / CSR (stable by edge-list order), edge data permuted into both
  // orders (gpugas.h:1358-1378): on the device for large graphs, by a
  // counting sort on the host otherwise (GAS_GRAPH_BUILD=host|device forces
  // one).
  const size_t eb = e->ebytes;
  const bool have_ed = edge_data && eb > 0;
  const bool want_perms = have_ed && e->prog == GAS_PROG_USER;
  const bool dev_build = gas::device_build_for(nE);
  std::vector<int32_t> csc_src, csc_perm, csr_off, csr_dst, csr_perm;
  std::vector<uint8_t> ed_csc, ed_csr;
  if (!dev_build) {
    try {
      e->h_csc_off.assign((size_t)nV + 1, 0);
      csc_src.resize(nE); csc_perm.resize(nE);
      csr_off.resize((size_t)nV + 1); csr_dst.resize(nE); csr_perm.resize(nE);
    } catch (...) {
      return gas::fail(GAS_ERR_NOMEM, "set_graph: host arrays");
    }
    GAS_TRY(gas::build_csr_host(nV, nE, dsts, srcs, e->h_csc_off.data(),
                                csc_src.data(), csc_perm.data()));
    GAS_TRY(gas::build_csr_host(nV, nE, srcs, dsts, csr_off.data(),
                                csr_dst.data(), csr_perm.data()));
    if (have_ed) {
      try {
        ed_csc.resize((size_t)nE * eb);
        ed_csr.resize((size_t)nE * eb);
      } catch (...) {
        return gas::fail(GAS_ERR_NOMEM, "set_graph: edge data");
      }
      const uint8_t *src = (const uint8_t *)edge_data;
      for (int64_t i = 0; i < nE; ++i) {
        memcpy(&ed_csc[i * eb], src + (size_t)csc_perm[i] * eb, eb);
        memcpy(&ed_csr[i * eb], src + (size_t)csr_perm[i] * eb, eb);
      }
    }
  }

  const size_t V = (size_t)nV, E = (size_t)nE;
  GAS_TRY(dalloc(&e->csc_off, V + 1));
  GAS_TRY(dalloc(&e->csr_off, V + 1));
  e->edges_on_host = e->edge_place == GAS_EDGES_HOST;
  if (e->edges_on_host) {
    GAS_TRY(halloc(&e->csc_src, E));
    GAS_TRY(halloc(&e->csr_dst, E));
    if (have_ed) {
      GAS_TRY(halloc((uint8_t **)&e->csc_ed, E * eb));
      GAS_TRY(halloc((uint8_t **)&e->csr_ed, E * eb));
    }
  } else {
    GAS_TRY(dalloc(&e->csc_src, E));
    GAS_TRY(dalloc(&e->csr_dst, E));
    if (have_ed) {
      GAS_TRY(dalloc((uint8_t **)&e->csc_ed, E * eb));
      GAS_TRY(dalloc((uint8_t **)&e->csr_ed, E * eb));
    }
  }
  GAS_TRY(dalloc((uint8_t **)&e->vd, V * e->vbytes));
  GAS_TRY(dalloc(&e->act, V));
  GAS_TRY(dalloc(&e->scan, V + 1));
  GAS_TRY(dalloc(&e->sscan, V + 1));
  GAS_TRY(dalloc(&e->ret, V));
  GAS_TRY(dalloc((uint8_t **)&e->slot, V * e->vbytes));
  GAS_TRY(dalloc((uint8_t **)&e->gres, V * std::max<size_t>(e->gbytes, 4)));
  const size_t nW = (V + 31) / 32;
  GAS_TRY(dalloc(&e->bits, nW));
  // smallest tile is kNT * 2 items (gather values larger than 16 bytes)
  const int64_t min_tile = kNT * 2;
  e->tile_cap = (int32_t)(((int64_t)V + (int64_t)E + min_tile - 1) / min_tile + 1);
  const size_t tv = std::max<size_t>(e->gbytes, 8);
  GAS_TRY(dalloc((uint8_t **)&e->tile_first, (size_t)e->tile_cap * tv));
  GAS_TRY(dalloc((uint8_t **)&e->tile_carry, (size_t)e->tile_cap * tv));
  GAS_TRY(dalloc(&e->tile_a0, (size_t)e->tile_cap));
  GAS_TRY(dalloc(&e->tpart, (size_t)e->tile_cap + 2));
  GAS_TRY(dalloc(&e->dpart, (size_t)e->tile_cap + 2));
  GAS_TRY(dalloc(&e->ppart, (V + kScanBlock - 1) / kScanBlock + 1));
  e->n_cblocks = (int32_t)std::max<size_t>(1, (nW + kCompactBlock - 1) / kCompactBlock);
  GAS_TRY(dalloc(&e->cpart, 2 * (size_t)e->n_cblocks));
  GAS_TRY(dalloc(&e->cnt, 1));

  if (dev_build)
    GAS_TRY(gas::build_graph_device(e, srcs, dsts, have_ed ? edge_data : nullptr,
                                    want_perms ? &csc_perm : nullptr,
                                    want_perms ? &csr_perm : nullptr, stream));
  if (want_perms) {
    // a user program may scatter into its edge data: keep what maps the
    // two device copies onto each other and back to the caller's order
    try {
      std::vector<int32_t> inv((size_t)nE);
      for (int64_t i = 0; i < nE; ++i) inv[csc_perm[i]] = (int32_t)i;
      e->h_csr_to_csc.resize((size_t)nE);
      for (int64_t j = 0; j < nE; ++j) e->h_csr_to_csc[j] = inv[csr_perm[j]];
      e->h_csr_perm = csr_perm;
    } catch (...) {
      return gas::fail(GAS_ERR_NOMEM, "set_graph: edge maps");
    }
    e->host_ed = const_cast<void *>(edge_data);
  }

  // rows of the CSC with in-edges, for the dense slab passes
  std::vector<int32_t> ne_vid, ne_end;
  try {
    ne_vid.reserve(V);
    ne_end.reserve(V);
    for (int32_t v = 0; v < nV; ++v) {
      if (e->h_csc_off[v + 1] > e->h_csc_off[v]) {
        ne_vid.push_back(v);
        ne_end.push_back(e->h_csc_off[v + 1]);
      }
    }
  } catch (...) {
    return gas::fail(GAS_ERR_NOMEM, "set_graph: row lists");
  }
  e->n_ne = (int32_t)ne_vid.size();
  GAS_TRY(dalloc(&e->ne_vid, ne_vid.size()));
  GAS_TRY(dalloc(&e->ne_end, ne_end.size()));
  e->slab_cap = (int32_t)((E + gasdev::kSlabChunk - 1) / gasdev::kSlabChunk + 1);
  GAS_TRY(dalloc(&e->slab_dpart, (size_t)e->slab_cap));
  // the push may cut its queue's edges into chunks as small as 64 edges
  GAS_TRY(dalloc(&e->slab_qpart,
                 (size_t)((E >> gasdev::kSlabChunkMinLog2) + 2)));
  GAS_TRY(dalloc(&e->slab_a0, (size_t)e->slab_cap));
  GAS_TRY(dalloc((uint8_t **)&e->slab_first, (size_t)e->slab_cap * 8));
  GAS_TRY(dalloc((uint8_t **)&e->slab_carry, (size_t)e->slab_cap * 8));
  GAS_TRY(dalloc(&e->slab_fix, (size_t)e->slab_cap));
  GAS_TRY(dalloc(&e->slab_fix_n, 1));
  GAS_TRY(dalloc(&e->trace, GAS_TRACE_CAP));
  GAS_TRY(dalloc(&e->hist, 8));

  cudaStream_t st = S(stream);
  if (!ne_vid.empty()) {
    CUDA_TRY(cudaMemcpyAsync(e->ne_vid, ne_vid.data(), ne_vid.size() * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(e->ne_end, ne_end.data(), ne_end.size() * 4, cudaMemcpyHostToDevice, st));
  }
  if (!dev_build) {
    CUDA_TRY(cudaMemcpyAsync(e->csc_off, e->h_csc_off.data(), (V + 1) * 4,
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(e->csr_off, csr_off.data(), (V + 1) * 4, cudaMemcpyHostToDevice,
                             st));
  }
  if (E && !dev_build) {
    CUDA_TRY(cudaMemcpyAsync(e->csc_src, csc_src.data(), E * 4, cudaMemcpyDefault, st));
    CUDA_TRY(cudaMemcpyAsync(e->csr_dst, csr_dst.data(), E * 4, cudaMemcpyDefault, st));
    if (have_ed) {
      CUDA_TRY(cudaMemcpyAsync(e->csc_ed, ed_csc.data(), E * eb, cudaMemcpyDefault, st));
      CUDA_TRY(cudaMemcpyAsync(e->csr_ed, ed_csr.data(), E * eb, cudaMemcpyDefault, st));
    }
  }
  if (V)
    CUDA_TRY(cudaMemcpyAsync(e->vd, vertex_data, V * e->vbytes, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(e->bits, 0, nW * 4, st));
  CUDA_TRY(cudaMemsetAsync(e->slab_fix_n, 0, sizeof(int32_t), st));
  CUDA_TRY(cudaMemsetAsync(e->hist, 0, 8 * sizeof(int32_t), st));
  CUDA_TRY(cudaMemsetAsync(e->trace, 0, GAS_TRACE_CAP * sizeof(gas_trace_record), st));
  CUDA_TRY(cudaMemsetAsync(e->cnt, 0, sizeof(gas_counters), st));
  CUDA_TRY(cudaMemsetAsync(e->ret, 0, V ? V : 1, st));
  // the host vectors are released at return: wait for the copies
  CUDA_TRY(cudaStreamSynchronize(st));
  e->n_active = 0;
  e->n_edges = 0;
  e->counts_dirty = false;
  e->pending_gather = e->have_gres = e->slots_pending = false;
  e->level = 0;
  e->has_graph = true;
  return GAS_OK;
}

gas_status_t gas_engine_set_active(gas_engine *e, int32_t start, int32_t end,
                                   void *stream) {
  if (!e || !e->has_graph) return gas::fail(GAS_ERR_STATE, "set_active before set_graph");
  if (start < 0 || end < start || end > e->nV)
    return gas::fail(GAS_ERR_INVALID, "set_active: [%d,%d) outside [0,%d)", start, end, e->nV);
  GAS_TRY(flush_pending_gather(e, stream));
  if (e->slots_pending) {
    // an applied but not yet scattered iteration: make its vertex data visible
    k_commit<<<grid_for(e->n_active, kNT, 8 * e->num_sms), kNT, 0, S(stream)>>>(
        e->act, e->cnt, (const uint8_t *)e->slot, (uint8_t *)e->vd, (int)e->vbytes);
    CUDA_TRY(cudaGetLastError());
    e->slots_pending = false;
  }
  const int n = end - start;
  k_set_range<<<grid_for((int64_t)n + 1, kNT, 8 * e->num_sms), kNT, 0, S(stream)>>>(
      start, n, e->csc_off, e->act, e->scan, e->cnt);
  CUDA_TRY(cudaGetLastError());
  e->n_active = n;
  e->n_edges = e->h_csc_off[end] - e->h_csc_off[start];
  e->counts_dirty = false;
  e->active_full = start == 0 && end == e->nV;
  return GAS_OK;
}

gas_status_t gas_engine_count_active(gas_engine *e, int32_t *n_active) {
  if (!e || !n_active) return gas::fail(GAS_ERR_INVALID, "null argument");
  if (e->counts_dirty) GAS_TRY(sync_counts(e, nullptr));
  *n_active = e->n_active;
  return GAS_OK;
}

gas_status_t gas_engine_gather(gas_engine *e, int32_t have_gather, void *stream) {
  (void)stream;
  if (!e || !e->has_graph) return gas::fail(GAS_ERR_STATE, "gather before set_graph");
  if (e->prog == GAS_PROG_USER)
    return gas::fail(GAS_ERR_UNSUPPORTED, "user programs gather through gpugas.h");
  if (e->counts_dirty) GAS_TRY(sync_counts(e, stream));
  e->pending_gather = have_gather != 0 && e->prog != GAS_PROG_BFS;
  e->have_gres = false;
  return GAS_OK;
}

gas_status_t gas_engine_apply(gas_engine *e, void *stream) {
  if (!e || !e->has_graph) return gas::fail(GAS_ERR_STATE, "apply before set_graph");
  if (e->prog == GAS_PROG_USER)
    return gas::fail(GAS_ERR_UNSUPPORTED, "user programs apply through gpugas.h");
  if (e->counts_dirty) GAS_TRY(sync_counts(e, stream));
  if (e->n_active == 0) return GAS_OK;
  if (e->pending_gather) {
    e->pending_gather = false;
    GAS_TRY(builtin_gather(e, /*fuse=*/true, false, stream));
    e->slots_pending = true;
    return GAS_OK;
  }
  return builtin_apply_only(e, stream);
}

gas_status_t gas_engine_scatter_activate(gas_engine *e, int32_t have_scatter,
                                         void *stream) {
  (void)have_scatter;
  if (!e || !e->has_graph) return gas::fail(GAS_ERR_STATE, "scatter before set_graph");
  if (e->counts_dirty) GAS_TRY(sync_counts(e, stream));
  GAS_TRY(flush_pending_gather(e, stream));
  return scatter_common(e, stream);
}

gas_status_t gas_engine_next_iter(gas_engine *e, int32_t *n_active, void *stream) {
  if (!e || !e->has_graph) return gas::fail(GAS_ERR_STATE, "next_iter before set_graph");
  if (e->counts_dirty) GAS_TRY(sync_counts(e, stream));
  if (n_active) *n_active = e->n_active;
  return GAS_OK;
}

gas_status_t gas_engine_get_results(gas_engine *e, void *stream) {
  if (!e || !e->has_graph) return gas::fail(GAS_ERR_STATE, "get_results before set_graph");
  GAS_TRY(flush_pending_gather(e, stream));
  if (e->slots_pending) {
    k_commit<<<grid_for(e->n_active, kNT, 8 * e->num_sms), kNT, 0, S(stream)>>>(
        e->act, e->cnt, (const uint8_t *)e->slot, (uint8_t *)e->vd, (int)e->vbytes);
    CUDA_TRY(cudaGetLastError());
    e->slots_pending = false;
  }
  if (e->nV && e->host_vd)
    CUDA_TRY(cudaMemcpyAsync(e->host_vd, e->vd, (size_t)e->nV * e->vbytes,
                             cudaMemcpyDeviceToHost, S(stream)));
  CUDA_TRY(cudaStreamSynchronize(S(stream)));
  if (e->edges_dirty && e->host_ed && e->nE) {
    // edge data a user scatter changed, back into the caller's order
    const size_t eb = e->ebytes;
    std::vector<uint8_t> tmp;
    try {
      tmp.resize((size_t)e->nE * eb);
    } catch (...) {
      return gas::fail(GAS_ERR_NOMEM, "get_results: edge data");
    }
    CUDA_TRY(cudaMemcpyAsync(tmp.data(), e->csr_ed, tmp.size(), cudaMemcpyDefault,
                             S(stream)));
    CUDA_TRY(cudaStreamSynchronize(S(stream)));
    uint8_t *dst = static_cast<uint8_t *>(e->host_ed);
    for (int32_t j = 0; j < e->nE; ++j)
      memcpy(dst + (size_t)e->h_csr_perm[j] * eb, &tmp[(size_t)j * eb], eb);
    e->edges_dirty = false;
  }
  return GAS_OK;
}

gas_status_t gas_engine_set_edge_placement(gas_engine *e, gas_edge_placement_t where) {
  if (!e) return gas::fail(GAS_ERR_INVALID, "null engine");
  if (where != GAS_EDGES_DEVICE && where != GAS_EDGES_HOST)
    return gas::fail(GAS_ERR_INVALID, "unknown edge placement %d", (int)where);
  e->edge_place = where;
  return GAS_OK;
}

gas_status_t gas_engine_download_graph(gas_engine *e, int32_t *csc_off, int32_t *csc_src,
                                       int32_t *csr_off, int32_t *csr_dst, void *csc_ed,
                                       void *csr_ed, void *stream) {
  if (!e || !e->has_graph) return gas::fail(GAS_ERR_STATE, "no graph");
  const size_t V1 = (size_t)e->nV + 1, E = (size_t)e->nE, eb = e->ebytes;
  cudaStream_t st = S(stream);
  const struct {
    void *dst;
    const void *src;
    size_t bytes;
  } cp[] = {{csc_off, e->csc_off, V1 * 4}, {csc_src, e->csc_src, E * 4},
            {csr_off, e->csr_off, V1 * 4}, {csr_dst, e->csr_dst, E * 4},
            {csc_ed, e->csc_ed, E * eb}, {csr_ed, e->csr_ed, E * eb}};
  for (const auto &c : cp)
    if (c.dst && c.src && c.bytes)
      CUDA_TRY(cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDefault, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return GAS_OK;
}

gas_status_t gas_engine_prepare_scatter(gas_engine *e, const int32_t **csr_to_csc,
                                        void *stream) {
  if (!e || !e->has_graph) return gas::fail(GAS_ERR_STATE, "scatter before set_graph");
  if (e->prog != GAS_PROG_USER)
    return gas::fail(GAS_ERR_UNSUPPORTED, "prepare_scatter is for user programs");
  if (e->counts_dirty) GAS_TRY(sync_counts(e, stream));
  if (e->slots_pending) {
    k_commit<<<grid_for(e->n_active, kNT, 8 * e->num_sms), kNT, 0, S(stream)>>>(
        e->act, e->cnt, (const uint8_t *)e->slot, (uint8_t *)e->vd, (int)e->vbytes);
    CUDA_TRY(cudaGetLastError());
    e->slots_pending = false;
  }
  const bool have = e->csr_ed && e->nE > 0 && !e->h_csr_to_csc.empty();
  if (have && !e->csr_to_csc) {
    GAS_TRY(dalloc(&e->csr_to_csc, (size_t)e->nE));
    CUDA_TRY(cudaMemcpyAsync(e->csr_to_csc, e->h_csr_to_csc.data(), (size_t)e->nE * 4,
                             cudaMemcpyHostToDevice, S(stream)));
  }
  if (csr_to_csc) *csr_to_csc = have ? e->csr_to_csc : nullptr;
  e->edges_dirty = e->edges_dirty || have;
  return GAS_OK;
}

gas_status_t gas_engine_set_iteration(gas_engine *e, int32_t level) {
  if (!e) return gas::fail(GAS_ERR_INVALID, "null engine");
  e->level = level;
  return GAS_OK;
}

gas_status_t gas_engine_run(gas_engine *e, int32_t *iterations, void *stream) {
  if (!e || !e->has_graph) return gas::fail(GAS_ERR_STATE, "run before set_graph");
  if (e->prog == GAS_PROG_USER)
    return gas::fail(GAS_ERR_UNSUPPORTED, "user programs run through gpugas.h");
  int32_t it = 0, n = 0;
  GAS_TRY(gas_engine_count_active(e, &n));
  while (n) {
    GAS_TRY(gas_engine_gather(e, 1, stream));
    GAS_TRY(gas_engine_apply(e, stream));
    GAS_TRY(gas_engine_scatter_activate(e, 1, stream));
    GAS_TRY(gas_engine_next_iter(e, &n, stream));
    ++it;
    if (e->prog == GAS_PROG_BFS) e->level = it;
  }
  if (iterations) *iterations = it;
  return GAS_OK;
}

gas_status_t gas_engine_vertex_data_device(gas_engine *e, void **ptr) {
  if (!e || !ptr || !e->has_graph) return gas::fail(GAS_ERR_STATE, "no graph");
  *ptr = e->vd;
  return GAS_OK;
}

gas_status_t gas_engine_upload_vertex_data(gas_engine *e, const void *host,
                                           void *stream) {
  if (!e || !host || !e->has_graph) return gas::fail(GAS_ERR_STATE, "no graph");
  CUDA_TRY(cudaMemcpyAsync(e->vd, host, (size_t)e->nV * e->vbytes,
                           cudaMemcpyDefault, S(stream)));
  return GAS_OK;
}

gas_status_t gas_engine_download_vertex_data(gas_engine *e, void *host,
                                             void *stream) {
  if (!e || !host || !e->has_graph) return gas::fail(GAS_ERR_STATE, "no graph");
  CUDA_TRY(cudaMemcpyAsync(host, e->vd, (size_t)e->nV * e->vbytes,
                           cudaMemcpyDefault, S(stream)));
  CUDA_TRY(cudaStreamSynchronize(S(stream)));
  return GAS_OK;
}

gas_status_t gas_engine_download_vertex_data_async(gas_engine *e, void *dst,
                                                   void *stream) {
  if (!e || !dst || !e->has_graph) return gas::fail(GAS_ERR_STATE, "no graph");
  CUDA_TRY(cudaMemcpyAsync(dst, e->vd, (size_t)e->nV * e->vbytes, cudaMemcpyDefault,
                           S(stream)));
  return GAS_OK;
}

gas_status_t gas_engine_view_get(gas_engine *e, gas_engine_view *v) {
  if (!e || !v || !e->has_graph) return gas::fail(GAS_ERR_STATE, "no graph");
  v->nV = e->nV;
  v->nE = e->nE;
  v->csc_off = e->csc_off;
  v->csc_src = e->csc_src;
  v->csc_ed = e->csc_ed;
  v->csr_off = e->csr_off;
  v->csr_dst = e->csr_dst;
  v->csr_ed = e->csr_ed;
  v->vertex_data = e->vd;
  v->active = e->act;
  v->active_scan = e->scan;
  v->apply_ret = e->ret;
  v->slot = e->slot;
  v->gather_tmp = e->gres;
  v->tile_first = e->tile_first;
  v->tile_carry = e->tile_carry;
  v->tile_a0 = e->tile_a0;
  v->tile_part = e->tpart;
  v->tile_cap = e->tile_cap;
  v->num_sms = e->num_sms;
  v->counters = e->cnt;
  return GAS_OK;
}

gas_status_t gas_engine_note_applied(gas_engine *e, int32_t wrote_slots) {
  if (!e) return gas::fail(GAS_ERR_INVALID, "null engine");
  e->slots_pending = wrote_slots != 0;
  return GAS_OK;
}

gas_status_t gas_engine_set_profiling(gas_engine *e, int32_t on) {
  if (!e) return gas::fail(GAS_ERR_INVALID, "null engine");
  if (on) {
    for (int i = 0; i < 2; ++i)
      if (!e->prof_ev[i]) CUDA_TRY(cudaEventCreate(&e->prof_ev[i]));
  }
  e->profiling = on != 0;
  return GAS_OK;
}

gas_status_t gas_engine_get_profile(gas_engine *e, gas_kernel_profile *out,
                                    int32_t reset) {
  if (!e || !out) return gas::fail(GAS_ERR_INVALID, "null argument");
  *out = e->prof;
  if (reset) e->prof = gas_kernel_profile{};
  return GAS_OK;
}

gas_status_t gas_engine_read_counters(gas_engine *e, gas_counters *out,
                                      void *stream) {
  if (!e || !out || !e->has_graph) return gas::fail(GAS_ERR_STATE, "no graph");
  GAS_TRY(sync_counts(e, stream));
  *out = *e->h_cnt;
  return GAS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Schedules, precision PageRank (gas_engine_run_schedule and friends) live in
// gas_runs.cu; they reach the engine through these accessors.
// ---------------------------------------------------------------------------
namespace gas {

void prof_begin(gas_engine *e, cudaStream_t s, int kind, int64_t bytes) {
  if (!e->profiling || e->in_graph || !e->prof_ev[0]) return;
  cudaEventRecord(e->prof_ev[0], s);
  e->prof_kind = kind;
  e->prof_bytes_pending = bytes;
}

void prof_end(gas_engine *e, cudaStream_t s) {
  if (e->prof_kind < 0) return;
  cudaEventRecord(e->prof_ev[1], s);
}

void prof_collect(gas_engine *e) {
  if (e->prof_kind < 0) return;
  float ms = 0.f;
  if (cudaEventSynchronize(e->prof_ev[1]) == cudaSuccess &&
      cudaEventElapsedTime(&ms, e->prof_ev[0], e->prof_ev[1]) == cudaSuccess) {
    gas_kernel_profile &p = e->prof;
    if (e->prof_kind == kProfPush) {
      p.push_ms += ms; p.push_bytes += e->prof_bytes_pending; ++p.push_launches;
    } else if (e->prof_kind == kProfPull) {
      p.pull_ms += ms; p.pull_bytes += e->prof_bytes_pending; ++p.pull_launches;
    } else {
      p.pagerank_ms += ms; p.pagerank_bytes += e->prof_bytes_pending; ++p.pagerank_launches;
    }
  }
  e->prof_kind = -1;
}

gas_status_t engine_scatter(gas_engine *e, void *stream) {
  return scatter_common(e, stream);
}
gas_status_t engine_sync_counts(gas_engine *e, void *stream) {
  return sync_counts(e, stream);
}
int engine_grid(int64_t work_items, int per_block, int cap) {
  return grid_for(work_items, per_block, cap);
}
int engine_partition_grid(gas_engine *e, int64_t items, int tile) {
  const int cap = 2 * e->num_sms;
  if (e->capturing || items < 0) return cap;
  return grid_for((items + tile - 1) / tile + 1, 256, cap);
}

gas_status_t engine_gather_apply(gas_engine *e, void *stream) {
  GAS_TRY(builtin_gather(e, true, false, stream));
  e->slots_pending = true;
  return GAS_OK;
}
gas_status_t engine_apply_only(gas_engine *e, void *stream) {
  return builtin_apply_only(e, stream);
}
gas_status_t engine_commit(gas_engine *e, void *stream) {
  const int g = e->capturing ? 8 * e->num_sms
                             : grid_for(e->n_active, kNT, 8 * e->num_sms);
  k_commit<<<g, kNT, 0, S(stream)>>>(e->act, e->cnt, (const uint8_t *)e->slot,
                                     (uint8_t *)e->vd, (int)e->vbytes);
  CUDA_TRY(cudaGetLastError());
  e->slots_pending = false;
  return GAS_OK;
}

gas_status_t engine_generic_iteration(gas_engine *e, bool ordered, void *stream) {
  if (e->prog == GAS_PROG_BFS) {
    GAS_TRY(builtin_apply_only(e, stream));
  } else {
    GAS_TRY(builtin_gather(e, true, ordered, stream));
    e->slots_pending = true;
  }
  return scatter_common(e, stream);
}
}  // namespace gas
