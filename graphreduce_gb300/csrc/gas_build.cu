// gas_build.cu -- CSR and CSC construction on the device (the work of
// edgeListToCSR / edgeListToCSC, util.cuh:80-121, done by setGraph at
// gpugas.h:1314-1503, moved off the host).
//
// The edge list goes to the device once; each of the two orders is a stable
// LSD radix sort of the edge indices by key (source for CSR, destination for
// CSC), 4 bits per pass over the bits the vertex count needs, followed by
// row offsets read off the sorted keys and gathers of the other endpoint and
// of the edge data.  Stability makes the result identical to the host build
// (edges of one key keep their edge-list order).
//
// One pass over n keys: k_rs_hist counts the digits of every 2048-key tile
// (digit-major table [16][tiles]); an exclusive scan of the table gives every
// (digit, tile) its output base; k_rs_scatter ranks the tile's keys stably in
// shared memory (per-thread digit counts, one block scan) and writes them out
// digit run by digit run, so the stores of a run are contiguous.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gas.h"
#include "gas_engine_impl.h"
#include "gas_internal.h"

namespace {

inline cudaStream_t S(void *s) { return (cudaStream_t)s; }

constexpr int kRBins = 16;                   // 4-bit digits
constexpr int kRThreads = 256;
constexpr int kRItems = 8;
constexpr int kRTile = kRThreads * kRItems;  // keys per tile
constexpr int kScanItems = 16;
constexpr int kScanTile = kRThreads * kScanItems;  // entries per scan block

__device__ __forceinline__ int rs_digit(int32_t k, int shift) {
  return (int)(((uint32_t)k >> shift) & (kRBins - 1));
}

// Exclusive CTA scan of one int per thread (kRThreads threads).
__device__ __forceinline__ int cta_scan_excl(int v, int *total) {
  __shared__ int s_w[kRThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int o = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += o;
  }
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  int pre = 0, tot = 0;
  for (int w = 0; w < kRThreads / 32; ++w) {
    if (w < warp) pre += s_w[w];
    tot += s_w[w];
  }
  __syncthreads();
  *total = tot;
  return pre + x - v;
}

// Ids outside [0, nV) put (index + 1) of the largest such edge in *bad.
__global__ void k_check_ids(const int32_t *a, const int32_t *b, int n, int nV, int32_t *bad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t x = a[i], y = b[i];
    if (x < 0 || x >= nV || y < 0 || y >= nV) atomicMax(bad, i + 1);
  }
}

__global__ void __launch_bounds__(kRThreads)
    k_rs_hist(const int32_t *keys, int n, int shift, int ntiles, int32_t *hist) {
  __shared__ int c[kRBins];
  if (threadIdx.x < kRBins) c[threadIdx.x] = 0;
  __syncthreads();
  const int base = blockIdx.x * kRTile;
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < kRItems; ++j) {
    const int i = base + j * kRThreads + threadIdx.x;
    const int d = i < n ? rs_digit(keys[i], shift) : kRBins;
    const unsigned same = __match_any_sync(0xffffffffu, d);
    if (d < kRBins && lane == __ffs(same) - 1) atomicAdd(&c[d], __popc(same));
  }
  __syncthreads();
  if (threadIdx.x < kRBins) hist[threadIdx.x * ntiles + blockIdx.x] = c[threadIdx.x];
}

__global__ void __launch_bounds__(kRThreads)
    k_rs_scatter(const int32_t *kin, const int32_t *vin, int32_t *kout, int32_t *vout, int n,
                 int shift, int ntiles, const int32_t *ghist) {
  __shared__ int32_t s_key[kRTile];
  __shared__ int32_t s_val[kRTile];
  __shared__ int32_t s_cnt[kRBins * kRThreads];  // [digit][thread]
  __shared__ int32_t s_dstart[kRBins], s_gbase[kRBins];
  const int t = threadIdx.x;
  const int base = blockIdx.x * kRTile;
  const int nvalid = min(kRTile, n - base);
  // striped, coalesced load
#pragma unroll
  for (int j = 0; j < kRItems; ++j) {
    const int i = j * kRThreads + t;
    s_key[i] = i < nvalid ? kin[base + i] : -1;
    s_val[i] = i < nvalid ? (vin ? vin[base + i] : base + i) : -1;
  }
  for (int k = t; k < kRBins * kRThreads; k += kRThreads) s_cnt[k] = 0;
  __syncthreads();
  // blocked view: thread t owns tile items [t * kRItems, (t + 1) * kRItems),
  // so thread order is tile order and the ranking below is stable
  int32_t myk[kRItems], myv[kRItems];
#pragma unroll
  for (int j = 0; j < kRItems; ++j) {
    myk[j] = s_key[t * kRItems + j];
    myv[j] = s_val[t * kRItems + j];
    if (myk[j] >= 0) ++s_cnt[rs_digit(myk[j], shift) * kRThreads + t];
  }
  __syncthreads();
  // exclusive scan of s_cnt in digit-major order; thread t scans entries
  // [t * 16, t * 16 + 16) after a CTA scan of the 16-entry sums
  int run = 0;
#pragma unroll
  for (int k = 0; k < kRBins; ++k) run += s_cnt[t * kRBins + k];
  int total;
  int pre = cta_scan_excl(run, &total);
#pragma unroll
  for (int k = 0; k < kRBins; ++k) {
    const int c = s_cnt[t * kRBins + k];
    s_cnt[t * kRBins + k] = pre;
    pre += c;
  }
  __syncthreads();
  if (t < kRBins) {
    s_dstart[t] = s_cnt[t * kRThreads];  // first tile position of digit t
    s_gbase[t] = ghist[t * ntiles + blockIdx.x];
  }
  __syncthreads();
  int pos[kRItems];
#pragma unroll
  for (int j = 0; j < kRItems; ++j)
    pos[j] = myk[j] >= 0 ? s_cnt[rs_digit(myk[j], shift) * kRThreads + t]++ : -1;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kRItems; ++j) {
    if (pos[j] >= 0) {
      s_key[pos[j]] = myk[j];
      s_val[pos[j]] = myv[j];
    }
  }
  __syncthreads();
  // striped store: consecutive tile positions of one digit are consecutive
  // output positions
#pragma unroll
  for (int j = 0; j < kRItems; ++j) {
    const int p = j * kRThreads + t;
    if (p < nvalid) {
      const int32_t k = s_key[p];
      const int d = rs_digit(k, shift);
      const int g = s_gbase[d] + (p - s_dstart[d]);
      kout[g] = k;
      vout[g] = s_val[p];
    }
  }
}

// Generic exclusive scan of n int32 in place: per-block sums, one block over
// the sums, per-block downsweep.
__global__ void __launch_bounds__(kRThreads)
    k_scan_reduce(const int32_t *a, int n, int32_t *part) {
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) s += base + k < n ? a[base + k] : 0;
  int total;
  cta_scan_excl(s, &total);
  if (threadIdx.x == 0) part[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kRThreads) k_scan_spine(int32_t *part, int nb) {
  __shared__ int s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < nb; b0 += kRThreads) {
    const int i = b0 + threadIdx.x;
    const int v = i < nb ? part[i] : 0;
    int total;
    const int e = cta_scan_excl(v, &total);
    const int c = s_carry;
    if (i < nb) part[i] = c + e;
    __syncthreads();
    if (threadIdx.x == 0) s_carry = c + total;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kRThreads)
    k_scan_down(int32_t *a, int n, const int32_t *part) {
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = base + k < n ? a[base + k] : 0;
    s += v[k];
  }
  int total;
  int pre = cta_scan_excl(s, &total) + part[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) a[base + k] = pre;
    pre += v[k];
  }
}

// Row offsets from sorted keys: off[v] = first position with key >= v.
__global__ void k_offsets_from_sorted(const int32_t *keys, int n, int nV, int32_t *off) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
    const int lo = i == 0 ? 0 : keys[i - 1] + 1;  // first row starting here
    const int hi = i == n ? nV : keys[i];          // last row starting here
    for (int v = lo; v <= hi; ++v) off[v] = i;
  }
}

__global__ void k_gather_i32(const int32_t *src, const int32_t *perm, int n, int32_t *out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = src[perm[i]];
}

// Edge data of w 32-bit words per edge, or of eb bytes when eb % 4 != 0.
__global__ void k_gather_rec(const uint8_t *src, const int32_t *perm, int n, int eb,
                             uint8_t *out) {
  const size_t total = (size_t)n * eb;
  if (eb % 4 == 0) {
    const int w = eb / 4;
    const uint32_t *s = reinterpret_cast<const uint32_t *>(src);
    uint32_t *o = reinterpret_cast<uint32_t *>(out);
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < (size_t)n * w;
         k += (size_t)gridDim.x * blockDim.x)
      o[k] = s[(size_t)perm[k / w] * w + k % w];
  } else {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
         k += (size_t)gridDim.x * blockDim.x)
      out[k] = src[(size_t)perm[k / eb] * eb + k % eb];
  }
}

template <class T>
gas_status_t tmp_alloc(T **p, size_t n) {
  *p = nullptr;
  cudaError_t ce = cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T));
  if (ce != cudaSuccess)
    return gas::fail(GAS_ERR_NOMEM, "device graph build: %s", cudaGetErrorString(ce));
  return GAS_OK;
}

struct Scratch {
  int32_t *a = nullptr, *b = nullptr, *c = nullptr, *d = nullptr, *e = nullptr, *f = nullptr;
  int32_t *hist = nullptr, *part = nullptr, *bad = nullptr;
  uint8_t *ed = nullptr;
  ~Scratch() {
    for (void *p : {(void *)a, (void *)b, (void *)c, (void *)d, (void *)e, (void *)f,
                    (void *)hist, (void *)part, (void *)bad, (void *)ed})
      if (p) cudaFree(p);
  }
};

gas_status_t scan_excl(int32_t *a, int n, int32_t *part, cudaStream_t s) {
  if (n <= 0) return GAS_OK;
  const int nb = (n + kScanTile - 1) / kScanTile;
  k_scan_reduce<<<nb, kRThreads, 0, s>>>(a, n, part);
  k_scan_spine<<<1, kRThreads, 0, s>>>(part, nb);
  k_scan_down<<<nb, kRThreads, 0, s>>>(a, n, part);
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

// Stable sort of the edge indices by keys[] (values 0..n-1 enter with the
// first pass), bits >= 1.  Sorted keys end in *kres, the permutation in
// *vres (two of the four work buffers).
gas_status_t radix_sort(const int32_t *keys, int n, int bits, int32_t *k0, int32_t *v0,
                        int32_t *k1, int32_t *v1, int32_t *hist, int32_t *part,
                        int32_t **kres, int32_t **vres, cudaStream_t s) {
  const int ntiles = (n + kRTile - 1) / kRTile;
  const int passes = (bits + 3) / 4;
  const int32_t *kin = keys;
  const int32_t *vin = nullptr;
  int32_t *ko = k0, *vo = v0, *ka = k1, *va = v1;
  for (int p = 0; p < passes; ++p) {
    const int shift = 4 * p;
    k_rs_hist<<<ntiles, kRThreads, 0, s>>>(kin, n, shift, ntiles, hist);
    GAS_TRY(scan_excl(hist, kRBins * ntiles, part, s));
    k_rs_scatter<<<ntiles, kRThreads, 0, s>>>(kin, vin, ko, vo, n, shift, ntiles, hist);
    CUDA_TRY(cudaGetLastError());
    kin = ko;
    vin = vo;
    std::swap(ko, ka);
    std::swap(vo, va);
  }
  *kres = const_cast<int32_t *>(kin);
  *vres = const_cast<int32_t *>(vin);
  return GAS_OK;
}

}  // namespace

namespace gas {

bool device_build_for(int64_t n_edges) {
  const char *v = getenv("GAS_GRAPH_BUILD");
  if (v && strcmp(v, "host") == 0) return false;
  if (v && strcmp(v, "device") == 0) return true;
  return n_edges >= (1 << 20);
}

gas_status_t build_graph_device(gas_engine *e, const int32_t *srcs, const int32_t *dsts,
                                const void *edge_data, std::vector<int32_t> *csc_perm,
                                std::vector<int32_t> *csr_perm, void *stream) {
  cudaStream_t s = S(stream);
  const int nV = e->nV, n = e->nE;
  const size_t eb = e->ebytes;
  const bool have_ed = edge_data && eb > 0 && e->csc_ed;
  Scratch w;
  const int ntiles = (n + kRTile - 1) / kRTile;
  const int hist_n = kRBins * std::max(ntiles, 1);
  const int nparts = (std::max(hist_n, nV + 1) + kScanTile - 1) / kScanTile + 1;
  GAS_TRY(tmp_alloc(&w.a, n));  // src
  GAS_TRY(tmp_alloc(&w.b, n));  // dst
  GAS_TRY(tmp_alloc(&w.c, n));
  GAS_TRY(tmp_alloc(&w.d, n));
  GAS_TRY(tmp_alloc(&w.e, n));
  GAS_TRY(tmp_alloc(&w.f, n));
  GAS_TRY(tmp_alloc(&w.hist, hist_n));
  GAS_TRY(tmp_alloc(&w.part, nparts));
  GAS_TRY(tmp_alloc(&w.bad, 1));
  if (have_ed) GAS_TRY(tmp_alloc(&w.ed, (size_t)n * eb));
  if (n) {
    CUDA_TRY(cudaMemcpyAsync(w.a, srcs, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(w.b, dsts, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    if (have_ed)
      CUDA_TRY(cudaMemcpyAsync(w.ed, edge_data, (size_t)n * eb, cudaMemcpyHostToDevice, s));
  }
  CUDA_TRY(cudaMemsetAsync(w.bad, 0, 4, s));
  const int grid = 8 * e->num_sms;
  if (n) k_check_ids<<<grid, 256, 0, s>>>(w.a, w.b, n, nV, w.bad);
  int32_t bad = 0;
  CUDA_TRY(cudaMemcpyAsync(&bad, w.bad, 4, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (bad) {
    const int i = bad - 1;
    return fail(GAS_ERR_INVALID, "edge %d: (%d, %d) outside [0,%d)", i, srcs[i], dsts[i], nV);
  }
  int bits = 1;
  while (bits < 31 && (1LL << bits) < nV) ++bits;  // keys are < nV <= 2^bits
  // order 0: CSC (key dst, other endpoint src); order 1: CSR (key src)
  for (int order = 0; order < 2; ++order) {
    const int32_t *key = order == 0 ? w.b : w.a;
    const int32_t *other = order == 0 ? w.a : w.b;
    int32_t *off = order == 0 ? e->csc_off : e->csr_off;
    std::vector<int32_t> *perm_out = order == 0 ? csc_perm : csr_perm;
    int32_t *ks = nullptr, *vs = nullptr;
    if (n) GAS_TRY(radix_sort(key, n, bits, w.c, w.d, w.e, w.f, w.hist, w.part, &ks, &vs, s));
    k_offsets_from_sorted<<<grid, 256, 0, s>>>(ks, n, nV, off);
    if (n) {
      k_gather_i32<<<grid, 256, 0, s>>>(other, vs, n, order == 0 ? e->csc_src : e->csr_dst);
      if (have_ed)
        k_gather_rec<<<grid, 256, 0, s>>>(w.ed, vs, n, (int)eb,
                                          (uint8_t *)(order == 0 ? e->csc_ed : e->csr_ed));
    }
    CUDA_TRY(cudaGetLastError());
    if (perm_out) {
      perm_out->resize(n);
      if (n)
        CUDA_TRY(cudaMemcpyAsync(perm_out->data(), vs, (size_t)n * 4, cudaMemcpyDeviceToHost,
                                 s));
    }
    // the next order reuses the work buffers
    CUDA_TRY(cudaStreamSynchronize(s));
  }
  e->h_csc_off.resize((size_t)nV + 1);
  CUDA_TRY(cudaMemcpyAsync(e->h_csc_off.data(), e->csc_off, ((size_t)nV + 1) * 4,
                           cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return GAS_OK;
}

}  // namespace gas
