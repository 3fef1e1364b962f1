// gas_noalloc.cu -- a PageRank step that allocates no memory.
//
// Some callers cannot allocate device memory at the moment they run graph
// work: code running inside a memory pool or arena that owns every byte of
// the device, a host process that has handed the device's memory budget to
// another runtime, or a service that must not allocate on its request path
// (cudaMalloc synchronises the device and can fail under fragmentation).
// They hand this entry point their graph and their rank vectors; the
// kernel's own scratch (merge-path tile boundaries, per-tile carries and
// per-CTA residual partials) lives in one file-scope device array of fixed
// size, so the call makes no allocation of any kind.
//
// The step is the precision-form PageRank update that
// gas_engine_pagerank_precision iterates:
//   rank_out[v] = (1-d)/N + d * sum_{u->v} rank_in[u] / out_degree[u]
// with a two-sum compensated FP32 fold per vertex and the FP64 L1 residual
// sum_v |rank_out[v] - rank_in[v]| written to *l1_out.
//
// Limits and sharing:
//   * nV + nE <= GAS_NOALLOC_MAX_ITEMS (2^29); larger graphs are rejected
//     with GAS_ERR_TOO_LARGE before any work is issued;
//   * the scratch array (kScratchBytes, about 6.3 MB) belongs to this
//     file's module.  Under CUDA's lazy module loading (the default since
//     CUDA 12.2) the module, and with it the array, is loaded on a device
//     the first time this entry point runs there; that first call therefore
//     does reserve the 6.3 MB.  A caller whose pool will own every byte of
//     the device makes one call first (nV = nE = 0 with a device l1_out is
//     enough), or runs with CUDA_MODULE_LOADING=EAGER, before the pool takes
//     the device; from then on the array stays reserved until the process
//     exits and calls allocate nothing;
//   * every call shares it and it keeps the previous call's contents: each
//     call rewrites every scratch word it reads (the per-CTA residual slots
//     are cleared first), but two calls whose kernels overlap on the GPU --
//     on different streams, or from different host threads -- race on it and
//     give wrong results; serialise them on one stream;
//   * every call looks up the array's device address (cudaGetSymbolAddress)
//     with the calling thread's device current, so the address stays right
//     after cudaDeviceReset reloads the module; make the first call on a
//     device before capturing work into a CUDA graph, since that one loads
//     the module.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "gas.h"
#include "gas_device.cuh"
#include "gas_internal.h"

using gasdev::kNT;
using gasdev::SegSource;

namespace {

struct NaVal {
  float s, c;
};

constexpr int kTile = gasdev::TileShape<sizeof(NaVal)>::kTile;  // 2048 items
constexpr int64_t kMaxTiles = (int64_t)1 << 18;
constexpr int kMaxCtas = 4096;  // residual partials: tile CTAs + fixup CTAs

// scratch layout (bytes)
constexpr size_t kPartOff = 0;
constexpr size_t kPartBytes = (size_t)(kMaxTiles + 2) * sizeof(int32_t);
constexpr size_t kFirstOff = (kPartOff + kPartBytes + 255) / 256 * 256;
constexpr size_t kFirstBytes = (size_t)kMaxTiles * sizeof(NaVal);
constexpr size_t kCarryOff = kFirstOff + kFirstBytes;
constexpr size_t kCarryBytes = (size_t)kMaxTiles * sizeof(NaVal);
constexpr size_t kA0Off = kCarryOff + kCarryBytes;
constexpr size_t kA0Bytes = (size_t)kMaxTiles * sizeof(int32_t);
constexpr size_t kL1Off = (kA0Off + kA0Bytes + 255) / 256 * 256;
constexpr size_t kL1Bytes = (size_t)kMaxCtas * sizeof(double);
constexpr size_t kScratchBytes = kL1Off + kL1Bytes;

static_assert(GAS_NOALLOC_MAX_ITEMS == kMaxTiles * kTile,
              "header limit must match the scratch array");

// The scratch.  In host code this name is only a stand-in for the device
// array: host code passes the address cudaGetSymbolAddress returns.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the scratch on the calling thread's current device.
// Looked up on every call (a table lookup once the module is loaded), so a
// context that was reset and created again never sees a stale address.
gas_status_t scratch_address(unsigned char **out) {
  void *p = nullptr;
  const cudaError_t ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (ce != cudaSuccess || !p)
    return gas::fail(GAS_ERR_CUDA, "pagerank_step_noalloc: scratch address: %s",
                     cudaGetErrorString(ce));
  *out = static_cast<unsigned char *>(p);
  return GAS_OK;
}

__device__ __forceinline__ NaVal na_two_sum(const NaVal &a, const NaVal &b) {
  const float s = __fadd_rn(a.s, b.s);
  const float bp = __fsub_rn(s, a.s);
  const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bp)), __fsub_rn(b.s, bp));
  return NaVal{s, __fadd_rn(__fadd_rn(a.c, b.c), err)};
}

struct NaPol {
  typedef NaVal Val;
  const int32_t *csc_src;
  const int32_t *out_degree;
  const float *rank_in;
  float *rank_out;
  float base;
  float damping;
  double l1;
  __device__ Val zero() const { return NaVal{0.0f, 0.0f}; }
  __device__ __forceinline__ Val reduce(const Val &a, const Val &b) const {
    return na_two_sum(a, b);
  }
  __device__ __forceinline__ Val map(int, int, int pos) const {
    const int u = __ldg(csc_src + pos);
    const int deg = __ldg(out_degree + u);
    return NaVal{deg ? __fdiv_rn(__ldg(rank_in + u), (float)deg) : 0.0f, 0.0f};
  }
  __device__ __forceinline__ void emit(int, int v, const Val &g) {
    const float r = __fadd_rn(base, __fmul_rn(damping, __fadd_rn(g.s, g.c)));
    rank_out[v] = r;
    l1 += fabs((double)r - (double)rank_in[v]);
  }
};

__device__ __forceinline__ void na_block_sum(double v, double *out) {
  __shared__ double s_w[kNT / 32];
  for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kNT / 32; ++w) t += s_w[w];
    *out = t;
  }
}

__global__ void k_na_clear(double *l1_part, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    l1_part[i] = 0.0;
}

__global__ void __launch_bounds__(kNT)
    k_na_tiles(NaPol pol, SegSource src, NaVal *tf, NaVal *tc, int32_t *ta0,
               double *l1_part) {
  gasdev::tile_loop<NaPol, true, true>(pol, src, tf, tc, ta0);
  na_block_sum(pol.l1, l1_part + blockIdx.x);
}

__global__ void __launch_bounds__(kNT)
    k_na_fixup(NaPol pol, SegSource src, const NaVal *tf, const NaVal *tc,
               const int32_t *ta0, double *l1_part) {
  gasdev::fixup_loop<NaPol, true>(pol, src, tf, tc, ta0);
  na_block_sum(pol.l1, l1_part + blockIdx.x);
}

__global__ void __launch_bounds__(kNT)
    k_na_finish(const double *l1_part, int n, double *l1_out) {
  __shared__ double s[kNT];
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += kNT) v += l1_part[i];
  s[threadIdx.x] = v;
  __syncthreads();
  for (int d = kNT / 2; d > 0; d >>= 1) {
    if (threadIdx.x < d) s[threadIdx.x] += s[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) *l1_out = s[0];
}

}  // namespace

extern "C" gas_status_t gas_pagerank_step_noalloc(
    int32_t nV, int32_t nE, const int32_t *csc_off, const int32_t *csc_src,
    const int32_t *out_degree, const float *rank_in, float *rank_out,
    double damping, double *l1_out, void *stream) {
  if (nV < 0 || nE < 0)
    return gas::fail(GAS_ERR_INVALID, "pagerank_step_noalloc: negative size");
  if ((int64_t)nV + nE > GAS_NOALLOC_MAX_ITEMS)
    return gas::fail(GAS_ERR_TOO_LARGE,
                     "pagerank_step_noalloc: nV + nE = %lld exceeds the fixed scratch "
                     "limit of %lld; use gas_engine_pagerank_precision",
                     (long long)nV + nE, (long long)GAS_NOALLOC_MAX_ITEMS);
  if (!l1_out || (nV > 0 && (!csc_off || !out_degree || !rank_in || !rank_out)) ||
      (nE > 0 && !csc_src))
    return gas::fail(GAS_ERR_INVALID, "pagerank_step_noalloc: null pointer");
  if (!(damping > 0.0 && damping < 1.0))
    return gas::fail(GAS_ERR_INVALID, "pagerank_step_noalloc: damping outside (0,1)");
  unsigned char *scratch = nullptr;
  gas_status_t st = scratch_address(&scratch);
  if (st != GAS_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  int32_t *part = reinterpret_cast<int32_t *>(scratch + kPartOff);
  NaVal *tf = reinterpret_cast<NaVal *>(scratch + kFirstOff);
  NaVal *tc = reinterpret_cast<NaVal *>(scratch + kCarryOff);
  int32_t *ta0 = reinterpret_cast<int32_t *>(scratch + kA0Off);
  double *l1_part = reinterpret_cast<double *>(scratch + kL1Off);

  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (ce == cudaSuccess)
    ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_na_tiles, kNT, 0);
  if (ce != cudaSuccess)
    return gas::fail(GAS_ERR_CUDA, "pagerank_step_noalloc: %s", cudaGetErrorString(ce));
  if (per_sm < 1) per_sm = 1;
  const int64_t items = (int64_t)nV + nE;
  const int64_t ntiles = (items + kTile - 1) / kTile;
  int tiles_grid = (int)std::min<int64_t>(std::max<int64_t>(ntiles, 1), (int64_t)sms * per_sm);
  int fix_grid = 2 * sms;
  if (tiles_grid + fix_grid > kMaxCtas) {
    tiles_grid = kMaxCtas / 2;
    fix_grid = kMaxCtas / 2;
  }
  NaPol pol;
  pol.csc_src = csc_src;
  pol.out_degree = out_degree;
  pol.rank_in = rank_in;
  pol.rank_out = rank_out;
  pol.base = nV ? (float)((1.0 - damping) / (double)nV) : 0.0f;
  pol.damping = (float)damping;
  pol.l1 = 0.0;
  const SegSource src = gasdev::dense_source(csc_off, nV, nE, part);
  k_na_clear<<<8, kNT, 0, s>>>(l1_part, kMaxCtas);
  if (nV > 0) {
    const int pgrid = (int)std::min<int64_t>((ntiles + 1 + 255) / 256, 2 * (int64_t)sms);
    gasdev::k_partition<kTile, true><<<pgrid, 256, 0, s>>>(src, part);
    k_na_tiles<<<tiles_grid, kNT, 0, s>>>(pol, src, tf, tc, ta0, l1_part);
    k_na_fixup<<<fix_grid, kNT, 0, s>>>(pol, src, tf, tc, ta0, l1_part + tiles_grid);
  }
  k_na_finish<<<1, kNT, 0, s>>>(l1_part, tiles_grid + fix_grid, l1_out);
  ce = cudaGetLastError();
  if (ce != cudaSuccess)
    return gas::fail(GAS_ERR_CUDA, "pagerank_step_noalloc: launch: %s", cudaGetErrorString(ce));
  return GAS_OK;
}
