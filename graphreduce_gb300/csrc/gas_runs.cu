// gas_runs.cu -- whole-algorithm runs on a device-resident graph:
//   * gas_engine_run_schedule: run() (gpugas.h:1792-1807) with the loop moved
//     onto the device -- one iteration's kernels are captured once into the
//     body of a CUDA-graph WHILE node whose condition a tiny kernel sets from
//     the device counters, so there is no host round trip per iteration;
//   * gas_engine_pagerank_precision: the normalised PageRank with FP32
//     compensated (two-sum) gather and an FP64 L1 residual deciding
//     convergence on the device.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "gas.h"
#include "gas_device.cuh"
#include "gas_engine_impl.h"
#include "gas_internal.h"
#include "gas_sched.h"

using gasdev::kNT;
using gasdev::SegSource;

namespace {

inline cudaStream_t S(void *s) { return (cudaStream_t)s; }

// Loop condition: one more iteration while the frontier is non-empty and the
// cap is not reached; hitting the cap with work left raises the error word.
__global__ void k_loop_cond(gas_counters *cnt, cudaGraphConditionalHandle h,
                            int in_graph) {
  const int max_iter = cnt->max_iter;
  const int it = ++cnt->iteration;
  const bool more = cnt->n_active > 0;
  if (more && it >= max_iter) cnt->error = GAS_ERR_ITER_CAP;
  cnt->cond = (more && it < max_iter) ? 1 : 0;
  if (in_graph) cudaGraphSetConditional(h, cnt->cond);
}

__global__ void k_reset_loop(gas_counters *cnt, int32_t max_iter) {
  cnt->iteration = 0;
  cnt->error = 0;
  cnt->cond = 1;
  cnt->max_iter = max_iter;
}

}  // namespace

namespace gas {

// Builds graph = WHILE(cond) { body(stream, handle) } and instantiates it.
gas_status_t build_while_graph(
    gas_engine *e,
    gas_status_t (*body)(gas_engine *, cudaStream_t, cudaGraphConditionalHandle,
                         void *),
    void *ctx, cudaGraphExec_t *out) {
  cudaGraph_t g = nullptr;
  cudaStream_t cs = nullptr;
  cudaGraphExec_t x = nullptr;
  gas_status_t st = GAS_OK;
  cudaGraphConditionalHandle h;
  cudaGraphNodeParams p = {};
  cudaGraphNode_t node;
  cudaGraph_t bodyg;
  CUDA_TRY(cudaGraphCreate(&g, 0));
  cudaError_t ce = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  if (ce == cudaSuccess) {
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    ce = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p);
  }
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(GAS_ERR_CUDA, "while-graph setup: %s", cudaGetErrorString(ce));
  }
  bodyg = p.conditional.phGraph_out[0];
  ce = cudaStreamBeginCaptureToGraph(cs, bodyg, nullptr, nullptr, 0,
                                     cudaStreamCaptureModeRelaxed);
  if (ce == cudaSuccess) {
    e->capturing = true;
    e->in_graph = true;
    st = body(e, cs, h, ctx);
    e->capturing = false;
    e->in_graph = false;
    cudaGraph_t captured = nullptr;
    cudaError_t ce2 = cudaStreamEndCapture(cs, &captured);
    if (st == GAS_OK && ce2 != cudaSuccess)
      st = fail(GAS_ERR_CUDA, "end capture: %s", cudaGetErrorString(ce2));
  } else {
    st = fail(GAS_ERR_CUDA, "begin capture: %s", cudaGetErrorString(ce));
  }
  if (st == GAS_OK) {
    ce = cudaGraphInstantiate(&x, g, 0);
    if (ce != cudaSuccess)
      st = fail(GAS_ERR_CUDA, "instantiate: %s", cudaGetErrorString(ce));
  }
  cudaStreamDestroy(cs);
  cudaGraphDestroy(g);
  if (st == GAS_OK) *out = x;
  return st;
}

bool host_loop_requested() {
  const char *v = getenv("GAS_HOST_LOOP");
  return v && v[0] == '1';
}

bool host_loop_for(const gas_engine *e) {
  return e->profiling || host_loop_requested();
}

// The same loop without a graph: body launches on the stream, the host
// reads the condition word after every iteration.
gas_status_t run_host_loop(
    gas_engine *e,
    gas_status_t (*body)(gas_engine *, cudaStream_t, cudaGraphConditionalHandle,
                         void *),
    void *ctx, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  gas_status_t st = GAS_OK;
  e->capturing = true;
  e->in_graph = false;
  for (;;) {
    cudaError_t ce = cudaMemcpyAsync(e->h_cnt, e->cnt, sizeof(gas_counters),
                                     cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) {
      st = fail(GAS_ERR_CUDA, "host loop: %s", cudaGetErrorString(ce));
      break;
    }
    if (!e->h_cnt->cond) break;
    st = body(e, s, 0, ctx);
    if (st != GAS_OK) break;
    prof_collect(e);
  }
  e->capturing = false;
  return st;
}

// Turns the device error word / a non-empty frontier after the loop into a
// status, and clears the word so the engine stays usable.
gas_status_t loop_status(gas_engine *e, const gas_counters &c, void *stream) {
  if (c.error)
    CUDA_TRY(cudaMemsetAsync(&e->cnt->error, 0, sizeof(int32_t), S(stream)));
  if (c.error == GAS_ERR_ITER_CAP || (c.error == 0 && c.n_active > 0))
    return fail(GAS_ERR_ITER_CAP, "no convergence within %d iterations", c.iteration);
  if (c.error)
    return fail(GAS_ERR_DEVICE, "device error word %d after %d iterations", c.error,
                c.iteration);
  return GAS_OK;
}

}  // namespace gas

namespace {

struct GenericCtx {
  bool ordered;
};

gas_status_t generic_body(gas_engine *e, cudaStream_t cs,
                          cudaGraphConditionalHandle h, void *ctx) {
  const GenericCtx *c = static_cast<const GenericCtx *>(ctx);
  GAS_TRY(gas::engine_generic_iteration(e, c->ordered, cs));
  k_loop_cond<<<1, 1, 0, cs>>>(e->cnt, h, e->in_graph ? 1 : 0);
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

}  // namespace

extern "C" gas_status_t gas_engine_run_schedule(gas_engine *e,
                                                gas_schedule_t schedule,
                                                int32_t max_iterations,
                                                gas_run_stats *stats,
                                                void *stream) {
  if (!e || !e->has_graph) return gas::fail(GAS_ERR_STATE, "run before set_graph");
  if (e->prog == GAS_PROG_USER)
    return gas::fail(GAS_ERR_UNSUPPORTED, "user programs run through gpugas.h");
  // default cap: nV + 2 bounds every correct BFS / SSSP / CC run (each
  // iteration settles at least one more vertex); PageRank gets 100000
  if (max_iterations <= 0)
    max_iterations = e->prog == GAS_PROG_PAGERANK ? 100000 : e->nV + 2;
  if (stats) *stats = gas_run_stats{};
  int32_t n = 0;
  GAS_TRY(gas_engine_count_active(e, &n));
  if (e->pending_gather || e->slots_pending)
    return gas::fail(GAS_ERR_STATE, "run_schedule in the middle of a step");
  if (n == 0) return GAS_OK;
  if (schedule != GAS_SCHED_GENERIC && schedule != GAS_SCHED_ORDERED)
    return gas::run_fast(e, schedule, max_iterations, stats, stream);

  GenericCtx ctx{schedule == GAS_SCHED_ORDERED};
  const int slot = ctx.ordered ? kGraphOrdered : kGraphGeneric;
  if (gas::host_loop_for(e)) {
    k_reset_loop<<<1, 1, 0, S(stream)>>>(e->cnt, max_iterations);
    CUDA_TRY(cudaGetLastError());
    e->level_from_counters = true;
    gas_status_t st = gas::run_host_loop(e, generic_body, &ctx, stream);
    e->level_from_counters = false;
    if (st != GAS_OK) return st;
  } else {
  if (!e->graphs[slot]) {
    e->level_from_counters = true;
    gas_status_t st = gas::build_while_graph(e, generic_body, &ctx, &e->graphs[slot]);
    e->level_from_counters = false;
    if (st != GAS_OK) return st;
  }
  k_reset_loop<<<1, 1, 0, S(stream)>>>(e->cnt, max_iterations);
  cudaError_t ce = cudaGetLastError();
  if (ce == cudaSuccess) ce = cudaGraphLaunch(e->graphs[slot], S(stream));
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(S(stream));
  if (ce != cudaSuccess)
    return gas::fail(GAS_ERR_CUDA, "generic run: %s", cudaGetErrorString(ce));
  }
  gas_counters c;
  GAS_TRY(gas_engine_read_counters(e, &c, stream));
  if (stats) {
    stats->iterations = c.iteration;
    // per iteration: gather tiles + fixup (or BFS apply), commit, 3 scan
    // passes, expand, 3 compaction passes, loop condition; plus the reset
    stats->kernel_launches = c.iteration * (e->prog == GAS_PROG_BFS ? 9 : 11) + 1;
  }
  e->level = c.iteration;
  e->active_full = false;
  return gas::loop_status(e, c, stream);
}

// ---------------------------------------------------------------------------
// Precision-form PageRank.
// ---------------------------------------------------------------------------
namespace {

struct PrVal {
  float s, c;
};

// Error-free transformation: a.s + b.s = s + err exactly (Knuth two-sum);
// compensation terms are carried in c.
__device__ __forceinline__ PrVal two_sum_add(const PrVal &a, const PrVal &b) {
  const float s = __fadd_rn(a.s, b.s);
  const float bp = __fsub_rn(s, a.s);
  const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bp)), __fsub_rn(b.s, bp));
  return PrVal{s, __fadd_rn(__fadd_rn(a.c, b.c), err)};
}

struct PrPol {
  typedef PrVal Val;
  static constexpr bool kMapNeedsVertex = false;
  const int32_t *csc_src;
  const float *inv_deg;  // RN(1 / out-degree), 0 without out-edges
  const float *contrib;
  const float *rank_old;
  float *rank_new;
  float *contrib_new;
  float base;       // (1-d)/N, every vertex (seed < 0)
  float base_seed;  // (1-d), the seed only (personalized)
  float damping;
  const int32_t *seed_p;
  int32_t seed;
  double l1;
  __device__ Val zero() const { return PrVal{0.0f, 0.0f}; }
  __device__ __forceinline__ Val reduce(const Val &a, const Val &b) const {
    return two_sum_add(a, b);
  }
  // Inside a 32-edge slab the contributions are summed as plain floats by
  // the log-depth segmented scan (relative error <= 5 u of the slab's sum,
  // the terms being non-negative); the slab sums of a row are combined with
  // two-sum.
  typedef float Scan;
  __device__ __forceinline__ Scan to_scan(const Val &v) const { return v.s; }
  __device__ __forceinline__ Val from_scan(Scan x) const { return PrVal{x, 0.0f}; }
  __device__ __forceinline__ Scan scan_add(Scan a, Scan b) const { return __fadd_rn(a, b); }
  __device__ __forceinline__ Val map(int, int, int pos) const {
    return PrVal{__ldg(contrib + __ldg(csc_src + pos)), 0.0f};
  }
  __device__ __forceinline__ void emit(int, int v, const Val &g) {
    const float sum = __fadd_rn(g.s, g.c);
    const float b = seed < 0 ? base : (v == seed ? base_seed : 0.0f);
    const float r = __fadd_rn(b, __fmul_rn(damping, sum));
    rank_new[v] = r;
    contrib_new[v] = __fmul_rn(r, __ldg(inv_deg + v));
    // the step in FP32 (exact while the two ranks are within a factor of
    // two of each other, Sterbenz), the sum in FP64
    l1 += (double)fabsf(__fsub_rn(r, rank_old[v]));
  }
};

struct PrBufs {
  float *rank[2];
  float *contrib[2];
};

__device__ __forceinline__ void pr_bind(PrPol &pol, const PrBufs &b,
                                        const gas_counters *cnt) {
  const int p = cnt->iteration & 1;
  pol.contrib = b.contrib[p];
  pol.rank_old = b.rank[p];
  pol.rank_new = b.rank[p ^ 1];
  pol.contrib_new = b.contrib[p ^ 1];
  pol.seed = *pol.seed_p;
  pol.l1 = 0.0;
}

__device__ __forceinline__ void block_sum_store(double v, double *out) {
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

__global__ void __launch_bounds__(kNT)
    k_pr_slab(PrPol pol, PrBufs bufs, gasdev::SlabSource src, PrVal *cf, PrVal *cc,
              int32_t *ca0, int32_t *fix, int32_t *fix_n, const gas_counters *cnt,
              double *l1_part) {
  pr_bind(pol, bufs, cnt);
  gasdev::slab_loop<PrPol, true>(pol, src, cf, cc, ca0, fix, fix_n);
  block_sum_store(pol.l1, l1_part + blockIdx.x);
}

__global__ void __launch_bounds__(kNT)
    k_pr_fixup(PrPol pol, PrBufs bufs, gasdev::SlabSource src, const PrVal *cf,
               const PrVal *cc, const int32_t *ca0, const int32_t *fix,
               const int32_t *fix_n, const gas_counters *cnt, double *l1_part) {
  pr_bind(pol, bufs, cnt);
  gasdev::slab_fixup_loop<PrPol>(pol, src, cf, cc, ca0, fix, fix_n);
  block_sum_store(pol.l1, l1_part + blockIdx.x);
}

// Vertices without in-edges: rank = (1-d)/N.
__global__ void __launch_bounds__(kNT)
    k_pr_empty(PrPol pol, PrBufs bufs, const int32_t *zero_vid, int n_zero,
               const gas_counters *cnt, double *l1_part) {
  pr_bind(pol, bufs, cnt);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_zero;
       i += gridDim.x * blockDim.x)
    pol.emit(0, zero_vid[i], pol.zero());
  block_sum_store(pol.l1, l1_part + blockIdx.x);
}

// Deterministic sum of the per-CTA residuals; sets the loop condition.
__global__ void __launch_bounds__(kNT)
    k_pr_finish(const double *l1_part, int n, const double *tol_p,
                gas_counters *cnt, double *residual, int32_t *fix_n,
                cudaGraphConditionalHandle h, int in_graph) {
  __shared__ double s[kNT];
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += kNT) v += l1_part[i];
  s[threadIdx.x] = v;
  __syncthreads();
  for (int d = kNT / 2; d > 0; d >>= 1) {
    if (threadIdx.x < d) s[threadIdx.x] += s[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double l1 = s[0];
    const double tol = *tol_p;
    *fix_n = 0;  // the fixup of this iteration has run
    const int max_iter = cnt->max_iter;
    *residual = l1;
    const int it = ++cnt->iteration;
    const bool more = !(l1 <= tol);
    if (more && it >= max_iter) cnt->error = GAS_ERR_ITER_CAP;
    cnt->cond = (more && it < max_iter) ? 1 : 0;
    if (in_graph) cudaGraphSetConditional(h, cnt->cond);
  }
}

// Initial ranks: 1/N, e_seed (seed >= 0), or the caller's vector already
// copied into rank; and the reciprocal out-degrees the iterations scale
// contributions by.
__global__ void k_pr_init(float *rank, float *contrib, float *inv_deg, const int32_t *csr_off,
                          int n, float r0, int have_init, int seed) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += gridDim.x * blockDim.x) {
    const int deg = csr_off[v + 1] - csr_off[v];
    const float inv = deg ? __frcp_rn((float)deg) : 0.0f;
    const float r = have_init ? rank[v] : seed < 0 ? r0 : (v == seed ? 1.0f : 0.0f);
    rank[v] = r;
    inv_deg[v] = inv;
    contrib[v] = __fmul_rn(r, inv);
  }
}

struct PrCtx {
  PrPol pol;
  PrBufs bufs;
  gasdev::SlabSource src;
  int tiles_grid;
  int fix_grid;
  int empty_grid;
  double *residual;
};

gas_status_t pr_body(gas_engine *e, cudaStream_t cs,
                     cudaGraphConditionalHandle h, void *vctx) {
  PrCtx *c = static_cast<PrCtx *>(vctx);
  // algorithmic bytes of one iteration: per edge its source index and the
  // source's contribution; per vertex offsets, old and new rank, new
  // contribution
  gas::prof_begin(e, cs, gas::kProfPagerank, 8LL * e->nE + 16LL * e->nV);
  k_pr_slab<<<c->tiles_grid, kNT, 0, cs>>>(
      c->pol, c->bufs, c->src, (PrVal *)e->slab_first, (PrVal *)e->slab_carry,
      e->slab_a0, e->slab_fix, e->slab_fix_n, e->cnt, e->pr_l1);
  k_pr_fixup<<<c->fix_grid, kNT, 0, cs>>>(
      c->pol, c->bufs, c->src, (const PrVal *)e->slab_first,
      (const PrVal *)e->slab_carry, e->slab_a0, e->slab_fix, e->slab_fix_n, e->cnt,
      e->pr_l1 + c->tiles_grid);
  gas::prof_end(e, cs);
  k_pr_empty<<<c->empty_grid, kNT, 0, cs>>>(c->pol, c->bufs, e->zero_vid, e->n_zero,
                                            e->cnt,
                                            e->pr_l1 + c->tiles_grid + c->fix_grid);
  k_pr_finish<<<1, kNT, 0, cs>>>(e->pr_l1, c->tiles_grid + c->fix_grid + c->empty_grid,
                                 c->residual + 1, e->cnt, c->residual, e->slab_fix_n, h,
                                 e->in_graph ? 1 : 0);
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

}  // namespace

extern "C" gas_status_t gas_engine_pagerank_precision(
    gas_engine *e, double damping, double tol, int32_t max_iterations,
    float *ranks, gas_run_stats *stats, void *stream) {
  return gas_engine_pagerank_precision_from(e, damping, tol, max_iterations, nullptr,
                                            ranks, stats, stream);
}

namespace {

gas_status_t pagerank_run(gas_engine *e, double damping, double tol, int32_t max_iterations,
                          const float *init, int32_t seed, float *ranks, gas_run_stats *stats,
                          void *stream) {
  if (!e || !e->has_graph) return gas::fail(GAS_ERR_STATE, "no graph");
  if (!(damping > 0.0 && damping < 1.0) || !(tol > 0.0))
    return gas::fail(GAS_ERR_INVALID, "damping must be in (0,1), tol > 0");
  if (max_iterations <= 0) max_iterations = 1000;
  if (stats) *stats = gas_run_stats{};
  const int nV = e->nV;
  if (nV == 0) return GAS_OK;
  if (seed >= nV) return gas::fail(GAS_ERR_INVALID, "seed %d outside [0, %d)", seed, nV);
  for (int i = 0; i < 2; ++i) {
    if (!e->pr_rank[i]) CUDA_TRY(cudaMalloc(&e->pr_rank[i], (size_t)nV * 4));
    if (!e->pr_contrib[i]) CUDA_TRY(cudaMalloc(&e->pr_contrib[i], (size_t)nV * 4));
  }
  if (!e->pr_seed) CUDA_TRY(cudaMalloc(&e->pr_seed, sizeof(int32_t)));
  if (!e->pr_inv_deg) CUDA_TRY(cudaMalloc(&e->pr_inv_deg, (size_t)nV * 4));
  PrCtx c;
  int per_sm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pr_slab, kNT, 0));
  c.tiles_grid = e->num_sms * (per_sm > 0 ? per_sm : 1);  // resident CTAs only
  c.fix_grid = 2 * e->num_sms;
  c.empty_grid = 2 * e->num_sms;
  const int nparts = c.tiles_grid + c.fix_grid + c.empty_grid;
  if (!e->pr_l1 || e->pr_l1_cap < nparts + 2) {
    if (e->pr_l1) cudaFree(e->pr_l1);
    e->pr_l1 = nullptr;
    if (e->graphs[kGraphPagerank]) cudaGraphExecDestroy(e->graphs[kGraphPagerank]);
    e->graphs[kGraphPagerank] = nullptr;
    e->pr_l1_cap = nparts + 2;
    CUDA_TRY(cudaMalloc(&e->pr_l1, sizeof(double) * (size_t)e->pr_l1_cap));
  }
  c.residual = e->pr_l1 + nparts;
  c.pol.csc_src = e->csc_src;
  c.pol.inv_deg = e->pr_inv_deg;
  c.pol.base = (float)((1.0 - damping) / (double)nV);
  c.pol.base_seed = (float)(1.0 - damping);
  c.pol.damping = (float)damping;
  c.pol.seed_p = e->pr_seed;
  c.pol.seed = -1;
  c.pol.l1 = 0.0;
  c.bufs.rank[0] = e->pr_rank[0];
  c.bufs.rank[1] = e->pr_rank[1];
  c.bufs.contrib[0] = e->pr_contrib[0];
  c.bufs.contrib[1] = e->pr_contrib[1];
  c.src = gasdev::slab_source(e->ne_end, e->ne_vid, nullptr, e->n_ne, e->nE, nullptr,
                              nullptr, e->slab_dpart);

  // damping is baked into the captured policy: rebuild when it changes
  if (e->graphs[kGraphPagerank] && e->pr_damping != damping) {
    cudaGraphExecDestroy(e->graphs[kGraphPagerank]);
    e->graphs[kGraphPagerank] = nullptr;
  }
  const bool host_loop = gas::host_loop_for(e);
  if (!host_loop && !e->graphs[kGraphPagerank]) {
    GAS_TRY(gas::build_while_graph(e, pr_body, &c, &e->graphs[kGraphPagerank]));
    e->pr_damping = damping;
  }
  CUDA_TRY(cudaMemcpyAsync(c.residual + 1, &tol, sizeof(double),
                           cudaMemcpyHostToDevice, S(stream)));
  CUDA_TRY(cudaMemcpyAsync(e->pr_seed, &seed, sizeof(int32_t), cudaMemcpyHostToDevice,
                           S(stream)));
  gasdev::k_slab_partition<><<<2 * e->num_sms, 256, 0, S(stream)>>>(c.src, e->slab_dpart);
  if (init)
    CUDA_TRY(cudaMemcpyAsync(e->pr_rank[0], init, (size_t)nV * 4, cudaMemcpyDefault,
                             S(stream)));
  k_pr_init<<<gas::engine_grid(nV, kNT, 8 * e->num_sms), kNT, 0, S(stream)>>>(
      e->pr_rank[0], e->pr_contrib[0], e->pr_inv_deg, e->csr_off, nV, (float)(1.0 / nV),
      init ? 1 : 0, seed);
  k_reset_loop<<<1, 1, 0, S(stream)>>>(e->cnt, max_iterations);
  cudaError_t ce = cudaGetLastError();
  if (host_loop) {
    if (ce == cudaSuccess) GAS_TRY(gas::run_host_loop(e, pr_body, &c, stream));
  } else if (ce == cudaSuccess) {
    ce = cudaGraphLaunch(e->graphs[kGraphPagerank], S(stream));
  }
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(S(stream));
  if (ce != cudaSuccess)
    return gas::fail(GAS_ERR_CUDA, "pagerank: %s", cudaGetErrorString(ce));
  gas_counters cnt;
  GAS_TRY(gas_engine_read_counters(e, &cnt, stream));
  if (cnt.error && cnt.error != GAS_ERR_ITER_CAP)
    return gas::loop_status(e, cnt, stream);
  if (cnt.error) CUDA_TRY(cudaMemsetAsync(&e->cnt->error, 0, sizeof(int32_t), S(stream)));
  double resid = 0.0;
  CUDA_TRY(cudaMemcpy(&resid, c.residual, sizeof(double), cudaMemcpyDeviceToHost));
  const int final_buf = cnt.iteration & 1;
  if (ranks)
    CUDA_TRY(cudaMemcpyAsync(ranks, e->pr_rank[final_buf], (size_t)nV * 4,
                             cudaMemcpyDefault, S(stream)));
  CUDA_TRY(cudaStreamSynchronize(S(stream)));
  if (stats) {
    stats->iterations = cnt.iteration;
    stats->pull_iters = cnt.iteration;
    stats->kernel_launches = 4 * cnt.iteration + 3;
    stats->edges_processed = (int64_t)cnt.iteration * e->nE;
    stats->residual = resid;
  }
  if (!(resid <= tol))
    return gas::fail(GAS_ERR_ITER_CAP, "pagerank: residual %.3e after %d iterations",
                     resid, cnt.iteration);
  return GAS_OK;
}

}  // namespace

extern "C" gas_status_t gas_engine_pagerank_precision_from(
    gas_engine *e, double damping, double tol, int32_t max_iterations,
    const float *init, float *ranks, gas_run_stats *stats, void *stream) {
  return pagerank_run(e, damping, tol, max_iterations, init, -1, ranks, stats, stream);
}

extern "C" gas_status_t gas_engine_ppr_precision(gas_engine *e, int32_t seed, double damping,
                                                 double tol, int32_t max_iterations,
                                                 float *ranks, gas_run_stats *stats,
                                                 void *stream) {
  if (seed < 0) return gas::fail(GAS_ERR_INVALID, "ppr: seed must be >= 0");
  return pagerank_run(e, damping, tol, max_iterations, nullptr, seed, ranks, stats, stream);
}
