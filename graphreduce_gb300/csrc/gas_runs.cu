// gas_runs.cu -- whole-algorithm runs on a device-resident graph:
//   * gas_engine_run_schedule: run() (gpugas.h:1792-1807) with the loop moved
//     onto the device -- one iteration's kernels are captured once into the
//     body of a CUDA-graph WHILE node whose condition a tiny kernel sets from
//     the device counters, so there is no host round trip per iteration;
//   * gas_engine_pagerank_precision: the normalised PageRank with FP32
//     compensated (two-sum) gather and an FP64 L1 residual deciding
//     convergence on the device.
#include <cuda_runtime.h>

#include <algorithm>
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
    stats->graph_launches = gas::host_loop_for(e) ? 0 : 1;
  }
  e->level = c.iteration;
  e->active_full = false;
  return gas::loop_status(e, c, stream);
}

// ---------------------------------------------------------------------------
// run() of a user program: the Program-typed kernels come from the caller's
// translation unit through a step callback; the rest of the iteration is
// libgas's, and the loop is a WHILE node on the device.
// ---------------------------------------------------------------------------
namespace {

struct UserCtx {
  gas_user_step_fn step;
  void *ctx;
  int32_t wrote_slots;
};

gas_status_t user_body(gas_engine *e, cudaStream_t cs, cudaGraphConditionalHandle h,
                       void *ctx) {
  const UserCtx *u = static_cast<const UserCtx *>(ctx);
  GAS_TRY(u->step(u->ctx, cs));
  CUDA_TRY(cudaGetLastError());
  e->slots_pending = u->wrote_slots != 0;
  GAS_TRY(gas::engine_scatter(e, cs));
  k_loop_cond<<<1, 1, 0, cs>>>(e->cnt, h, e->in_graph ? 1 : 0);
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

}  // namespace

extern "C" gas_status_t gas_engine_run_user(gas_engine *e, gas_user_step_fn step,
                                            void *ctx, int32_t wrote_slots,
                                            int32_t max_iterations, gas_run_stats *stats,
                                            void *stream) {
  if (!e || !step) return gas::fail(GAS_ERR_INVALID, "run_user: null argument");
  if (!e->has_graph) return gas::fail(GAS_ERR_STATE, "run before set_graph");
  if (e->prog != GAS_PROG_USER)
    return gas::fail(GAS_ERR_UNSUPPORTED, "run_user: built-in programs use run_schedule");
  if (max_iterations <= 0) max_iterations = 1000000;
  if (stats) *stats = gas_run_stats{};
  int32_t n = 0;
  GAS_TRY(gas_engine_count_active(e, &n));
  if (e->pending_gather || e->slots_pending)
    return gas::fail(GAS_ERR_STATE, "run_user in the middle of a step");
  if (n == 0) return GAS_OK;
  UserCtx u{step, ctx, wrote_slots != 0 ? 1 : 0};
  const bool direct = gas::host_loop_for(e);
  if (direct) {
    k_reset_loop<<<1, 1, 0, S(stream)>>>(e->cnt, max_iterations);
    CUDA_TRY(cudaGetLastError());
    GAS_TRY(gas::run_host_loop(e, user_body, &u, stream));
  } else {
    if (e->graphs[kGraphUser] && (e->user_step != step || e->user_ctx != ctx ||
                                  e->user_wrote_slots != u.wrote_slots)) {
      cudaGraphExecDestroy(e->graphs[kGraphUser]);
      e->graphs[kGraphUser] = nullptr;
    }
    if (!e->graphs[kGraphUser]) {
      GAS_TRY(gas::build_while_graph(e, user_body, &u, &e->graphs[kGraphUser]));
      e->user_step = step;
      e->user_ctx = ctx;
      e->user_wrote_slots = u.wrote_slots;
    }
    k_reset_loop<<<1, 1, 0, S(stream)>>>(e->cnt, max_iterations);
    cudaError_t ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaGraphLaunch(e->graphs[kGraphUser], S(stream));
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(S(stream));
    if (ce != cudaSuccess)
      return gas::fail(GAS_ERR_CUDA, "user run: %s", cudaGetErrorString(ce));
  }
  gas_counters c;
  GAS_TRY(gas_engine_read_counters(e, &c, stream));
  if (stats) {
    stats->iterations = c.iteration;
    // per iteration: the caller's partition, tiles and fixup; commit, 3 scan
    // passes, partition, expand, 3 compaction passes, loop condition; reset
    stats->kernel_launches = 13 * c.iteration + 1;
    stats->graph_launches = direct ? 0 : 1;
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

// The row epilogue of the precision PageRank: the gathered sum (value +
// compensation) of a destination row becomes its new rank and contribution;
// the L1 step accumulates per thread.
struct PrPol {
  typedef PrVal Val;
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
  // inv and old: the row's reciprocal out-degree and previous rank
  __device__ __forceinline__ void emit(int v, const Val &g, float inv, float old) {
    const float sum = __fadd_rn(g.s, g.c);
    const float b = seed < 0 ? base : (v == seed ? base_seed : 0.0f);
    const float r = __fadd_rn(b, __fmul_rn(damping, sum));
    rank_new[v] = r;
    contrib_new[v] = __fmul_rn(r, inv);
    // the step in FP32 (exact while the two ranks are within a factor of
    // two of each other, Sterbenz), the sum in FP64
    l1 += (double)fabsf(__fsub_rn(r, old));
  }
  __device__ __forceinline__ void emit(int v, const Val &g) {
    emit(v, g, __ldg(inv_deg + v), rank_old[v]);
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

// ---- merge-path gather (Merrill & Garland, "Merge-based parallel sparse
// matrix-vector multiplication", SC'16) ----
// The CSC is walked as one merge path of nV row ends and nE in-edges (an
// edge is taken while its index is below the current row's end offset).  A
// warp owns a tile of kPrW consecutive path items, a lane kPrK of them; the
// warps of a CTA never wait for one another.  A tile stages its row end
// offsets and the gathered contributions of its edges in the warp's shared
// memory (coalesced index loads, kPrK independent gathers per lane), each
// lane sums its items sequentially, a segmented warp scan of the lanes'
// open-row partials joins rows that span lanes, and the rows that start and
// end inside the tile are finished there with coalesced writes.  A row that
// spans tiles leaves its first part as the tile's tail record and the
// following parts as head records; k_pr_merge_fix joins them.
constexpr int kPrK = 8;
constexpr int kPrW = 32 * kPrK;
constexpr int kPrWarps = kNT / 32;
// s_val is padded by one word per kPrK: a lane reads about kPrK words past
// its neighbour, which without the pad puts 32 / kPrK lanes on one bank
__device__ __forceinline__ int pr_pad(int j) { return j + j / kPrK; }
constexpr int kPrValWords = kPrW + kPrW / kPrK;

struct PrCarry {
  int32_t row;   // -1: no record
  int32_t done;  // head: the row ends in this tile
  float s, c;
};

// Merge-path coordinate (rows ended) of each tile start, once per run.
__global__ void k_pr_tiles(const int32_t *csc_off, int nV, int nE, int n_tiles,
                           int32_t *tile_row) {
  const long long path = (long long)nV + nE;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t <= n_tiles;
       t += gridDim.x * blockDim.x) {
    const long long d = min((long long)t * kPrW, path);
    long long lo = max(d - nE, 0LL), hi = min(d, (long long)nV);
    while (lo < hi) {
      const long long p = (lo + hi) >> 1;
      if (csc_off[p + 1] <= d - p - 1)
        lo = p + 1;
      else
        hi = p;
    }
    tile_row[t] = (int32_t)lo;
  }
}

__device__ __forceinline__ int32_t pr_ld_stream(const int32_t *p) {
  int32_t v;
  asm volatile("ld.global.nc.L1::no_allocate.b32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}

__global__ void __launch_bounds__(kNT, 3)
    k_pr_merge(PrPol pol, PrBufs bufs, const int32_t *csc_off, int nV, int nE,
               const int32_t *tile_row, int n_tiles, PrCarry *head, PrCarry *tail,
               const gas_counters *cnt, double *l1_part) {
  __shared__ int32_t s_end_all[kPrWarps][kPrW + 1];
  __shared__ float s_val_all[kPrWarps][kPrValWords];
  __shared__ float2 s_sum_all[kPrWarps][kPrW];
  pr_bind(pol, bufs, cnt);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t *s_end = s_end_all[warp];
  float *s_val = s_val_all[warp];
  float2 *s_sum = s_sum_all[warp];
  const long long path = (long long)nV + nE;
  const int nwarps = gridDim.x * kPrWarps;
  // software pipeline: the next tile's coordinates and edge indices load
  // while this tile's gathers and sums run
  int tile = blockIdx.x * kPrWarps + warp;
  int r0 = 0, r1 = 0;
  int idx[kPrK];
  if (tile < n_tiles) {
    r0 = tile_row[tile];
    r1 = tile_row[tile + 1];
    const int e0 = (int)((long long)tile * kPrW - r0);
    const int ne = (int)(min((long long)tile * kPrW + kPrW, path) - r1) - e0;
#pragma unroll
    for (int k = 0; k < kPrK; ++k) {
      const int j = lane + 32 * k;
      idx[k] = j < ne ? pr_ld_stream(pol.csc_src + e0 + j) : 0;
    }
  }
  for (; tile < n_tiles; tile += nwarps) {
    const long long D0 = (long long)tile * kPrW;
    const long long D1 = min(D0 + kPrW, path);
    const int e0 = (int)(D0 - r0), e1 = (int)(D1 - r1);
    const int nrows = r1 - r0, ne = e1 - e0;
    float val[kPrK];
#pragma unroll
    for (int k = 0; k < kPrK; ++k) {
      const int j = lane + 32 * k;
      val[k] = j < ne ? __ldg(pol.contrib + idx[k]) : 0.0f;
    }
    const int off0 = csc_off[r0];
#pragma unroll
    for (int k = 0; k < kPrK; ++k) {
      const int j = lane + 32 * k;
      if (j < nrows) s_end[j] = csc_off[r0 + 1 + j];
    }
    if (lane == 0) s_end[nrows] = INT_MAX;
    const int next = tile + nwarps;
    int nr0 = 0, nr1 = 0;
    if (next < n_tiles) {
      nr0 = tile_row[next];
      nr1 = tile_row[next + 1];
      const int ne0 = (int)((long long)next * kPrW - nr0);
      const int nne = (int)(min((long long)next * kPrW + kPrW, path) - nr1) - ne0;
#pragma unroll
      for (int k = 0; k < kPrK; ++k) {
        const int j = lane + 32 * k;
        idx[k] = j < nne ? pr_ld_stream(pol.csc_src + ne0 + j) : 0;
      }
    }
#pragma unroll
    for (int k = 0; k < kPrK; ++k) {
      const int j = lane + 32 * k;
      if (j < ne) s_val[pr_pad(j)] = val[k];
    }
    // the epilogue's inputs for the tile's first 32 rows
    float inv0 = 0.0f, old0 = 0.0f;
    if (lane < nrows) {
      inv0 = __ldg(pol.inv_deg + r0 + lane);
      old0 = pol.rank_old[r0 + lane];
    }
    __syncwarp();
    // this lane's kPrK items: find its start on the tile's path
    const int tlen = nrows + ne;
    const int dt = min(lane * kPrK, tlen), dend = min(dt + kPrK, tlen);
    int lo = max(dt - ne, 0), hi = min(dt, nrows);
    while (lo < hi) {
      const int p = (lo + hi) >> 1;
      if (s_end[p] <= e0 + dt - p - 1)
        lo = p + 1;
      else
        hi = p;
    }
    int r = lo, e = e0 + dt - lo;
    int end_r = s_end[r];
    float acc = 0.0f, first = 0.0f;
    int first_r = 0;
    bool ended = false;
#pragma unroll
    for (int k = 0; k < kPrK; ++k) {
      if (dt + k < dend) {
        if (e < end_r) {
          acc = __fadd_rn(acc, s_val[pr_pad(e - e0)]);
          ++e;
        } else {
          if (!ended) {
            first = acc;
            first_r = r;
          } else {
            s_sum[r] = make_float2(acc, 0.0f);
          }
          ended = true;
          acc = 0.0f;
          ++r;
          end_r = s_end[r];
        }
      }
    }
    // segmented inclusive scan of the open-row partials (a lane that ended
    // a row starts a segment)
    PrVal v{acc, 0.0f};
    int f = ended;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const PrVal u{__shfl_up_sync(0xffffffffu, v.s, o), __shfl_up_sync(0xffffffffu, v.c, o)};
      const int g = __shfl_up_sync(0xffffffffu, f, o);
      if (lane >= o) {
        if (!f) v = two_sum_add(u, v);
        f |= g;
      }
    }
    PrVal cin{__shfl_up_sync(0xffffffffu, v.s, 1), __shfl_up_sync(0xffffffffu, v.c, 1)};
    if (lane == 0) cin = PrVal{0.0f, 0.0f};
    if (ended) {
      const PrVal t = two_sum_add(cin, PrVal{first, 0.0f});
      s_sum[first_r] = make_float2(t.s, t.c);
    }
    const PrVal tot{__shfl_sync(0xffffffffu, v.s, 31), __shfl_sync(0xffffffffu, v.c, 31)};
    __syncwarp();
    // rows that start and end in this tile; row r0 started in an earlier
    // tile when e0 is past its first edge
    const bool split = e0 > off0;
    if (lane < nrows && !(lane == 0 && split)) {
      const float2 t = s_sum[lane];
      pol.emit(r0 + lane, PrVal{t.x, t.y}, inv0, old0);
    }
    for (int i = lane + 32; i < nrows; i += 32) {
      const float2 t = s_sum[i];
      pol.emit(r0 + i, PrVal{t.x, t.y});
    }
    if (lane == 0) {
      PrCarry h{-1, 0, 0.0f, 0.0f}, tl{-1, 0, 0.0f, 0.0f};
      if (split) {
        if (nrows > 0)
          h = PrCarry{r0, 1, s_sum[0].x, s_sum[0].y};
        else
          h = PrCarry{r0, 0, tot.s, tot.c};
      }
      if (r1 < nV && !(split && nrows == 0)) {
        const int off_r1 = nrows > 0 ? s_end[nrows - 1] : off0;
        if (e1 > max(off_r1, e0)) tl = PrCarry{r1, 0, tot.s, tot.c};
      }
      head[tile] = h;
      tail[tile] = tl;
    }
    __syncwarp();
    r0 = nr0;
    r1 = nr1;
  }
  block_sum_store(pol.l1, l1_part + blockIdx.x);
}

// Rows that span tiles.  A thread per tile with a tail record: when the
// next tile's head ends the row (a row of fewer than about kPrW in-edges),
// the two parts are the row.  Longer rows are walked by the whole warp, 32
// head records at a time, up to the tile the row ends in.  A broken chain
// sets the device error word instead of a rank.
__global__ void __launch_bounds__(kNT)
    k_pr_merge_fix(PrPol pol, PrBufs bufs, const PrCarry *head, const PrCarry *tail,
                   int n_tiles, gas_counters *cnt, double *l1_part) {
  pr_bind(pol, bufs, cnt);
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * kNT;
  bool bad = false;
  for (int t0 = blockIdx.x * kNT + (threadIdx.x & ~31); t0 < n_tiles; t0 += stride) {
    const int t = t0 + lane;
    PrCarry tl{-1, 0, 0.0f, 0.0f};
    if (t < n_tiles) tl = tail[t];
    bool walk = false;
    if (tl.row >= 0) {
      if (t + 1 < n_tiles) {
        const PrCarry h = head[t + 1];
        bad |= h.row != tl.row;
        if (h.done)
          pol.emit(tl.row, two_sum_add(PrVal{tl.s, tl.c}, PrVal{h.s, h.c}));
        else
          walk = true;
      } else {
        bad = true;
      }
    }
    unsigned m = __ballot_sync(0xffffffffu, walk);
    while (m) {
      const int src_lane = __ffs(m) - 1;
      m &= m - 1;
      const int wt = __shfl_sync(0xffffffffu, t, src_lane);
      const int row = __shfl_sync(0xffffffffu, tl.row, src_lane);
      PrVal sum{__shfl_sync(0xffffffffu, tl.s, src_lane),
                __shfl_sync(0xffffffffu, tl.c, src_lane)};
      if (lane != 0) sum = PrVal{0.0f, 0.0f};
      bool done = false;
      for (int c = wt + 1; c < n_tiles && !done; c += 32) {
        const int i = c + lane;
        PrCarry h{-1, 0, 0.0f, 0.0f};
        if (i < n_tiles) h = head[i];
        const unsigned dm = __ballot_sync(0xffffffffu, i < n_tiles && h.done);
        const int stop = dm ? __ffs(dm) - 1 : 31;
        if (lane <= stop && i < n_tiles) {
          bad |= h.row != row;
          sum = two_sum_add(sum, PrVal{h.s, h.c});
        }
        done = dm != 0u;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const PrVal u{__shfl_down_sync(0xffffffffu, sum.s, o),
                      __shfl_down_sync(0xffffffffu, sum.c, o)};
        sum = two_sum_add(sum, u);
      }
      if (lane == 0) {
        if (done)
          pol.emit(row, sum);
        else
          bad = true;
      }
    }
  }
  if (bad) atomicExch(&cnt->error, (int32_t)GAS_ERR_DEVICE);
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
    if (fix_n) *fix_n = 0;  // the fixup of this iteration has run
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
  int32_t *tile_row;
  PrCarry *head, *tail;
  int n_tiles;
  int merge_grid;
  int fix_grid;
  double *residual;
};

gas_status_t pr_body(gas_engine *e, cudaStream_t cs,
                     cudaGraphConditionalHandle h, void *vctx) {
  PrCtx *c = static_cast<PrCtx *>(vctx);
  // algorithmic bytes of one iteration: per edge its source index and the
  // source's contribution; per vertex offsets, old and new rank, new
  // contribution
  gas::prof_begin(e, cs, gas::kProfPagerank, 8LL * e->nE + 16LL * e->nV);
  k_pr_merge<<<c->merge_grid, kNT, 0, cs>>>(c->pol, c->bufs, e->csc_off, e->nV, e->nE,
                                            c->tile_row, c->n_tiles, c->head, c->tail,
                                            e->cnt, e->pr_l1);
  k_pr_merge_fix<<<c->fix_grid, kNT, 0, cs>>>(c->pol, c->bufs, c->head, c->tail, c->n_tiles,
                                              e->cnt, e->pr_l1 + c->merge_grid);
  gas::prof_end(e, cs);
  k_pr_finish<<<1, kNT, 0, cs>>>(e->pr_l1, c->merge_grid + c->fix_grid, c->residual + 1,
                                 e->cnt, c->residual, nullptr, h, e->in_graph ? 1 : 0);
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
  const long long path = (long long)nV + e->nE;
  c.n_tiles = (int)((path + kPrW - 1) / kPrW);
  if (!e->pr_tile_row || e->pr_tile_cap < c.n_tiles) {
    if (e->pr_tile_row) cudaFree(e->pr_tile_row);
    if (e->pr_head) cudaFree(e->pr_head);
    if (e->pr_tail) cudaFree(e->pr_tail);
    e->pr_tile_row = nullptr;
    e->pr_head = e->pr_tail = nullptr;
    e->pr_tile_cap = 0;
    if (e->graphs[kGraphPagerank]) cudaGraphExecDestroy(e->graphs[kGraphPagerank]);
    e->graphs[kGraphPagerank] = nullptr;
    CUDA_TRY(cudaMalloc(&e->pr_tile_row, ((size_t)c.n_tiles + 1) * 4));
    CUDA_TRY(cudaMalloc(&e->pr_head, (size_t)c.n_tiles * sizeof(PrCarry)));
    CUDA_TRY(cudaMalloc(&e->pr_tail, (size_t)c.n_tiles * sizeof(PrCarry)));
    e->pr_tile_cap = c.n_tiles;
  }
  c.tile_row = e->pr_tile_row;
  c.head = static_cast<PrCarry *>(e->pr_head);
  c.tail = static_cast<PrCarry *>(e->pr_tail);
  int per_sm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pr_merge, kNT, 0));
  c.merge_grid = e->num_sms * (per_sm > 0 ? per_sm : 1);  // resident CTAs only
  // a thread per tile record, at most 16 CTAs per SM: the records' loads
  // are dependent chains, so they want many threads in flight
  c.fix_grid = (int)std::min<long long>(16LL * e->num_sms,
                                        std::max(1, (c.n_tiles + kNT - 1) / kNT));
  const int nparts = c.merge_grid + c.fix_grid;
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
  k_pr_tiles<<<gas::engine_grid(c.n_tiles + 1, kNT, 2 * e->num_sms), kNT, 0, S(stream)>>>(
      e->csc_off, nV, e->nE, c.n_tiles, e->pr_tile_row);
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
    stats->kernel_launches = 3 * cnt.iteration + 3;
    stats->edges_processed = (int64_t)cnt.iteration * e->nE;
    stats->residual = resid;
    stats->graph_launches = host_loop ? 0 : 1;
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
