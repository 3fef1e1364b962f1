// gas_small.cu -- BFS on small graphs as one persistent kernel.
//
// For a graph of a few hundred thousand vertices every BFS level is a few
// microseconds of work, and the fast schedule's per-level cost -- a WHILE
// iteration of the loop graph and its five kernel nodes -- is most of the
// run.  Here one cooperative launch (every CTA resident) runs all levels:
// the same level sets as run() (the reference's pull-over-active loop,
// refgas.h:143-214 with bfs.cu:58-71's apply), chosen top-down or bottom-up
// per level by the same direction rule as the fast schedule (bottom-up while
// the frontier's out-edges exceed E/16; PULL forces bottom-up, and PUSH
// keeps the fast schedule), with a grid barrier between levels.
//
//   level 0      apply over the caller's active set: unvisited vertices get
//                depth 0 and form C_0;
//   top-down     a warp per frontier bitmap word, its lanes over each light
//                member's out-edges; members with more than kSbHeavy
//                out-edges are listed instead and, after a barrier, their
//                edges are spread over every thread of the grid.  An
//                unvisited target is claimed with atomicCAS (-1 -> level), so
//                exactly one thread adds it to C_{k+1};
//   bottom-up    a thread per unvisited vertex scans its in-edges for a member
//                of C_k, the first alone and then four at a time (independent
//                loads), and stops at the first found.
//
// Iteration k+1 exists iff C_k has an out-edge (A_{k+1} = N(C_k)), so the
// count equals run()'s.  Frontiers are bitmaps in three rotating buffers (a
// level reads one, fills the next and clears the third, so a bottom-up level
// needs one barrier, a top-down level two).  Data written during the kernel
// by other SMs (depths, bitmaps, the heavy list) is read with L2-only loads,
// since L1 is not coherent across SMs.  The barrier's wait is bounded: past
// the limit it raises an error word and every CTA leaves the kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "gas.h"
#include "gas_engine_impl.h"
#include "gas_grid.cuh"
#include "gas_internal.h"
#include "gas_sched.h"

namespace {

constexpr int kSbNT = 1024;     // one CTA per SM
constexpr int kSbPullDiv = 16;  // the fast schedule's BFS rule
constexpr int kSbHeavy = 256;   // out-edges of a member walked by the grid

using gasgrid::warp_add;

struct SmallCtl {
  gasgrid::Barrier bar;  // bar.err: 1 a barrier wait gave up
  int iterations;
  int n_push, n_pull;
  int n_heavy[2];        // heavy members listed at a level (by level parity)
  long long f_edges[3];  // out-edges of the vertices found at a level
  long long bytes;       // algorithmic bytes (profiling)
};

template <bool kCount>
__global__ void __launch_bounds__(kSbNT, 1)
    k_bfs_small(const int32_t *__restrict__ csr_off, const int32_t *__restrict__ csr_dst,
                const int32_t *__restrict__ csc_off, const int32_t *__restrict__ csc_src,
                int32_t *depth, const int32_t *__restrict__ act, int n_act, uint32_t *bits,
                int32_t *heavy, int nW, int nV, long long nE, int forced, int max_iter,
                SmallCtl *c, gas_counters *cnt) {
  // a barrier wait that gave up: every CTA leaves; the error goes straight
  // to the engine's counters (the epilogue below does not run)
#define SB_SYNC()                                                     \
  do {                                                                \
    if (!gasgrid::barrier(&c->bar)) {                                 \
      if (threadIdx.x == 0) atomicExch(&cnt->error, (int)GAS_ERR_DEVICE); \
      return;                                                         \
    }                                                                 \
  } while (0)
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31, gwarp = tid >> 5, nwarps = nthr >> 5;
  long long found = 0, bytes = 0;
  // level 0: the active set's unvisited vertices
  for (int i = tid; i < n_act; i += nthr) {
    const int v = __ldg(act + i);
    if (kCount) bytes += 8;
    if (depth[v] == -1) {
      depth[v] = 0;
      atomicOr(bits + (v >> 5), 1u << (v & 31));
      found += __ldg(csr_off + v + 1) - __ldg(csr_off + v);
    }
  }
  warp_add(found, &c->f_edges[0]);
  SB_SYNC();
  int it = 1;
  // the cap stays in each CTA: marked in the barrier's error word, a CTA
  // still leaving the previous barrier would read it as a failed wait
  bool capped = false;
  for (int k = 0;; ++k) {
    const int cur = k % 3, nxt = (k + 1) % 3, old = (k + 2) % 3;
    const long long fe = *(volatile long long *)&c->f_edges[cur];
    if (fe == 0) break;  // A_{k+1} = N(C_k) is empty
    if (it >= max_iter) {  // every CTA stops here at the same level
      capped = true;
      break;
    }
    ++it;
    const int level = k + 1;
    const bool pull = forced == 2 || (forced == 0 && fe * kSbPullDiv > nE);
    const uint32_t *F = bits + (size_t)cur * nW;
    uint32_t *N = bits + (size_t)nxt * nW;
    uint32_t *O = bits + (size_t)old * nW;
    // the buffers of level k-1 were last read before the previous barrier
    for (int w = tid; w < nW; w += nthr) O[w] = 0u;
    if (tid == 0) {
      c->f_edges[old] = 0;
      // the next level's heavy count: last read at level k-1, before the
      // barrier that ended it; the next level appends after this one ends
      c->n_heavy[(k + 1) & 1] = 0;
    }
    int *n_heavy = &c->n_heavy[k & 1];
    found = 0;
    if (!pull) {
      for (int w = gwarp; w < nW; w += nwarps) {
        uint32_t m = __ldcg(F + w);
        while (m) {
          const int u = (w << 5) + __ffs(m) - 1;
          m &= m - 1;
          const int b = __ldg(csr_off + u), e1 = __ldg(csr_off + u + 1);
          if (e1 - b > kSbHeavy) {
            if (lane == 0) heavy[atomicAdd(n_heavy, 1)] = u;
            continue;
          }
          if (kCount && lane == 0) bytes += 12 + 8LL * (e1 - b);
          for (int i = b + lane; i < e1; i += 32) {
            const int v = __ldg(csr_dst + i);
            if (__ldcg(depth + v) == -1 && atomicCAS(depth + v, -1, level) == -1) {
              atomicOr(N + (v >> 5), 1u << (v & 31));
              found += __ldg(csr_off + v + 1) - __ldg(csr_off + v);
            }
          }
        }
      }
      // the heavy members: every thread of the grid over their edges
      SB_SYNC();
      const int nh = *(volatile int *)n_heavy;
      for (int h = 0; h < nh; ++h) {
        const int u = __ldcg(heavy + h);
        const int b = __ldg(csr_off + u), e1 = __ldg(csr_off + u + 1);
        if (kCount && tid == 0) bytes += 12 + 8LL * (e1 - b);
        for (int i = b + tid; i < e1; i += nthr) {
          const int v = __ldg(csr_dst + i);
          if (__ldcg(depth + v) == -1 && atomicCAS(depth + v, -1, level) == -1) {
            atomicOr(N + (v >> 5), 1u << (v & 31));
            found += __ldg(csr_off + v + 1) - __ldg(csr_off + v);
          }
        }
      }
    } else {
      for (int v = tid; v < nV; v += nthr) {
        if (kCount) bytes += 4;
        if (__ldcg(depth + v) != -1) continue;
        const int b = __ldg(csc_off + v), e1 = __ldg(csc_off + v + 1);
        if (kCount) bytes += 8;
        // the first in-edge alone (sources are in id order and low ids are
        // the hubs, so it is the likeliest parent), then four at a time
        bool hit = false;
        if (b < e1) {
          const int u = __ldg(csc_src + b);
          hit = (__ldcg(F + (u >> 5)) >> (u & 31)) & 1u;
          if (kCount) bytes += 8;
        }
        for (int i = b + 1; i < e1 && !hit; i += 4) {
          int u[4];
          uint32_t f[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) u[j] = i + j < e1 ? __ldg(csc_src + i + j) : -1;
#pragma unroll
          for (int j = 0; j < 4; ++j) f[j] = u[j] >= 0 ? __ldcg(F + (u[j] >> 5)) : 0u;
#pragma unroll
          for (int j = 0; j < 4; ++j) hit |= u[j] >= 0 && ((f[j] >> (u[j] & 31)) & 1u);
          if (kCount) bytes += 8LL * min(4, e1 - i);
        }
        if (hit) {
          depth[v] = level;
          atomicOr(N + (v >> 5), 1u << (v & 31));
          found += __ldg(csr_off + v + 1) - __ldg(csr_off + v);
        }
      }
    }
    warp_add(found, &c->f_edges[nxt]);
    if (tid == 0) {
      if (pull)
        ++c->n_pull;
      else
        ++c->n_push;
    }
    SB_SYNC();
  }
  if (kCount) warp_add(bytes, &c->bytes);
  // the next run finds the bitmaps clear (nothing reads them any more)
  for (int w = tid; w < 3 * nW; w += nthr) bits[w] = 0u;
  if (tid == 0) {
    // the engine's counters, as the fast schedule leaves them
    // a wait that gave up in another CTA has written GAS_ERR_DEVICE already
    const bool failed = *(volatile int *)&c->bar.err != 0;
    cnt->iteration = it;
    cnt->n_push = c->n_push;
    cnt->n_pull = c->n_pull;
    if (!failed) cnt->error = capped ? GAS_ERR_ITER_CAP : 0;
    if (!failed && !capped) cnt->n_active = 0;
    // and the control word clear for the next run: its counts are read by
    // no thread after the loop (a thread still to test f_edges reads 0 and
    // leaves as well)
    c->iterations = it;
    c->n_push = c->n_pull = 0;
    c->n_heavy[0] = c->n_heavy[1] = 0;
    c->f_edges[0] = c->f_edges[1] = c->f_edges[2] = 0;
  }
#undef SB_SYNC
}

}  // namespace

namespace gas {

bool bfs_small_eligible(const gas_engine *e, gas_schedule_t schedule) {
  const char *v = getenv("GAS_BFS_SMALL");
  if (v && v[0] == '0') return false;
  // forced top-down walks big frontiers a warp per bitmap word here, where
  // the fast schedule balances their edges over warp slabs: it keeps that
  return e->prog == GAS_PROG_BFS && schedule != GAS_SCHED_PUSH && !e->edges_on_host &&
         e->nV <= kBfsSmallMaxV && e->nV > 0;
}

gas_status_t run_bfs_small(gas_engine *e, gas_schedule_t schedule, int32_t max_iterations,
                           gas_run_stats *stats, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const int nW = (e->nV + 31) / 32;
  if (!e->sb_bits) CUDA_TRY(cudaMalloc(&e->sb_bits, (size_t)3 * nW * sizeof(uint32_t)));
  if (!e->sb_ctl) CUDA_TRY(cudaMalloc(&e->sb_ctl, sizeof(SmallCtl)));
  if (!e->sb_heavy) CUDA_TRY(cudaMalloc(&e->sb_heavy, (size_t)e->nV * sizeof(int32_t)));
  SmallCtl *ctl = static_cast<SmallCtl *>(e->sb_ctl);
  const bool count = e->profiling;
  void *fn = count ? (void *)k_bfs_small<true> : (void *)k_bfs_small<false>;
  int per_sm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSbNT, 0));
  if (per_sm < 1) return fail(GAS_ERR_CUDA, "small BFS: no resident CTA");
  const int grid = e->num_sms;  // one CTA per SM: the barrier's atomics are per CTA
  // the kernel leaves its bitmaps and control word clear; they are cleared
  // here after allocation, after a run that failed, and when bytes count
  if (!e->sb_clean || count) {
    CUDA_TRY(cudaMemsetAsync(e->sb_bits, 0, (size_t)3 * nW * sizeof(uint32_t), s));
    CUDA_TRY(cudaMemsetAsync(ctl, 0, sizeof(SmallCtl), s));
  }
  e->sb_clean = false;
  gas_counters *cnt = e->cnt;
  const int32_t *csr_off = e->csr_off, *csr_dst = e->csr_dst, *csc_off = e->csc_off,
                *csc_src = e->csc_src;
  int32_t *depth = static_cast<int32_t *>(e->vd);
  const int32_t *act = e->act;
  int n_act = e->n_active, nV = e->nV;
  uint32_t *bits = e->sb_bits;
  int32_t *heavy = e->sb_heavy;
  long long nE = e->nE;
  int forced = schedule == GAS_SCHED_PULL ? 2 : 0;
  int max_iter = max_iterations;
  int nw = nW;
  void *args[] = {&csr_off, &csr_dst, &csc_off, &csc_src,  &depth, &act, &n_act, &bits,
                  &heavy,   &nw,      &nV,      &nE,      &forced, &max_iter, &ctl, &cnt};
  if (count) prof_begin(e, s, kProfPush, 0);
  CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kSbNT), args, 0, s));
  prof_end(e, s);
  if (count) {
    SmallCtl h;
    CUDA_TRY(cudaMemcpyAsync(&h, ctl, sizeof(h), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    e->prof_bytes_pending = h.bytes;
    prof_collect(e);
  }
  gas_counters c;
  GAS_TRY(engine_sync_counts(e, stream));
  c = *e->h_cnt;
  e->sb_clean = c.error == 0 || c.error == GAS_ERR_ITER_CAP;
  if (stats) {
    stats->iterations = c.iteration;
    stats->push_iters = c.n_push;
    stats->pull_iters = c.n_pull;
    stats->kernel_launches = 1;
    stats->graph_launches = 0;
  }
  e->level = c.iteration;
  e->active_full = false;
  return loop_status(e, c, stream);
}

}  // namespace gas
