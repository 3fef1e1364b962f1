// gas_batch.cu -- many BFS sources and personalized-PageRank seeds over many
// graphs in one CUDA-graph launch (no reference counterpart).
//
// The graphs are concatenated into one disjoint union graph (vertex ids
// offset per graph), so one device loop serves every instance:
//
//   * multi-source BFS: lane l of a vertex belongs to source l of the
//     vertex's own graph (graphs are disjoint, so lanes of different graphs
//     never meet).  vn[v] = {visited, next}, two 32-bit lane masks in one
//     8-byte record, so a push reads both with one access.  One level
//     pushes every queued vertex's new-lane mask to its out-neighbours
//     (atomicOr, pre-filtered by visited), marking touched vertices in a
//     bitmap; a two-pass compaction over that bitmap writes the level into
//     depth[v][l] for every new lane, folds the lanes into visited and
//     builds the next queue (lane mask, inclusive out-edge ends, CSR offset).
//     Depths equal those of one BFS per source.
//   * multi-source SSSP (integer weights, unweighted graphs count 1 per
//     edge): dist[v][l] rows of LS = L rounded up to 4 lanes, cmask[v] the
//     lanes of v that changed in the current iteration.  One bulk-synchronous
//     iteration pushes every queued vertex's changed lanes along its
//     out-edges: the destination's whole row is read once (one 32-byte load
//     for 8 lanes) for all lanes, a lane improves with atomicMin when its
//     candidate is below the value read, and the improved lanes go into
//     cmask and the vertex into the touched bitmap (reductions).  The compaction snapshots
//     each queued vertex's row.  Per lane, distances and iteration counts
//     equal those of one SSSP per source.
//   * multi-seed personalized PageRank, r_l = (1-d) e_{s_l} + d A^T D^-1 r_l
//     for every lane l at once: ranks and contributions are [V][L] rows, so
//     the L lanes of an in-edge's source are one contiguous 4L-byte read.
//     The CSC edge range is cut into pieces of P edges (P autotuned); a group
//     of L threads (one per lane) folds a piece in edge order with FP32
//     two-sum compensation, finishing every row that lies inside the piece;
//     rows cut by piece boundaries leave per-piece partials that a second
//     pass folds in piece order.  The sums are deterministic.  The loop runs
//     until the largest per-lane FP64 L1 residual is <= tol.
//
// The loops are WHILE nodes of one CUDA graph (BFS, SSSP, then PPR), each
// preceded by its prologue; a run is one cudaGraphLaunch.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "gas.h"
#include "gas_device.cuh"
#include "gas_engine_impl.h"
#include "gas_internal.h"
#include "gas_sched.h"

using gasdev::kNT;
using gas::fail;

namespace {

inline cudaStream_t S(void *s) { return (cudaStream_t)s; }

constexpr int kMaxLanes = GAS_BATCH_MAX_LANES;

// Device parameters of a run (read by the captured kernels, so that one
// instantiated graph serves any sources, seeds, damping, tolerance and caps).
struct BatchParams {
  double damping;
  double tol;
  int32_t bfs_max_iter;
  int32_t ppr_max_iter;
  int32_t n_sources;  // G * bfs_lanes
  int32_t sssp_max_iter;
  int32_t n_sssp_sources;  // G * sssp_lanes
  int32_t pad;
};

__device__ __forceinline__ void set_cond(gas_counters *cnt, bool more, int it,
                                         cudaGraphConditionalHandle h, int in_graph) {
  if (more && it >= cnt->max_iter) cnt->error = GAS_ERR_ITER_CAP;
  cnt->cond = (more && it < cnt->max_iter) ? 1 : 0;
  if (in_graph) cudaGraphSetConditional(h, cnt->cond);
}

__global__ void k_b_reset(gas_counters *cnt, const BatchParams *prm, int which,
                          unsigned long long *edges) {
  cnt->iteration = 0;
  cnt->error = 0;
  cnt->cond = 0;
  cnt->n_changed = 0;
  cnt->n_scatter_edges = 0;
  cnt->max_iter = which == 0 ? prm->bfs_max_iter
                 : which == 1 ? prm->ppr_max_iter : prm->sssp_max_iter;
  if (edges) *edges = 0ull;
}

// ---------------------------------------------------------------------------
// multi-source BFS
// ---------------------------------------------------------------------------
struct MsPushPol {
  typedef int32_t Val;
  static constexpr bool kMapNeedsVertex = false;
  const int32_t *csr_dst;
  const int32_t *q_mask;
  uint32_t *vn;  // [V][2]: visited, next
  uint32_t *tbits;
  __device__ Val zero() const { return 0; }
  __device__ Val reduce(Val a, Val) const { return a; }
  __device__ Val map(int, int, int) const { return 0; }
  __device__ void emit(int, int, Val) const {}
  // a: queue position of the pushing vertex, pos: CSR position of the edge.
  // visited does not change during the push; next[v] starts the push at 0
  // and only gains bits, so lanes already seen in it (a plain, possibly
  // stale load) need no atomic; every thread that adds lanes also marks v
  // as touched (both reductions, no thread waits for a result).
  __device__ __forceinline__ void visit(int a, int, int pos) const {
    const int v = __ldg(csr_dst + pos);
    const uint2 p = reinterpret_cast<const uint2 *>(vn)[v];
    const uint32_t m = (uint32_t)__ldg(q_mask + a) & ~p.x;
    if (m && (p.y & m) != m) {
      atomicOr(vn + 2 * (size_t)v + 1, m);  // fire-and-forget; the touched bit is idempotent
      atomicOr(tbits + ((uint32_t)v >> 5), 1u << (v & 31));
    }
  }
};

__global__ void __launch_bounds__(kNT)
    k_ms_push(MsPushPol pol, gasdev::SlabSource src) {
  gasdev::slab_loop<MsPushPol, false>(pol, src, nullptr, nullptr, nullptr, nullptr, nullptr);
}

// Level 0: every (graph, lane) source.
__global__ void k_ms_seed(const int32_t *src_global, const BatchParams *prm, int L,
                          uint32_t *vn, uint32_t *tbits) {
  const int n = prm->n_sources;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int v = src_global[i];
    if (v < 0) continue;
    atomicOr(vn + 2 * (size_t)v + 1, 1u << (i % L));
    atomicOr(tbits + ((uint32_t)v >> 5), 1u << (v & 31));
  }
}

// The touched-vertex traversal shared by the two compaction passes: a warp
// owns a run of 16 words of the touched bitmap (lanes 0..15 load them) and
// walks it in two rounds of 8 words, skipping a round whose words are all
// clear; lane l takes vertex 32 w + l of each word, and a round's 8 words'
// loads are issued before any is used.  For a touched vertex: its new lanes
// and out-edge range.  The count pass keeps each warp's totals, so the
// write passes take their offsets without counting again.
constexpr int kMsWarpWords = 16;
constexpr int kMsRound = 8;
constexpr int kMsWarps = kNT / 32;
constexpr int kMsBlockWords = kMsWarpWords * kMsWarps;  // 128 words

struct MsRound {
  uint32_t nw[kMsRound];  // new lanes (0: not touched or nothing new)
  int off[kMsRound];
  int deg[kMsRound];
};

// The lane's word of the warp's run (lanes 0..15; 0 past the bitmap).
__device__ __forceinline__ uint32_t ms_word(const uint32_t *tbits, int nW, int w0) {
  const int lane = threadIdx.x & 31;
  return lane < kMsWarpWords && w0 + lane < nW ? tbits[w0 + lane] : 0u;
}

__device__ __forceinline__ bool ms_round_live(unsigned nz, int r) {
  return ((nz >> r) & ((1u << kMsRound) - 1u)) != 0u;
}

// Round r (words w0 + r .. w0 + r + 7).  next: the SSSP's changed-lane
// words; vn (BFS, next unused): the {visited, next} pairs, new lanes =
// next & ~visited.
__device__ __forceinline__ void ms_round_load(uint32_t myword, const uint32_t *next,
                                              const uint32_t *vn, const int32_t *csr_off,
                                              int w0, int r, MsRound &m) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < kMsRound; ++i) {
    const uint32_t word = __shfl_sync(0xffffffffu, myword, r + i);
    m.nw[i] = 0u;
    m.off[i] = 0;
    m.deg[i] = 0;
    if ((word >> lane) & 1u) {
      const int v = (w0 + r + i) * 32 + lane;
      if (vn) {
        const uint2 p = reinterpret_cast<const uint2 *>(vn)[v];
        m.nw[i] = p.y & ~p.x;
      } else {
        m.nw[i] = next[v];
      }
      m.off[i] = csr_off[v];
      m.deg[i] = csr_off[v + 1] - m.off[i];
    }
  }
}

// Pass 1: per block (queue entries, out-edges) for the spine and per warp
// for the write pass; with lanes_active, also the OR of the new lanes of the
// queue's entries (the SSSP loop).
__global__ void __launch_bounds__(kNT)
    k_ms_count(const uint32_t *tbits, const uint32_t *next, const uint32_t *vn,
               const int32_t *csr_off, int nW, int32_t *part, int2 *wpart,
               uint32_t *lanes_active) {
  __shared__ int s_q[kMsWarps], s_d[kMsWarps];
  __shared__ uint32_t s_l[kMsWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w0 = (blockIdx.x * kMsWarps + warp) * kMsWarpWords;
  const uint32_t myword = ms_word(tbits, nW, w0);
  const unsigned nz = __ballot_sync(0xffffffffu, myword != 0u);
  int q = 0, d = 0;
  uint32_t lanes = 0u;
#pragma unroll 1
  for (int r = 0; r < kMsWarpWords; r += kMsRound) {
    if (!ms_round_live(nz, r)) continue;  // warp-uniform
    MsRound m;
    ms_round_load(myword, next, vn, csr_off, w0, r, m);
#pragma unroll
    for (int i = 0; i < kMsRound; ++i) {
      const bool in = m.nw[i] && m.deg[i] > 0;
      q += in;
      d += in ? m.deg[i] : 0;
      if (m.deg[i] > 0) lanes |= m.nw[i];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    q += __shfl_xor_sync(0xffffffffu, q, o);
    d += __shfl_xor_sync(0xffffffffu, d, o);
    lanes |= __shfl_xor_sync(0xffffffffu, lanes, o);
  }
  if (lane == 0) {
    s_q[warp] = q;
    s_d[warp] = d;
    s_l[warp] = lanes;
    wpart[blockIdx.x * kMsWarps + warp] = make_int2(q, d);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int tq = 0, td = 0;
    uint32_t tl = 0u;
    for (int k = 0; k < kMsWarps; ++k) {
      tq += s_q[k];
      td += s_d[k];
      tl |= s_l[k];
    }
    part[2 * blockIdx.x] = tq;
    part[2 * blockIdx.x + 1] = td;
    if (lanes_active && tl) atomicOr(lanes_active, tl);
  }
}

// The warp's first queue entry and out-edge offset: its block's (scanned by
// the spine) plus the totals of the block's earlier warps.
__device__ __forceinline__ int2 ms_warp_base(const int32_t *part, const int2 *wpart,
                                             int warp) {
  int2 b = make_int2(part[2 * blockIdx.x], part[2 * blockIdx.x + 1]);
  for (int k = 0; k < warp; ++k) {
    const int2 t = wpart[blockIdx.x * kMsWarps + k];
    b.x += t.x;
    b.y += t.y;
  }
  return b;
}

// Pass 2: depths of the new lanes (level = the iteration the spine just
// counted), visited, the next queue and the push's chunk partition at the
// chunk size the spine chose; clears next and the touched bitmap.
__global__ void __launch_bounds__(kNT, 5)
    k_ms_write(uint32_t *tbits, uint32_t *vn, const int32_t *csr_off,
               int nW, const int32_t *part, const int2 *wpart, int L, const gas_counters *cnt,
               int32_t *depth, int32_t *q_mask, int32_t *q_end, int32_t *q_delta,
               int32_t *chunk_row) {
  // rows spanning many chunks (hubs), written by the whole warp at the end
  constexpr int kBig = 64;
  __shared__ int3 s_big[kMsWarps][kBig];
  __shared__ int s_nbig[kMsWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w0 = (blockIdx.x * kMsWarps + warp) * kMsWarpWords;
  const uint32_t myword = ms_word(tbits, nW, w0);
  const unsigned nz = __ballot_sync(0xffffffffu, myword != 0u);
  if (!nz) return;  // warp-uniform: nothing touched in the run
  const int level = cnt->iteration;
  const int cl = cnt->push_chunk_log2;
  if (lane == 0) s_nbig[warp] = 0;
  __syncwarp();
  const int2 base = ms_warp_base(part, wpart, warp);
  int bq = base.x, bd = base.y;
  if (myword) tbits[w0 + lane] = 0u;
#pragma unroll 1
  for (int r = 0; r < kMsWarpWords; r += kMsRound) {
    if (!ms_round_live(nz, r)) continue;  // warp-uniform
    MsRound m;
    ms_round_load(myword, nullptr, vn, csr_off, w0, r, m);
#pragma unroll
    for (int i = 0; i < kMsRound; ++i) {
      const int v = (w0 + r + i) * 32 + lane;
      const uint32_t word = __shfl_sync(0xffffffffu, myword, r + i);
      if (!word) continue;  // warp-uniform
      const bool touched = (word >> lane) & 1u;
      const uint32_t nw = m.nw[i];
      if (touched) vn[2 * (size_t)v + 1] = 0u;
      if (nw) {
        vn[2 * (size_t)v] |= nw;
        for (uint32_t k = nw; k; k &= k - 1) depth[(size_t)v * L + (__ffs(k) - 1)] = level;
      }
      const int deg = nw ? m.deg[i] : 0;
      const unsigned qb = __ballot_sync(0xffffffffu, deg > 0);
      if (!qb) continue;
      int incl = deg;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (deg > 0) {
        const int pos = bq + __popc(qb & ((1u << lane) - 1u));
        const int end = bd + incl;
        q_mask[pos] = (int32_t)nw;
        q_end[pos] = end;
        q_delta[pos] = m.off[i] - (end - deg);
        // chunk partition of the next push (chunks starting in this range)
        const int c0 = (end - deg + (1 << cl) - 1) >> cl, c1 = (end + (1 << cl) - 1) >> cl;
        int slot = kBig;
        if (c1 - c0 > 4) slot = atomicAdd(&s_nbig[warp], 1);
        if (slot < kBig)
          s_big[warp][slot] = make_int3(pos, c0, c1);
        else
          for (int c = c0; c < c1; ++c) chunk_row[c] = pos;
      }
      bq += __popc(qb);
      bd += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  __syncwarp();
  const int nbig = min(s_nbig[warp], kBig);
  for (int k = 0; k < nbig; ++k) {
    const int3 rr = s_big[warp][k];
    for (int c = rr.y + lane; c < rr.z; c += 32) chunk_row[c] = rr.x;
  }
}

// ---------------------------------------------------------------------------
// multi-source SSSP
// ---------------------------------------------------------------------------
constexpr int32_t kSsspInf = INT_MAX - 100000;  // the SSSP Program's gatherZero

struct MssPushPol {
  typedef int32_t Val;
  static constexpr bool kMapNeedsVertex = false;
  const int32_t *csr_dst;
  const int32_t *csr_w;   // null: every edge weighs 1
  const int32_t *q_mask;  // [queue] lanes that changed
  const int32_t *q_vals;  // [queue][LS] row at the end of the last iteration
  int32_t *dist;          // [V][LS]
  uint32_t *cmask;        // [V] lanes changed in this iteration
  uint32_t *tbits;
  int LS;
  __device__ Val zero() const { return 0; }
  __device__ Val reduce(Val a, Val) const { return a; }
  __device__ Val map(int, int, int) const { return 0; }
  __device__ void emit(int, int, Val) const {}
  // The row read is a plain load: a value it returns was held by the lane
  // during this iteration, so a candidate below it lowers the lane's final
  // value under its start value (the lane changed) and a candidate at or
  // above it cannot lower the final value.
  __device__ __forceinline__ void visit(int a, int, int pos) const {
    const int v = __ldg(csr_dst + pos);
    const long long w = csr_w ? __ldg(csr_w + pos) : 1;
    const uint32_t m = (uint32_t)__ldg(q_mask + a);
    const int4 *cur4 = reinterpret_cast<const int4 *>(dist + (size_t)v * LS);
    const int4 *qv4 = reinterpret_cast<const int4 *>(q_vals + (size_t)a * LS);
    int32_t *row = dist + (size_t)v * LS;
    uint32_t nb = 0u;
    for (int c = 0; c < (LS >> 2); ++c) {
      const uint32_t mc = (m >> (4 * c)) & 0xFu;
      if (!mc) continue;
      const int4 cu = cur4[c];
      const int4 qv = __ldg(qv4 + c);
      const int cur[4] = {cu.x, cu.y, cu.z, cu.w};
      const int val[4] = {qv.x, qv.y, qv.z, qv.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (!((mc >> k) & 1u)) continue;
        const long long cl = (long long)val[k] + w;
        const int cand = cl > kSsspInf ? kSsspInf : (int)cl;
        if (cand < cur[k]) {
          atomicMin(row + 4 * c + k, cand);
          nb |= 1u << (4 * c + k);
        }
      }
    }
    if (nb && (cmask[v] & nb) != nb) {
      atomicOr(cmask + v, nb);  // reductions: the touched bit is idempotent
      atomicOr(tbits + ((uint32_t)v >> 5), 1u << (v & 31));
    }
  }
};

// 32-byte row loads (one instruction, one sector): the row must be 32-byte
// aligned.  row8 is a plain load (the row changes during the push), nc8 a
// read-only one.
__device__ __forceinline__ void row8(const int32_t *p, int (&r)[8]) {
  asm volatile("ld.global.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7])
               : "l"(p));
}
__device__ __forceinline__ void nc8(const int32_t *p, int (&r)[8]) {
  asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "l"(p));
}

// Rows of at most 8 lanes (NC = 1 or 2 16-byte chunks): the same push split
// into probe (the edge's loads and the destination row) and commit, so that
// both slabs' row reads are in flight before either slab's updates.  Every
// lane of the row is tried, not only the changed ones: a lane of u that did
// not change in the last iteration already pushed its value along this edge
// when it last changed, so its candidate is at or above the destination's
// value at the start of this iteration (and of any value read during it)
// and changes nothing.  Weights are at most 100000, as the SSSP Program's
// gatherZero assumes, so val + w does not overflow.
template <int NC>
struct MssPushPolStaged {
  typedef int32_t Val;
  static constexpr bool kMapNeedsVertex = false;
  const int32_t *csr_dst;
  const int32_t *csr_w;
  const int32_t *q_vals;
  int32_t *dist;
  uint32_t *cmask;
  uint32_t *tbits;
  __device__ Val zero() const { return 0; }
  __device__ Val reduce(Val a, Val) const { return a; }
  __device__ Val map(int, int, int) const { return 0; }
  __device__ void emit(int, int, Val) const {}
  struct Probe {
    int v, w, a;  // v < 0: no edge
    int cur[4 * NC];
  };
  __device__ __forceinline__ Probe probe(bool valid, int a, int, int pos) const {
    Probe p;
    p.v = -1;
    p.w = 0;
    p.a = a;
    if (valid) {
      p.v = __ldg(csr_dst + pos);
      p.w = csr_w ? __ldg(csr_w + pos) : 1;
      const int32_t *r = dist + (size_t)p.v * (4 * NC);
      if constexpr (NC == 2) {
        row8(r, p.cur);
      } else {
        const int4 c4 = *reinterpret_cast<const int4 *>(r);
        p.cur[0] = c4.x;
        p.cur[1] = c4.y;
        p.cur[2] = c4.z;
        p.cur[3] = c4.w;
      }
    }
    return p;
  }
  __device__ __forceinline__ void commit(const Probe &p) const {
    if (p.v < 0) return;
    const int32_t *q = q_vals + (size_t)p.a * (4 * NC);
    int val[4 * NC];
    if constexpr (NC == 2) {
      nc8(q, val);
    } else {
      const int4 q4 = __ldg(reinterpret_cast<const int4 *>(q));
      val[0] = q4.x;
      val[1] = q4.y;
      val[2] = q4.z;
      val[3] = q4.w;
    }
    int32_t *row = dist + (size_t)p.v * (4 * NC);
    uint32_t nb = 0u;
#pragma unroll
    for (int k = 0; k < 4 * NC; ++k) {
      const int cand = min(val[k] + p.w, kSsspInf);
      if (cand < p.cur[k]) {
        atomicMin(row + k, cand);
        nb |= 1u << k;
      }
    }
    // the lanes and the touched bit as fire-and-forget reductions (both are
    // idempotent, so no thread waits for an atomic's result); issued
    // without first loading cmask[v] to skip repeats: that dependent load
    // cost more than the repeated reductions (8 lanes at R-MAT scale 22:
    // 0.406 -> 0.370 ms per push)
    if (nb) {
      atomicOr(cmask + p.v, nb);
      atomicOr(tbits + ((uint32_t)p.v >> 5), 1u << (p.v & 31));
    }
  }
};

template <class Pol>
__global__ void __launch_bounds__(kNT) k_mss_push(Pol pol, gasdev::SlabSource src) {
  gasdev::slab_loop<Pol, false>(pol, src, nullptr, nullptr, nullptr, nullptr, nullptr);
}

__global__ void k_mss_init(int32_t *dist, size_t n, uint32_t *lanes_active,
                           int32_t *lane_rounds) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    dist[k] = kSsspInf;
  if (blockIdx.x == 0 && threadIdx.x < kMaxLanes) {
    lane_rounds[threadIdx.x] = 0;
    if (threadIdx.x == 0) *lanes_active = 0u;
  }
}

// Iteration 0: every (graph, lane) source gets distance 0 and is changed.
__global__ void k_mss_seed(const int32_t *src_global, const BatchParams *prm, int L, int LS,
                           int32_t *dist, uint32_t *cmask, uint32_t *tbits) {
  const int n = prm->n_sssp_sources;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int v = src_global[i];
    if (v < 0) continue;
    dist[(size_t)v * LS + i % L] = 0;
    atomicOr(cmask + v, 1u << (i % L));
    atomicOr(tbits + ((uint32_t)v >> 5), 1u << (v & 31));
  }
}

// Pass 2 of the compaction: the next queue (snapshot row, inclusive
// out-edge ends, CSR offset; the changed lanes for rows wider than 8 lanes)
// and the push's chunk partition at the chunk size the spine chose; clears
// cmask and the touched bitmap.
__global__ void __launch_bounds__(kNT, 4)
    k_mss_write(uint32_t *tbits, uint32_t *cmask, const int32_t *csr_off, int nW,
                const int32_t *part, const int2 *wpart, int LS, const int32_t *dist,
                int32_t *q_mask, int32_t *q_vals, int32_t *q_end, int32_t *q_delta,
                int32_t *chunk_row, const gas_counters *cnt) {
  // rows spanning many chunks (hubs), written by the whole warp at the end
  constexpr int kBig = 64;
  __shared__ int3 s_big[kMsWarps][kBig];
  __shared__ int s_nbig[kMsWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w0 = (blockIdx.x * kMsWarps + warp) * kMsWarpWords;
  const uint32_t myword = ms_word(tbits, nW, w0);
  const unsigned nz = __ballot_sync(0xffffffffu, myword != 0u);
  if (!nz) return;  // warp-uniform: nothing touched in the run
  const int cl = cnt->push_chunk_log2;
  if (lane == 0) s_nbig[warp] = 0;
  __syncwarp();
  const int2 base = ms_warp_base(part, wpart, warp);
  int bq = base.x, bd = base.y;
  if (myword) tbits[w0 + lane] = 0u;
#pragma unroll 1
  for (int r = 0; r < kMsWarpWords; r += kMsRound) {
    if (!ms_round_live(nz, r)) continue;  // warp-uniform
    MsRound m;
    ms_round_load(myword, cmask, nullptr, csr_off, w0, r, m);
#pragma unroll
    for (int i = 0; i < kMsRound; ++i) {
      const int v = (w0 + r + i) * 32 + lane;
      const uint32_t word = __shfl_sync(0xffffffffu, myword, r + i);
      if (!word) continue;  // warp-uniform
      if ((word >> lane) & 1u) cmask[v] = 0u;
      const uint32_t nw = m.nw[i];
      const int deg = nw ? m.deg[i] : 0;
      const unsigned qb = __ballot_sync(0xffffffffu, deg > 0);
      if (!qb) continue;
      int incl = deg;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (deg > 0) {
        const int pos = bq + __popc(qb & ((1u << lane) - 1u));
        const int end = bd + incl;
        if (LS > 8) q_mask[pos] = (int32_t)nw;  // rows of up to 8 lanes try every lane
        q_end[pos] = end;
        q_delta[pos] = m.off[i] - (end - deg);
        const int4 *src4 = reinterpret_cast<const int4 *>(dist + (size_t)v * LS);
        int4 *dst4 = reinterpret_cast<int4 *>(q_vals + (size_t)pos * LS);
        for (int c = 0; c < (LS >> 2); ++c) dst4[c] = src4[c];
        const int c0 = (end - deg + (1 << cl) - 1) >> cl, c1 = (end + (1 << cl) - 1) >> cl;
        int slot = kBig;
        if (c1 - c0 > 4) slot = atomicAdd(&s_nbig[warp], 1);
        if (slot < kBig)
          s_big[warp][slot] = make_int3(pos, c0, c1);
        else
          for (int c = c0; c < c1; ++c) chunk_row[c] = pos;
      }
      bq += __popc(qb);
      bd += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  __syncwarp();
  const int nbig = min(s_nbig[warp], kBig);
  for (int k = 0; k < nbig; ++k) {
    const int3 rr = s_big[warp][k];
    for (int c = rr.y + lane; c < rr.z; c += 32) chunk_row[c] = rr.x;
  }
}

// Exclusive scan of the block pairs in one pass (1024 threads, each holding a
// run of ceil(nb / 1024) pairs in registers), then the loop control of the
// BFS and SSSP loops: queue totals, the push's chunk size (512 edges per
// warp, halved down to 64 while there would be fewer than two chunks per
// push warp), the lanes of the new queue (each has one more push to run;
// SSSP only), the WHILE condition.
constexpr int kMssSpineNT = 1024;
constexpr int kMssSpineRegs = 8;

__global__ void __launch_bounds__(kMssSpineNT)
    k_mss_spine(int2 *part, int nb, gas_counters *cnt, int push_warps,
                unsigned long long *edges, uint32_t *lanes_active, int32_t *lane_rounds,
                cudaGraphConditionalHandle h, int in_graph, int first) {
  const int per = (nb + kMssSpineNT - 1) / kMssSpineNT;
  const int b0 = threadIdx.x * per, b1 = min(nb, b0 + per);
  const bool in_regs = per <= kMssSpineRegs;
  int2 x[kMssSpineRegs];
  int sq = 0, sd = 0;
  if (in_regs) {
#pragma unroll
    for (int k = 0; k < kMssSpineRegs; ++k) x[k] = b0 + k < b1 ? part[b0 + k] : make_int2(0, 0);
#pragma unroll
    for (int k = 0; k < kMssSpineRegs; ++k) {
      sq += x[k].x;
      sd += x[k].y;
    }
  } else {
    for (int b = b0; b < b1; ++b) {
      sq += part[b].x;
      sd += part[b].y;
    }
  }
  __shared__ int2 s_w[kMssSpineNT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int iq = sq, id = sd;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int oq = __shfl_up_sync(0xffffffffu, iq, d);
    const int od = __shfl_up_sync(0xffffffffu, id, d);
    if (lane >= d) {
      iq += oq;
      id += od;
    }
  }
  if (lane == 31) s_w[warp] = make_int2(iq, id);
  __syncthreads();
  int pq = iq - sq, pd = id - sd, tq = 0, td = 0;
#pragma unroll 8
  for (int k = 0; k < kMssSpineNT / 32; ++k) {
    const int2 t = s_w[k];
    if (k < warp) {
      pq += t.x;
      pd += t.y;
    }
    tq += t.x;
    td += t.y;
  }
  if (in_regs) {
#pragma unroll
    for (int k = 0; k < kMssSpineRegs; ++k) {
      if (b0 + k < b1) {
        part[b0 + k] = make_int2(pq, pd);
        pq += x[k].x;
        pd += x[k].y;
      }
    }
  } else {
    for (int b = b0; b < b1; ++b) {
      const int2 y = part[b];
      part[b] = make_int2(pq, pd);
      pq += y.x;
      pd += y.y;
    }
  }
  if (threadIdx.x == 0) {
    cnt->n_changed = tq;
    cnt->n_scatter_edges = td;
    int cl = gasdev::kSlabChunkLog2;
    while (cl > gasdev::kSlabChunkMinLog2 && (td >> cl) < 2 * push_warps) --cl;
    cnt->push_chunk_log2 = cl;
    if (lanes_active) {
      const uint32_t la = *lanes_active;
      *lanes_active = 0u;
      for (int l = 0; l < kMaxLanes; ++l)
        if ((la >> l) & 1u) ++lane_rounds[l];
    }
    const int it = first ? 0 : ++cnt->iteration;
    set_cond(cnt, td > 0, it, h, in_graph);
    if (cnt->cond) *edges += (unsigned long long)td;
  }
}

// ---------------------------------------------------------------------------
// multi-seed personalized PageRank
// ---------------------------------------------------------------------------
struct CVal {
  float s, c;
};

// Knuth two-sum: a.s + b.s = s + err exactly; compensations add up in c.
__device__ __forceinline__ CVal two_sum_add(CVal a, CVal b) {
  const float s = __fadd_rn(a.s, b.s);
  const float bp = __fsub_rn(s, a.s);
  const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bp)), __fsub_rn(b.s, bp));
  return CVal{s, __fadd_rn(__fadd_rn(a.c, b.c), err)};
}

struct PprArgs {
  const int32_t *csc_off, *csc_src, *csr_off;
  const int32_t *first_row;  // [n_pieces] first row with an edge in the piece
  int32_t n_pieces, P, E, L, G;
  const int32_t *fix;        // [n_fix][3] (row, first piece, last piece):
  int32_t n_fix;             // rows cut by pieces, then rows without
  int32_t n_split;           // in-edges (first piece -1) from n_split on
  CVal *head, *tail;         // [n_pieces][L] partials of cut rows
  float *rank[2], *contrib[2];
  const uint32_t *seed_mask;
  const BatchParams *prm;
  gas_counters *cnt;
};

struct PprLane {
  const float *contrib, *rank_old;
  float *rank_new, *contrib_new;
  float d, base;
  int l;
  bool on;
};

__device__ __forceinline__ PprLane ppr_lane(const PprArgs &a) {
  PprLane o;
  const int p = a.cnt->iteration & 1;
  o.contrib = a.contrib[p];
  o.rank_old = a.rank[p];
  o.rank_new = a.rank[p ^ 1];
  o.contrib_new = a.contrib[p ^ 1];
  o.d = (float)a.prm->damping;
  o.base = (float)(1.0 - a.prm->damping);
  o.l = threadIdx.x % a.G;
  o.on = o.l < a.L;
  return o;
}

__device__ __forceinline__ void ppr_finish_row(const PprArgs &a, const PprLane &t, int v,
                                               CVal acc, double &l1) {
  const float sum = __fadd_rn(acc.s, acc.c);
  const float b = ((__ldg(a.seed_mask + v) >> t.l) & 1u) ? t.base : 0.f;
  const float r = __fadd_rn(b, __fmul_rn(t.d, sum));
  const int deg = __ldg(a.csr_off + v + 1) - __ldg(a.csr_off + v);
  const size_t k = (size_t)v * a.L + t.l;
  l1 += fabs((double)r - (double)t.rank_old[k]);
  t.rank_new[k] = r;
  t.contrib_new[k] = deg ? __fdiv_rn(r, (float)deg) : 0.f;
}

// Edge-order fold of one lane over [e, stop): groups of 8 contributions are
// summed pairwise in FP32 (relative error <= 3 u of the group's sum, the
// terms being non-negative), and the group sums are accumulated with two-sum
// compensation, so the error of a row stays near 3 u of its value.
__device__ __forceinline__ CVal ppr_fold(const PprArgs &a, const PprLane &t, int e, int stop) {
  CVal acc{0.f, 0.f};
  constexpr int U = 8;
  for (; e + U <= stop; e += U) {
    int u[U];
    float x[U];
#pragma unroll
    for (int j = 0; j < U; ++j) u[j] = __ldg(a.csc_src + e + j);
#pragma unroll
    for (int j = 0; j < U; ++j) x[j] = __ldg(t.contrib + (size_t)u[j] * a.L + t.l);
    const float g = __fadd_rn(__fadd_rn(__fadd_rn(x[0], x[1]), __fadd_rn(x[2], x[3])),
                              __fadd_rn(__fadd_rn(x[4], x[5]), __fadd_rn(x[6], x[7])));
    acc = two_sum_add(acc, CVal{g, 0.f});
  }
  for (; e < stop; ++e) {
    const int u = __ldg(a.csc_src + e);
    acc = two_sum_add(acc, CVal{__ldg(t.contrib + (size_t)u * a.L + t.l), 0.f});
  }
  return acc;
}

// Per-lane block sums of l1 in a fixed order into out[lane].
__device__ __forceinline__ void lane_block_sums(double l1, int G, double *out) {
  __shared__ double s[kNT];
  s[threadIdx.x] = l1;
  __syncthreads();
  if (threadIdx.x < G) {
    double t = 0.0;
    for (int j = threadIdx.x; j < kNT; j += G) t += s[j];
    out[threadIdx.x] = t;
  }
}

__global__ void __launch_bounds__(kNT) k_ppr_pieces(PprArgs a, double *l1_part) {
  const PprLane t = ppr_lane(a);
  const int per_block = kNT / a.G;
  const int local = threadIdx.x / a.G;
  double l1 = 0.0;
  if (t.on) {
    for (int k = blockIdx.x * per_block + local; k < a.n_pieces; k += gridDim.x * per_block) {
      int e = k * a.P;
      const int end = min(a.E, e + a.P);
      int r = __ldg(a.first_row + k);
      int row_end = __ldg(a.csc_off + r + 1);
      bool cont = __ldg(a.csc_off + r) < e;
      for (;;) {
        const int stop = min(row_end, end);
        const CVal acc = ppr_fold(a, t, e, stop);
        if (stop < row_end) {  // the piece ends inside row r
          (cont ? a.head : a.tail)[(size_t)k * a.L + t.l] = acc;
          break;
        }
        if (cont)
          a.head[(size_t)k * a.L + t.l] = acc;
        else
          ppr_finish_row(a, t, r, acc, l1);
        if (stop == end) break;
        do {  // next row with in-edges (one exists: stop < end <= E)
          ++r;
          row_end = __ldg(a.csc_off + r + 1);
        } while (row_end == stop);
        cont = false;
        e = stop;
      }
    }
  }
  lane_block_sums(l1, a.G, l1_part + (size_t)blockIdx.x * a.G);
}

// Rows cut by piece boundaries (partials folded in piece order), and in the
// first iteration the rows without in-edges (first piece -1): their rank is
// (1-d) [seed] from then on, so it is written into both buffers once and
// those rows are skipped afterwards.
__global__ void __launch_bounds__(kNT) k_ppr_fix(PprArgs a, double *l1_part) {
  const PprLane t = ppr_lane(a);
  const int per_block = kNT / a.G;
  const int local = threadIdx.x / a.G;
  const bool first = a.cnt->iteration == 0;
  const int limit = first ? a.n_fix : a.n_split;
  double l1 = 0.0;
  if (t.on) {
    for (int i = blockIdx.x * per_block + local; i < limit; i += gridDim.x * per_block) {
      const int v = a.fix[3 * i], ps = a.fix[3 * i + 1], pe = a.fix[3 * i + 2];
      CVal acc{0.f, 0.f};
      if (ps >= 0) {
        acc = a.tail[(size_t)ps * a.L + t.l];
        for (int k = ps + 1; k <= pe; ++k) acc = two_sum_add(acc, a.head[(size_t)k * a.L + t.l]);
      }
      ppr_finish_row(a, t, v, acc, l1);
      if (ps < 0) {  // first iteration only: the other buffer too (the
                     // pieces of this iteration have read it already)
        const size_t k = (size_t)v * a.L + t.l;
        a.rank[0][k] = t.rank_new[k];
        a.contrib[0][k] = t.contrib_new[k];
      }
    }
  }
  lane_block_sums(l1, a.G, l1_part + (size_t)blockIdx.x * a.G);
}

// Per-lane residuals (fixed-order sums over the blocks); the loop goes on
// while the largest is above tol.
__global__ void __launch_bounds__(kNT)
    k_ppr_finish(const double *l1_part, int nblocks, int G, int L, const BatchParams *prm,
                 gas_counters *cnt, double *lane_resid, cudaGraphConditionalHandle h,
                 int in_graph) {
  __shared__ double s[kNT];
  const int l = threadIdx.x % G, j = threadIdx.x / G, nj = kNT / G;
  double v = 0.0;
  for (int b = j; b < nblocks; b += nj) v += l1_part[(size_t)b * G + l];
  s[threadIdx.x] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < G)
    for (int q = 0; q < nj; ++q) t += s[q * G + threadIdx.x];
  __syncthreads();
  if (threadIdx.x < G) s[threadIdx.x] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mx = 0.0;
    for (int q = 0; q < L; ++q) {
      lane_resid[1 + q] = s[q];
      mx = s[q] > mx ? s[q] : mx;
    }
    lane_resid[0] = mx;
    const int it = ++cnt->iteration;
    set_cond(cnt, !(mx <= prm->tol), it, h, in_graph);
  }
}

// r0 = e_seed per lane; contributions accordingly.
__global__ void k_ppr_init(const uint32_t *seed_mask, const int32_t *csr_off, int nV, int L,
                           float *rank, float *contrib) {
  const size_t n = (size_t)nV * L;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const int v = (int)(k / L), l = (int)(k % L);
    const float r = ((seed_mask[v] >> l) & 1u) ? 1.f : 0.f;
    const int deg = csr_off[v + 1] - csr_off[v];
    rank[k] = r;
    contrib[k] = deg ? __fdiv_rn(r, (float)deg) : 0.f;
  }
}

__global__ void k_ppr_precond(gas_counters *cnt, cudaGraphConditionalHandle h, int in_graph) {
  set_cond(cnt, true, 0, h, in_graph);
}

}  // namespace

// ---------------------------------------------------------------------------
// The batch object.
// ---------------------------------------------------------------------------
struct gas_batch {
  std::vector<int32_t> v_off{0};  // first vertex of every graph; back() = V
  std::vector<int32_t> src, dst;  // union edge list (global ids) until built
  std::vector<int32_t> w;         // its weights, once a weighted graph came
  bool weighted = false;
  int64_t n_edges = 0;
  gas_engine *eng = nullptr;      // holds the union graph (CSR + CSC)
  bool built = false;
  gas_counters *cnt = nullptr;    // [3] device: BFS loop, PPR loop, SSSP loop
  gas_counters *h_cnt = nullptr;  // [3] pinned
  BatchParams *prm = nullptr;     // device
  unsigned long long *edges = nullptr;  // BFS edges pushed
  double *resid = nullptr;        // [1 + 32] max and per-lane PPR residual
  // BFS
  uint32_t *vn = nullptr, *next = nullptr, *tbits = nullptr;  // vn: [V][2] BFS pairs
  int32_t *depth = nullptr, *q_mask = nullptr, *q_end = nullptr,
          *q_delta = nullptr, *part = nullptr, *qpart = nullptr, *srcs = nullptr;
  int32_t depth_lanes = 0, srcs_cap = 0;
  // SSSP (shares the frontier arrays above; next is the changed-lane mask)
  int32_t *dist = nullptr, *q_vals = nullptr, *sssp_srcs = nullptr, *lane_rounds = nullptr;
  uint32_t *lanes_active = nullptr;
  unsigned long long *sssp_edges = nullptr;
  int32_t dist_ls = 0, sssp_srcs_cap = 0;
  // profiling of the SSSP pushes (direct launches, events around each push)
  bool profiling = false;
  cudaEvent_t pev[2] = {nullptr, nullptr};
  gas_kernel_profile prof{};
  // PPR
  int32_t *first_row = nullptr, *fix = nullptr;
  CVal *head = nullptr, *tail = nullptr;
  float *rank[2] = {nullptr, nullptr}, *contrib[2] = {nullptr, nullptr};
  uint32_t *seed_mask = nullptr;
  double *l1 = nullptr;
  int32_t n_pieces = 0, n_fix = 0, n_split = 0, piece_edges = 0, ppr_lanes = 0, l1_cap = 0;
  int32_t tuned_piece = 0;
  // cached graph
  cudaGraphExec_t graph = nullptr;
  int32_t g_bfs_lanes = -1, g_ppr_lanes = -1, g_piece = -1, g_sssp_lanes = -1;
};

namespace {

template <class T>
void bfree(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

void drop_graph(gas_batch *b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->g_bfs_lanes = b->g_ppr_lanes = b->g_piece = b->g_sssp_lanes = -1;
}

void free_state(gas_batch *b) {
  drop_graph(b);
  bfree(b->vn); bfree(b->next); bfree(b->tbits); bfree(b->depth);
  bfree(b->q_mask); bfree(b->q_end); bfree(b->q_delta);
  bfree(b->part); bfree(b->qpart); bfree(b->srcs);
  bfree(b->first_row); bfree(b->fix); bfree(b->head); bfree(b->tail);
  bfree(b->seed_mask); bfree(b->l1);
  bfree(b->dist); bfree(b->q_vals); bfree(b->sssp_srcs); bfree(b->lane_rounds);
  bfree(b->lanes_active);
  b->dist_ls = b->sssp_srcs_cap = 0;
  for (int i = 0; i < 2; ++i) { bfree(b->rank[i]); bfree(b->contrib[i]); }
  b->n_pieces = b->n_fix = b->n_split = b->piece_edges = b->ppr_lanes = b->depth_lanes = 0;
  b->srcs_cap = b->l1_cap = 0;
}

int lane_group(int L) {
  int g = 1;
  while (g < L) g <<= 1;
  return g;
}

int nwords(const gas_batch *b) { return (b->eng->nV + 31) / 32; }
int ms_blocks(const gas_batch *b) {
  return std::max(1, (nwords(b) + kMsBlockWords - 1) / kMsBlockWords);
}
// qpart: the blocks' (entries, out-edges) pairs, one spare pair, then the
// blocks' per-warp pairs
int2 *ms_wpart(const gas_batch *b) {
  return reinterpret_cast<int2 *>(b->qpart + 2 * ((size_t)ms_blocks(b) + 1));
}

// The frontier arrays the BFS and SSSP loops share (they run one after the
// other, each prologue resetting them).
gas_status_t ensure_frontier(gas_batch *b) {
  gas_engine *e = b->eng;
  const size_t nV = std::max(1, e->nV), nW = std::max(1, nwords(b));
  if (!b->next) {
    CUDA_TRY(cudaMalloc(&b->next, nV * 4));
    CUDA_TRY(cudaMalloc(&b->tbits, nW * 4));
    for (int32_t **p : {&b->q_mask, &b->q_end, &b->q_delta})
      CUDA_TRY(cudaMalloc(p, nV * 4));
    // the SSSP push cuts its queue's edges into chunks of 64 to 512 edges
    CUDA_TRY(cudaMalloc(&b->part, (((size_t)e->nE >> gasdev::kSlabChunkMinLog2) + 2) * 4));
    CUDA_TRY(cudaMalloc(&b->qpart,
                        2 * ((size_t)ms_blocks(b) + 1 + (size_t)ms_blocks(b) * kMsWarps) * 4));
  }
  return GAS_OK;
}

gas_status_t ensure_sssp(gas_batch *b, int lanes, int n_sources) {
  gas_engine *e = b->eng;
  const size_t nV = std::max(1, e->nV);
  GAS_TRY(ensure_frontier(b));
  const int LS = (lanes + 3) & ~3;
  if (b->dist_ls != LS) {
    drop_graph(b);
    bfree(b->dist);
    bfree(b->q_vals);
    CUDA_TRY(cudaMalloc(&b->dist, nV * LS * 4));
    CUDA_TRY(cudaMalloc(&b->q_vals, nV * LS * 4));
    b->dist_ls = LS;
  }
  if (!b->lane_rounds) {
    CUDA_TRY(cudaMalloc(&b->lane_rounds, kMaxLanes * 4));
    CUDA_TRY(cudaMalloc(&b->lanes_active, 4));
  }
  if (b->sssp_srcs_cap < n_sources) {
    drop_graph(b);
    bfree(b->sssp_srcs);
    CUDA_TRY(cudaMalloc(&b->sssp_srcs, (size_t)std::max(1, n_sources) * 4));
    b->sssp_srcs_cap = n_sources;
  }
  return GAS_OK;
}

gas_status_t ensure_bfs(gas_batch *b, int lanes, int n_sources) {
  gas_engine *e = b->eng;
  const size_t nV = std::max(1, e->nV);
  GAS_TRY(ensure_frontier(b));
  if (!b->vn) CUDA_TRY(cudaMalloc(&b->vn, nV * 8));
  if (b->depth_lanes != lanes) {
    drop_graph(b);
    bfree(b->depth);
    CUDA_TRY(cudaMalloc(&b->depth, nV * lanes * 4));
    b->depth_lanes = lanes;
  }
  if (b->srcs_cap < n_sources) {
    drop_graph(b);
    bfree(b->srcs);
    CUDA_TRY(cudaMalloc(&b->srcs, (size_t)std::max(1, n_sources) * 4));
    b->srcs_cap = n_sources;
  }
  return GAS_OK;
}

// Pieces of P edges over the CSC, their first rows, and the rows the second
// pass finishes (cut rows and rows without in-edges).
gas_status_t ensure_ppr(gas_batch *b, int lanes, int P, int grid_pieces, int grid_fix) {
  gas_engine *e = b->eng;
  const size_t nV = std::max(1, e->nV);
  if (b->ppr_lanes != lanes) {
    drop_graph(b);
    for (int i = 0; i < 2; ++i) { bfree(b->rank[i]); bfree(b->contrib[i]); }
    for (int i = 0; i < 2; ++i) {
      CUDA_TRY(cudaMalloc(&b->rank[i], nV * lanes * 4));
      CUDA_TRY(cudaMalloc(&b->contrib[i], nV * lanes * 4));
    }
    b->ppr_lanes = lanes;
    b->piece_edges = 0;  // head/tail are sized by lanes
  }
  if (!b->seed_mask) CUDA_TRY(cudaMalloc(&b->seed_mask, nV * 4));
  const int G = lane_group(lanes);
  const int need_l1 = (grid_pieces + grid_fix) * G;
  if (b->l1_cap < need_l1) {
    drop_graph(b);
    bfree(b->l1);
    CUDA_TRY(cudaMalloc(&b->l1, (size_t)need_l1 * sizeof(double)));
    b->l1_cap = need_l1;
  }
  if (b->piece_edges == P) return GAS_OK;
  drop_graph(b);
  const std::vector<int32_t> &off = e->h_csc_off;
  const int32_t E = e->nE, V = e->nV;
  const int32_t n_pieces = (int32_t)(((int64_t)E + P - 1) / P);
  std::vector<int32_t> first((size_t)std::max(1, n_pieces));
  for (int32_t k = 0, r = 0; k < n_pieces; ++k) {
    const int64_t e0 = (int64_t)k * P;
    while (off[r + 1] <= e0) ++r;  // first row with csc_off[r+1] > e0
    first[k] = r;
  }
  std::vector<int32_t> fix, zero;
  for (int32_t v = 0; v < V; ++v) {
    const int32_t lo = off[v], hi = off[v + 1];
    if (lo == hi) {
      zero.insert(zero.end(), {v, -1, -1});
    } else {
      const int32_t ps = lo / P, pe = (hi - 1) / P;
      if (ps != pe) fix.insert(fix.end(), {v, ps, pe});
    }
  }
  const int32_t n_split = (int32_t)(fix.size() / 3);
  fix.insert(fix.end(), zero.begin(), zero.end());
  bfree(b->first_row);
  bfree(b->fix);
  bfree(b->head);
  bfree(b->tail);
  CUDA_TRY(cudaMalloc(&b->first_row, first.size() * 4));
  CUDA_TRY(cudaMalloc(&b->fix, std::max<size_t>(1, fix.size()) * 4));
  const size_t hp = std::max<size_t>(1, (size_t)n_pieces * lanes) * sizeof(CVal);
  CUDA_TRY(cudaMalloc(&b->head, hp));
  CUDA_TRY(cudaMalloc(&b->tail, hp));
  CUDA_TRY(cudaMemcpy(b->first_row, first.data(), first.size() * 4, cudaMemcpyHostToDevice));
  if (!fix.empty())
    CUDA_TRY(cudaMemcpy(b->fix, fix.data(), fix.size() * 4, cudaMemcpyHostToDevice));
  b->n_pieces = n_pieces;
  b->n_fix = (int32_t)(fix.size() / 3);
  b->n_split = n_split;
  b->piece_edges = P;
  return GAS_OK;
}

struct RunCtx {
  gas_batch *b;
  int bfs_lanes, ppr_lanes, sssp_lanes;
  int slab_grid, grid_pieces, grid_fix, sssp_grid;
  PprArgs ppr;
};

PprArgs ppr_args(gas_batch *b, int lanes) {
  gas_engine *e = b->eng;
  PprArgs a;
  a.csc_off = e->csc_off;
  a.csc_src = e->csc_src;
  a.csr_off = e->csr_off;
  a.first_row = b->first_row;
  a.n_pieces = b->n_pieces;
  a.P = b->piece_edges;
  a.E = e->nE;
  a.L = lanes;
  a.G = lane_group(lanes);
  a.fix = b->fix;
  a.n_fix = b->n_fix;
  a.n_split = b->n_split;
  a.head = b->head;
  a.tail = b->tail;
  for (int i = 0; i < 2; ++i) {
    a.rank[i] = b->rank[i];
    a.contrib[i] = b->contrib[i];
  }
  a.seed_mask = b->seed_mask;
  a.prm = b->prm;
  a.cnt = b->cnt + 1;
  return a;
}

typedef gas_status_t (*StepFn)(RunCtx *, cudaStream_t, cudaGraphConditionalHandle, int);

// The next frontier of new lanes, then the loop control (first: the
// prologue's sources, level 0).
gas_status_t bfs_compact(RunCtx *c, cudaStream_t s, cudaGraphConditionalHandle h, int ig,
                         int first) {
  gas_batch *b = c->b;
  gas_engine *e = b->eng;
  const int nb = ms_blocks(b);
  k_ms_count<<<nb, kNT, 0, s>>>(b->tbits, nullptr, b->vn, e->csr_off, nwords(b), b->qpart,
                                ms_wpart(b), nullptr);
  k_mss_spine<<<1, kMssSpineNT, 0, s>>>(reinterpret_cast<int2 *>(b->qpart), nb, b->cnt,
                                        c->slab_grid * (kNT / 32), b->edges, nullptr, nullptr,
                                        h, ig, first);
  k_ms_write<<<nb, kNT, 0, s>>>(b->tbits, b->vn, e->csr_off, nwords(b), b->qpart,
                               ms_wpart(b), c->bfs_lanes, b->cnt, b->depth, b->q_mask, b->q_end, b->q_delta,
                               b->part);
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

gas_status_t bfs_prologue(RunCtx *c, cudaStream_t s, cudaGraphConditionalHandle h, int ig) {
  gas_batch *b = c->b;
  gas_engine *e = b->eng;
  const size_t nV = std::max(1, e->nV), nW = std::max(1, nwords(b));
  const int L = c->bfs_lanes;
  k_b_reset<<<1, 1, 0, s>>>(b->cnt, b->prm, 0, b->edges);
  CUDA_TRY(cudaMemsetAsync(b->vn, 0, nV * 8, s));
  CUDA_TRY(cudaMemsetAsync(b->tbits, 0, nW * 4, s));
  CUDA_TRY(cudaMemsetAsync(b->depth, 0xff, nV * L * 4, s));
  k_ms_seed<<<2 * e->num_sms, 256, 0, s>>>(b->srcs, b->prm, L, b->vn, b->tbits);
  return bfs_compact(c, s, h, ig, 1);
}

gas_status_t bfs_push(RunCtx *c, cudaStream_t s) {
  gas_batch *b = c->b;
  gas_engine *e = b->eng;
  const gasdev::SlabSource q = gasdev::slab_source(
      b->q_end, nullptr, b->q_delta, 0, 0, &b->cnt->n_changed, &b->cnt->n_scatter_edges,
      b->part, &b->cnt->push_chunk_log2);
  MsPushPol pol{e->csr_dst, b->q_mask, b->vn, b->tbits};
  k_ms_push<<<c->slab_grid, kNT, 0, s>>>(pol, q);
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

gas_status_t bfs_body(RunCtx *c, cudaStream_t s, cudaGraphConditionalHandle h, int ig) {
  gas_batch *b = c->b;
  if (b->profiling && !ig) {  // direct launches: the counters were just read
    // algorithmic bytes: per union edge its index and the destination's
    // visited and next words; per queue entry its edge range and lane mask
    const gas_counters &k = b->h_cnt[0];
    CUDA_TRY(cudaEventRecord(b->pev[0], s));
    GAS_TRY(bfs_push(c, s));
    CUDA_TRY(cudaEventRecord(b->pev[1], s));
    CUDA_TRY(cudaEventSynchronize(b->pev[1]));
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, b->pev[0], b->pev[1]));
    b->prof.push_ms += ms;
    b->prof.push_bytes += (int64_t)k.n_scatter_edges * 12 + (int64_t)k.n_changed * 12;
    b->prof.push_launches += 1;
  } else {
    GAS_TRY(bfs_push(c, s));
  }
  return bfs_compact(c, s, h, ig, 0);
}

// The queue of the changed lanes, then the loop control (first: the
// prologue's queue).
gas_status_t sssp_compact(RunCtx *c, cudaStream_t s, cudaGraphConditionalHandle h, int ig,
                          int first) {
  gas_batch *b = c->b;
  gas_engine *e = b->eng;
  const int nb = ms_blocks(b);
  k_ms_count<<<nb, kNT, 0, s>>>(b->tbits, b->next, nullptr, e->csr_off, nwords(b), b->qpart,
                                ms_wpart(b), b->lanes_active);
  k_mss_spine<<<1, kMssSpineNT, 0, s>>>(reinterpret_cast<int2 *>(b->qpart), nb, b->cnt + 2,
                                        c->sssp_grid * (kNT / 32), b->sssp_edges,
                                        b->lanes_active, b->lane_rounds, h, ig, first);
  k_mss_write<<<nb, kNT, 0, s>>>(b->tbits, b->next, e->csr_off, nwords(b), b->qpart,
                                 ms_wpart(b), b->dist_ls, b->dist, b->q_mask, b->q_vals, b->q_end,
                                 b->q_delta, b->part, b->cnt + 2);
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

gas_status_t sssp_prologue(RunCtx *c, cudaStream_t s, cudaGraphConditionalHandle h, int ig) {
  gas_batch *b = c->b;
  gas_engine *e = b->eng;
  const size_t nV = std::max(1, e->nV), nW = std::max(1, nwords(b));
  k_b_reset<<<1, 1, 0, s>>>(b->cnt + 2, b->prm, 2, b->sssp_edges);
  CUDA_TRY(cudaMemsetAsync(b->next, 0, nV * 4, s));
  CUDA_TRY(cudaMemsetAsync(b->tbits, 0, nW * 4, s));
  k_mss_init<<<8 * e->num_sms, 256, 0, s>>>(b->dist, nV * b->dist_ls, b->lanes_active,
                                           b->lane_rounds);
  k_mss_seed<<<2 * e->num_sms, 256, 0, s>>>(b->sssp_srcs, b->prm, c->sssp_lanes, b->dist_ls,
                                           b->dist, b->next, b->tbits);
  return sssp_compact(c, s, h, ig, 1);
}

gas_status_t sssp_push(RunCtx *c, cudaStream_t s) {
  gas_batch *b = c->b;
  gas_engine *e = b->eng;
  const gasdev::SlabSource q = gasdev::slab_source(
      b->q_end, nullptr, b->q_delta, 0, 0, &b->cnt[2].n_changed, &b->cnt[2].n_scatter_edges,
      b->part, &b->cnt[2].push_chunk_log2);
  const int32_t *w = b->weighted ? (const int32_t *)e->csr_ed : nullptr;
  if (b->dist_ls == 4) {
    MssPushPolStaged<1> pol{e->csr_dst, w, b->q_vals, b->dist, b->next, b->tbits};
    k_mss_push<<<c->sssp_grid, kNT, 0, s>>>(pol, q);
  } else if (b->dist_ls == 8) {
    MssPushPolStaged<2> pol{e->csr_dst, w, b->q_vals, b->dist, b->next, b->tbits};
    k_mss_push<<<c->sssp_grid, kNT, 0, s>>>(pol, q);
  } else {
    MssPushPol pol{e->csr_dst, w, b->q_mask, b->q_vals, b->dist, b->next, b->tbits,
                   b->dist_ls};
    k_mss_push<<<c->sssp_grid, kNT, 0, s>>>(pol, q);
  }
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

// Algorithmic bytes of one SSSP push: per union edge its index, its weight
// and the destination row; per queue entry its edge range and snapshot row.
int64_t sssp_push_bytes(const gas_batch *b, const gas_counters &c) {
  const int64_t row = 4LL * b->dist_ls;
  return (int64_t)c.n_scatter_edges * ((b->weighted ? 8 : 4) + row) +
         (int64_t)c.n_changed * (8 + row);
}

gas_status_t sssp_body(RunCtx *c, cudaStream_t s, cudaGraphConditionalHandle h, int ig) {
  gas_batch *b = c->b;
  if (b->profiling && !ig) {  // direct launches: the counters were just read
    CUDA_TRY(cudaEventRecord(b->pev[0], s));
    GAS_TRY(sssp_push(c, s));
    CUDA_TRY(cudaEventRecord(b->pev[1], s));
    CUDA_TRY(cudaEventSynchronize(b->pev[1]));
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, b->pev[0], b->pev[1]));
    b->prof.push_ms += ms;
    b->prof.push_bytes += sssp_push_bytes(b, b->h_cnt[2]);
    b->prof.push_launches += 1;
  } else {
    GAS_TRY(sssp_push(c, s));
  }
  return sssp_compact(c, s, h, ig, 0);
}

gas_status_t ppr_prologue(RunCtx *c, cudaStream_t s, cudaGraphConditionalHandle h, int ig) {
  gas_batch *b = c->b;
  gas_engine *e = b->eng;
  k_b_reset<<<1, 1, 0, s>>>(b->cnt + 1, b->prm, 1, nullptr);
  k_ppr_init<<<8 * e->num_sms, 256, 0, s>>>(b->seed_mask, e->csr_off, e->nV, c->ppr_lanes,
                                           b->rank[0], b->contrib[0]);
  k_ppr_precond<<<1, 1, 0, s>>>(b->cnt + 1, h, ig);
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

gas_status_t ppr_body(RunCtx *c, cudaStream_t s, cudaGraphConditionalHandle h, int ig) {
  gas_batch *b = c->b;
  const int G = c->ppr.G;
  k_ppr_pieces<<<c->grid_pieces, kNT, 0, s>>>(c->ppr, b->l1);
  k_ppr_fix<<<c->grid_fix, kNT, 0, s>>>(c->ppr, b->l1 + (size_t)c->grid_pieces * G);
  k_ppr_finish<<<1, kNT, 0, s>>>(b->l1, c->grid_pieces + c->grid_fix, G, c->ppr_lanes,
                                 b->prm, b->cnt + 1, b->resid, h, ig);
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

struct Loop {
  StepFn pro, body;
};

// One graph: for each loop, its prologue then WHILE(cond) { body }.
gas_status_t build_chain(RunCtx *c, const Loop *loops, int n, cudaGraphExec_t *out) {
  cudaGraph_t g = nullptr;
  cudaStream_t cs = nullptr;
  gas_status_t st = GAS_OK;
  CUDA_TRY(cudaGraphCreate(&g, 0));
  cudaError_t ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(GAS_ERR_CUDA, "batch graph stream: %s", cudaGetErrorString(ce));
  }
  cudaGraphNode_t prev = nullptr;
  for (int i = 0; i < n && st == GAS_OK; ++i) {
    cudaGraphConditionalHandle h;
    ce = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    if (ce == cudaSuccess)
      ce = cudaStreamBeginCaptureToGraph(cs, g, prev ? &prev : nullptr, nullptr, prev ? 1 : 0,
                                         cudaStreamCaptureModeRelaxed);
    if (ce != cudaSuccess) {
      st = fail(GAS_ERR_CUDA, "batch prologue capture: %s", cudaGetErrorString(ce));
      break;
    }
    st = loops[i].pro(c, cs, h, 1);
    std::vector<cudaGraphNode_t> deps;
    if (st == GAS_OK) {
      cudaStreamCaptureStatus cst;
      const cudaGraphNode_t *d = nullptr;
      size_t nd = 0;
      ce = cudaStreamGetCaptureInfo(cs, &cst, nullptr, nullptr, &d, nullptr, &nd);
      if (ce == cudaSuccess) deps.assign(d, d + nd);
      else st = fail(GAS_ERR_CUDA, "capture info: %s", cudaGetErrorString(ce));
    }
    cudaGraph_t cap = nullptr;
    ce = cudaStreamEndCapture(cs, &cap);
    if (st == GAS_OK && ce != cudaSuccess)
      st = fail(GAS_ERR_CUDA, "end prologue capture: %s", cudaGetErrorString(ce));
    if (st != GAS_OK) break;
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    ce = cudaGraphAddNode(&node, g, deps.data(), nullptr, deps.size(), &p);
    if (ce != cudaSuccess) {
      st = fail(GAS_ERR_CUDA, "add while node: %s", cudaGetErrorString(ce));
      break;
    }
    ce = cudaStreamBeginCaptureToGraph(cs, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                       cudaStreamCaptureModeRelaxed);
    if (ce != cudaSuccess) {
      st = fail(GAS_ERR_CUDA, "body capture: %s", cudaGetErrorString(ce));
      break;
    }
    st = loops[i].body(c, cs, h, 1);
    cudaGraph_t bc = nullptr;
    ce = cudaStreamEndCapture(cs, &bc);
    if (st == GAS_OK && ce != cudaSuccess)
      st = fail(GAS_ERR_CUDA, "end body capture: %s", cudaGetErrorString(ce));
    prev = node;
  }
  if (st == GAS_OK) {
    ce = cudaGraphInstantiate(out, g, 0);
    if (ce != cudaSuccess) st = fail(GAS_ERR_CUDA, "instantiate: %s", cudaGetErrorString(ce));
  }
  cudaStreamDestroy(cs);
  cudaGraphDestroy(g);
  return st;
}

// The same loops as direct launches with one host read of the condition per
// iteration (GAS_HOST_LOOP=1: ncu cannot profile kernels inside graphs with
// conditional nodes).
gas_status_t run_direct(RunCtx *c, const Loop *loops, const int *which, int n, cudaStream_t s) {
  gas_batch *b = c->b;
  for (int i = 0; i < n; ++i) {
    GAS_TRY(loops[i].pro(c, s, 0, 0));
    for (;;) {
      CUDA_TRY(cudaMemcpyAsync(b->h_cnt + which[i], b->cnt + which[i], sizeof(gas_counters),
                               cudaMemcpyDeviceToHost, s));
      CUDA_TRY(cudaStreamSynchronize(s));
      if (!b->h_cnt[which[i]].cond) break;
      GAS_TRY(loops[i].body(c, s, 0, 0));
    }
  }
  return GAS_OK;
}

void grids(gas_batch *b, RunCtx *c) {
  gas_engine *e = b->eng;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ms_push, kNT, 0);
  c->slab_grid = e->num_sms * (per_sm > 0 ? per_sm : 1);
  per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ppr_pieces, kNT, 0);
  c->grid_pieces = e->num_sms * (per_sm > 0 ? per_sm : 1);
  c->grid_fix = 8 * e->num_sms;
  per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mss_push<MssPushPolStaged<2>>, kNT,
                                                0);
  c->sssp_grid = e->num_sms * (per_sm > 0 ? per_sm : 1);
}

gas_status_t check_job(const gas_batch *b, const gas_batch_job *j) {
  if (!j) return fail(GAS_ERR_INVALID, "null job");
  if (j->bfs_lanes < 0 || j->bfs_lanes > kMaxLanes || j->ppr_lanes < 0 ||
      j->ppr_lanes > kMaxLanes || j->sssp_lanes < 0 || j->sssp_lanes > kMaxLanes)
    return fail(GAS_ERR_INVALID, "lanes must be in [0, %d]", kMaxLanes);
  if (j->bfs_lanes == 0 && j->ppr_lanes == 0 && j->sssp_lanes == 0)
    return fail(GAS_ERR_INVALID, "job has no BFS, SSSP or PPR lanes");
  if (j->bfs_lanes > 0 && !j->bfs_sources) return fail(GAS_ERR_INVALID, "null bfs_sources");
  if (j->sssp_lanes > 0 && !j->sssp_sources)
    return fail(GAS_ERR_INVALID, "null sssp_sources");
  if (j->ppr_lanes > 0) {
    if (!j->ppr_seeds) return fail(GAS_ERR_INVALID, "null ppr_seeds");
    if (!(j->damping > 0.0 && j->damping < 1.0) || !(j->tol > 0.0))
      return fail(GAS_ERR_INVALID, "damping must be in (0,1), tol > 0");
  }
  if (j->piece_edges < 0 || j->piece_edges > (1 << 20))
    return fail(GAS_ERR_INVALID, "piece_edges must be in [0, 2^20]");
  const int G = (int)b->v_off.size() - 1;
  for (int pass = 0; pass < 3; ++pass) {
    const int L = pass == 0 ? j->bfs_lanes : pass == 1 ? j->ppr_lanes : j->sssp_lanes;
    const int32_t *ids = pass == 0 ? j->bfs_sources : pass == 1 ? j->ppr_seeds : j->sssp_sources;
    for (int g = 0; g < G; ++g)
      for (int l = 0; l < L; ++l) {
        const int32_t s = ids[(size_t)g * L + l];
        if (s < -1 || s >= b->v_off[g + 1] - b->v_off[g])
          return fail(GAS_ERR_INVALID, "%s %d of graph %d lane %d out of range",
                      pass == 1 ? "seed" : "source", s, g, l);
      }
  }
  return GAS_OK;
}

int default_piece(const gas_batch *b) { return b->tuned_piece > 0 ? b->tuned_piece : 256; }

}  // namespace

extern "C" {

gas_status_t gas_batch_create(gas_batch **out) {
  if (!out) return fail(GAS_ERR_INVALID, "null out");
  *out = nullptr;
  gas_batch *b = new (std::nothrow) gas_batch;
  if (!b) return fail(GAS_ERR_NOMEM, "batch");
  gas_status_t st = gas_engine_create(GAS_PROG_BFS, &b->eng);
  if (st != GAS_OK) {
    delete b;
    return st;
  }
  *out = b;
  return GAS_OK;
}

void gas_batch_destroy(gas_batch *b) {
  if (!b) return;
  free_state(b);
  for (cudaEvent_t &ev : b->pev)
    if (ev) cudaEventDestroy(ev);
  bfree(b->cnt);
  bfree(b->prm);
  bfree(b->edges);
  bfree(b->sssp_edges);
  bfree(b->resid);
  if (b->h_cnt) cudaFreeHost(b->h_cnt);
  gas_engine_destroy(b->eng);
  delete b;
}

gas_status_t gas_batch_add_graph(gas_batch *b, int32_t nV, int64_t nE, const int32_t *srcs,
                                 const int32_t *dsts, int32_t *graph_id) {
  return gas_batch_add_graph_weighted(b, nV, nE, srcs, dsts, nullptr, graph_id);
}

gas_status_t gas_batch_add_graph_weighted(gas_batch *b, int32_t nV, int64_t nE,
                                          const int32_t *srcs, const int32_t *dsts,
                                          const int32_t *weights, int32_t *graph_id) {
  if (!b || nV < 0 || nE < 0 || (nE > 0 && (!srcs || !dsts)))
    return fail(GAS_ERR_INVALID, "batch_add_graph: bad arguments");
  if (b->built) return fail(GAS_ERR_STATE, "batch already built");
  const int64_t base = b->v_off.back();
  if (base + nV > INT32_MAX - 1 || b->n_edges + nE > INT32_MAX - 1)
    return fail(GAS_ERR_TOO_LARGE, "batch exceeds the 32-bit index space");
  for (int64_t i = 0; i < nE; ++i)
    if (srcs[i] < 0 || srcs[i] >= nV || dsts[i] < 0 || dsts[i] >= nV)
      return fail(GAS_ERR_INVALID, "batch_add_graph: edge %lld outside [0, %d)",
                  (long long)i, nV);
  if (weights)  // the SSSP Program's margin: dist + w never passes INT_MAX
    for (int64_t i = 0; i < nE; ++i)
      if (weights[i] < 0 || weights[i] > 100000)
        return fail(GAS_ERR_INVALID, "batch_add_graph: weight %d of edge %lld outside "
                    "[0, 100000]", weights[i], (long long)i);
  try {
    const size_t n0 = b->src.size();
    b->src.resize(n0 + nE);
    b->dst.resize(n0 + nE);
    for (int64_t i = 0; i < nE; ++i) {
      b->src[n0 + i] = (int32_t)(srcs[i] + base);
      b->dst[n0 + i] = (int32_t)(dsts[i] + base);
    }
    if (weights && !b->weighted) {  // earlier graphs weigh 1 per edge
      b->w.assign(n0, 1);
      b->weighted = true;
    }
    if (b->weighted) {
      b->w.resize(n0 + nE, 1);
      if (weights) std::copy(weights, weights + nE, b->w.begin() + n0);
    }
    b->v_off.push_back((int32_t)(base + nV));
  } catch (...) {
    return fail(GAS_ERR_NOMEM, "batch edge list");
  }
  b->n_edges += nE;
  if (graph_id) *graph_id = (int32_t)b->v_off.size() - 2;
  return GAS_OK;
}

gas_status_t gas_batch_build(gas_batch *b, void *stream) {
  if (!b) return fail(GAS_ERR_INVALID, "null batch");
  if (b->built) return fail(GAS_ERR_STATE, "batch already built");
  if (b->v_off.size() < 2) return fail(GAS_ERR_STATE, "batch has no graphs");
  const int32_t nV = b->v_off.back();
  if (b->weighted) {  // an engine whose graph carries int32 edge data
    gas_engine *we = nullptr;
    GAS_TRY(gas_engine_create(GAS_PROG_SSSP, &we));
    gas_engine_destroy(b->eng);
    b->eng = we;
  }
  std::vector<int32_t> vd((size_t)std::max(1, nV), -1);
  GAS_TRY(gas_engine_set_graph(b->eng, nV, vd.data(), (int64_t)b->src.size(),
                               b->weighted ? b->w.data() : nullptr, b->src.data(),
                               b->dst.data(), stream));
  if (!b->cnt) {
    CUDA_TRY(cudaMalloc(&b->cnt, 3 * sizeof(gas_counters)));
    CUDA_TRY(cudaMemset(b->cnt, 0, 3 * sizeof(gas_counters)));
    CUDA_TRY(cudaMallocHost(&b->h_cnt, 3 * sizeof(gas_counters)));
    CUDA_TRY(cudaMalloc(&b->prm, sizeof(BatchParams)));
    CUDA_TRY(cudaMalloc(&b->edges, sizeof(unsigned long long)));
    CUDA_TRY(cudaMalloc(&b->sssp_edges, sizeof(unsigned long long)));
    CUDA_TRY(cudaMalloc(&b->resid, (1 + kMaxLanes) * sizeof(double)));
  }
  std::vector<int32_t>().swap(b->src);
  std::vector<int32_t>().swap(b->dst);
  std::vector<int32_t>().swap(b->w);
  b->built = true;
  return GAS_OK;
}

int32_t gas_batch_num_graphs(const gas_batch *b) {
  return b ? (int32_t)b->v_off.size() - 1 : 0;
}

int32_t gas_batch_num_vertices(const gas_batch *b) { return b ? b->v_off.back() : 0; }

int64_t gas_batch_num_edges(const gas_batch *b) { return b ? b->n_edges : 0; }

int32_t gas_batch_vertex_offset(const gas_batch *b, int32_t g) {
  return (b && g >= 0 && g < (int32_t)b->v_off.size()) ? b->v_off[g] : -1;
}

gas_status_t gas_batch_run(gas_batch *b, const gas_batch_job *job, int32_t *depth_out,
                           int32_t *dist_out, float *rank_out, gas_batch_stats *stats,
                           void *stream) {
  if (!b || !b->built) return fail(GAS_ERR_STATE, "batch not built");
  GAS_TRY(check_job(b, job));
  gas_engine *e = b->eng;
  cudaStream_t s = S(stream);
  const int G = gas_batch_num_graphs(b), nV = e->nV;
  const int LB = job->bfs_lanes, LP = job->ppr_lanes, LS = job->sssp_lanes;
  if (stats) *stats = gas_batch_stats{};
  RunCtx c;
  c.b = b;
  c.bfs_lanes = LB;
  c.ppr_lanes = LP;
  c.sssp_lanes = LS;
  grids(b, &c);
  const int P = job->piece_edges > 0 ? job->piece_edges : default_piece(b);
  BatchParams prm{};
  prm.damping = LP ? job->damping : 0.85;
  prm.tol = LP ? job->tol : 1.0;
  prm.bfs_max_iter = job->max_bfs_levels > 0 ? job->max_bfs_levels : nV + 2;
  prm.ppr_max_iter = job->max_ppr_iterations > 0 ? job->max_ppr_iterations : 1000;
  prm.n_sources = G * LB;
  prm.sssp_max_iter = job->max_sssp_iterations > 0 ? job->max_sssp_iterations : nV + 2;
  prm.n_sssp_sources = G * LS;
  std::vector<int32_t> sg, ss;
  if (LB) {
    GAS_TRY(ensure_bfs(b, LB, G * LB));
    sg.resize((size_t)G * LB);
    for (int g = 0; g < G; ++g)
      for (int l = 0; l < LB; ++l) {
        const int32_t v = job->bfs_sources[(size_t)g * LB + l];
        sg[(size_t)g * LB + l] = v < 0 ? -1 : v + b->v_off[g];
      }
  }
  if (LS) {
    GAS_TRY(ensure_sssp(b, LS, G * LS));
    ss.resize((size_t)G * LS);
    for (int g = 0; g < G; ++g)
      for (int l = 0; l < LS; ++l) {
        const int32_t v = job->sssp_sources[(size_t)g * LS + l];
        ss[(size_t)g * LS + l] = v < 0 ? -1 : v + b->v_off[g];
      }
  }
  std::vector<uint32_t> mask;
  if (LP) {
    GAS_TRY(ensure_ppr(b, LP, P, c.grid_pieces, c.grid_fix));
    mask.assign((size_t)std::max(1, nV), 0u);
    for (int g = 0; g < G; ++g)
      for (int l = 0; l < LP; ++l) {
        const int32_t v = job->ppr_seeds[(size_t)g * LP + l];
        if (v >= 0) mask[(size_t)v + b->v_off[g]] |= 1u << l;
      }
    c.ppr = ppr_args(b, LP);
  }
  Loop loops[3];
  int which[3];
  int n = 0;
  if (LB) { loops[n] = Loop{bfs_prologue, bfs_body}; which[n++] = 0; }
  if (LS) { loops[n] = Loop{sssp_prologue, sssp_body}; which[n++] = 2; }
  if (LP) { loops[n] = Loop{ppr_prologue, ppr_body}; which[n++] = 1; }
  const bool direct = gas::host_loop_requested() || b->profiling;
  if (!direct && (!b->graph || b->g_bfs_lanes != LB || b->g_ppr_lanes != LP ||
                  b->g_sssp_lanes != LS || b->g_piece != (LP ? P : -1))) {
    drop_graph(b);
    GAS_TRY(build_chain(&c, loops, n, &b->graph));
    b->g_bfs_lanes = LB;
    b->g_ppr_lanes = LP;
    b->g_sssp_lanes = LS;
    b->g_piece = LP ? P : -1;
  }
  CUDA_TRY(cudaMemcpyAsync(b->prm, &prm, sizeof(prm), cudaMemcpyHostToDevice, s));
  if (LB) CUDA_TRY(cudaMemcpyAsync(b->srcs, sg.data(), sg.size() * 4, cudaMemcpyHostToDevice, s));
  if (LS)
    CUDA_TRY(cudaMemcpyAsync(b->sssp_srcs, ss.data(), ss.size() * 4, cudaMemcpyHostToDevice, s));
  if (LP)
    CUDA_TRY(cudaMemcpyAsync(b->seed_mask, mask.data(), mask.size() * 4, cudaMemcpyHostToDevice,
                             s));
  if (direct) {
    GAS_TRY(run_direct(&c, loops, which, n, s));
  } else {
    CUDA_TRY(cudaGraphLaunch(b->graph, s));
  }
  CUDA_TRY(cudaMemcpyAsync(b->h_cnt, b->cnt, 3 * sizeof(gas_counters), cudaMemcpyDeviceToHost, s));
  unsigned long long edges = 0, sedges = 0;
  double resid[1 + kMaxLanes] = {};
  int32_t rounds[kMaxLanes] = {};
  if (LB) CUDA_TRY(cudaMemcpyAsync(&edges, b->edges, sizeof(edges), cudaMemcpyDeviceToHost, s));
  if (LS) {
    CUDA_TRY(cudaMemcpyAsync(&sedges, b->sssp_edges, sizeof(sedges), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(rounds, b->lane_rounds, sizeof(rounds), cudaMemcpyDeviceToHost, s));
  }
  if (LP) CUDA_TRY(cudaMemcpyAsync(resid, b->resid, sizeof(resid), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  const gas_counters cb = b->h_cnt[0], cp = b->h_cnt[1], cs = b->h_cnt[2];
  if (depth_out && LB)
    CUDA_TRY(cudaMemcpyAsync(depth_out, b->depth, (size_t)nV * LB * 4, cudaMemcpyDefault, s));
  if (dist_out && LS && nV > 0)  // rows of LS lanes in the device layout
    CUDA_TRY(cudaMemcpy2DAsync(dist_out, (size_t)LS * 4, b->dist, (size_t)b->dist_ls * 4,
                               (size_t)LS * 4, (size_t)nV, cudaMemcpyDefault, s));
  if (rank_out && LP)
    CUDA_TRY(cudaMemcpyAsync(rank_out, b->rank[cp.iteration & 1], (size_t)nV * LP * 4,
                             cudaMemcpyDefault, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (stats) {
    stats->bfs_iterations = LB ? cb.iteration : 0;
    stats->bfs_edges = (int64_t)edges;
    stats->ppr_iterations = LP ? cp.iteration : 0;
    stats->ppr_residual = resid[0];
    stats->piece_edges = LP ? P : 0;
    stats->sssp_iterations = LS ? cs.iteration : 0;
    stats->sssp_edges = (int64_t)sedges;
    for (int l = 0; l < LS; ++l) stats->sssp_lane_iterations[l] = rounds[l];
    // BFS: prologue 5 kernels (reset, seed, 3 compaction), 4 per level;
    // SSSP: prologue 6 (reset, init, seed, 3 compaction), 4 per iteration;
    // PPR: prologue 3, 3 per iteration
    stats->kernel_launches = (LB ? 5 + 4 * cb.iteration : 0) +
                             (LS ? 6 + 4 * cs.iteration : 0) + (LP ? 3 + 3 * cp.iteration : 0);
    stats->graph_launches = direct ? 0 : 1;
    for (int l = 0; l < LP; ++l) stats->ppr_lane_residual[l] = resid[1 + l];
  }
  if (LS && cs.error) {
    CUDA_TRY(cudaMemset(&b->cnt[2].error, 0, sizeof(int32_t)));
    return fail(cs.error == GAS_ERR_ITER_CAP ? GAS_ERR_ITER_CAP : GAS_ERR_DEVICE,
                "batch sssp: device error %d after %d iterations", cs.error, cs.iteration);
  }
  if (LB && cb.error) {
    CUDA_TRY(cudaMemset(&b->cnt[0].error, 0, sizeof(int32_t)));
    return fail(cb.error == GAS_ERR_ITER_CAP ? GAS_ERR_ITER_CAP : GAS_ERR_DEVICE,
                "batch bfs: device error %d after %d levels", cb.error, cb.iteration);
  }
  if (LP && cp.error) {
    CUDA_TRY(cudaMemset(&b->cnt[1].error, 0, sizeof(int32_t)));
    return fail(cp.error == GAS_ERR_ITER_CAP ? GAS_ERR_ITER_CAP : GAS_ERR_DEVICE,
                "batch ppr: residual %.3e after %d iterations", resid[0], cp.iteration);
  }
  return GAS_OK;
}

gas_status_t gas_batch_set_profiling(gas_batch *b, int32_t on) {
  if (!b) return fail(GAS_ERR_INVALID, "null batch");
  if (on && !b->pev[0]) {
    CUDA_TRY(cudaEventCreate(&b->pev[0]));
    CUDA_TRY(cudaEventCreate(&b->pev[1]));
  }
  b->profiling = on != 0;
  return GAS_OK;
}

gas_status_t gas_batch_get_profile(gas_batch *b, gas_kernel_profile *out, int32_t reset) {
  if (!b || !out) return fail(GAS_ERR_INVALID, "bad arguments");
  *out = b->prof;
  if (reset) b->prof = gas_kernel_profile{};
  return GAS_OK;
}

gas_status_t gas_batch_tune(gas_batch *b, int32_t ppr_lanes, double damping, int32_t trials,
                            int32_t *piece_edges_out, float *ms_per_iter_out, void *stream) {
  if (!b || !b->built) return fail(GAS_ERR_STATE, "batch not built");
  if (ppr_lanes < 1 || ppr_lanes > kMaxLanes || !(damping > 0.0 && damping < 1.0))
    return fail(GAS_ERR_INVALID, "batch_tune: bad arguments");
  if (trials <= 0) trials = 3;
  gas_engine *e = b->eng;
  cudaStream_t s = S(stream);
  RunCtx c;
  c.b = b;
  c.bfs_lanes = 0;
  c.sssp_lanes = 0;
  c.ppr_lanes = ppr_lanes;
  grids(b, &c);
  BatchParams prm{};
  prm.damping = damping;
  prm.tol = 0.0;
  prm.ppr_max_iter = INT_MAX;
  CUDA_TRY(cudaMemcpyAsync(b->prm, &prm, sizeof(prm), cudaMemcpyHostToDevice, s));
  const int cands[] = {64, 128, 256, 512, 1024, 2048};
  int best = 0;
  float best_ms = 0.f;
  cudaEvent_t ev[2];
  CUDA_TRY(cudaEventCreate(&ev[0]));
  CUDA_TRY(cudaEventCreate(&ev[1]));
  gas_status_t st = GAS_OK;
  for (int P : cands) {
    st = ensure_ppr(b, ppr_lanes, P, c.grid_pieces, c.grid_fix);
    if (st != GAS_OK) break;
    c.ppr = ppr_args(b, ppr_lanes);
    // a seed in lane 0 of vertex 0 makes the timed iterations do real work
    const uint32_t one = 1u;
    if (cudaMemsetAsync(b->seed_mask, 0, (size_t)std::max(1, e->nV) * 4, s) != cudaSuccess ||
        cudaMemcpyAsync(b->seed_mask, &one, 4, cudaMemcpyHostToDevice, s) != cudaSuccess) {
      st = fail(GAS_ERR_CUDA, "batch_tune: seed upload");
      break;
    }
    st = ppr_prologue(&c, s, 0, 0);
    if (st == GAS_OK) st = ppr_body(&c, s, 0, 0);  // warm-up
    if (st != GAS_OK) break;
    cudaEventRecord(ev[0], s);
    for (int t = 0; t < trials && st == GAS_OK; ++t) st = ppr_body(&c, s, 0, 0);
    cudaEventRecord(ev[1], s);
    if (cudaEventSynchronize(ev[1]) != cudaSuccess) {
      st = fail(GAS_ERR_CUDA, "batch_tune: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[0], ev[1]);
    ms /= (float)trials;
    if (!best || ms < best_ms) {
      best = P;
      best_ms = ms;
    }
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (st != GAS_OK) return st;
  b->tuned_piece = best;
  drop_graph(b);
  if (piece_edges_out) *piece_edges_out = best;
  if (ms_per_iter_out) *ms_per_iter_out = best_ms;
  return GAS_OK;
}

}  // extern "C"
