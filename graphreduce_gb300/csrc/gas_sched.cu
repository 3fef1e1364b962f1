// gas_sched.cu -- fast schedules of the built-in programs (BFS, SSSP, CC).
//
// The reference iterates "pull over the active set": A_{k+1} = out-neighbours
// of C_k, the vertices whose apply() returned true, and every active vertex
// folds all of its in-edges (refgas.h:143-214).  For the monotone min
// programs the same vertex data, the same C_k and the same iteration count
// come out of cheaper schedules:
//
//   iteration 0   the generic kernels on the caller's active set (exact);
//   push          every u in C_k sends d_u (+ w) along its out-edges with
//                 atomicMin; v joins C_{k+1} iff a send lowered it.  The d_u
//                 sent are the values at the end of iteration k, captured in
//                 the frontier queue, so the iteration stays bulk-synchronous;
//   dense pull    every vertex folds its in-edges from C_k (bitmap test,
//                 snapshot values), for frontiers whose out-edges are a large
//                 share of the graph.
//
// Why push == pull: after every iteration each edge u->v satisfies
// d_v <= d_u + w unless u is in C_k (induction from iteration 0, which folds
// every in-edge), so in-neighbours outside C_k can neither lower d_v nor make
// apply() return true.  Iteration k+1 exists iff C_k has an out-edge.
//
// BFS (bfs.cu:58-71): C_k = vertices first reached at level k; push marks
// unvisited out-neighbours (plain store of the level, reduction of the
// changed bit); the bottom-up pull lets every unvisited vertex look for an
// in-neighbour in C_k and stop at the first -- the same level k+1 set.
//
// The whole run is one CUDA graph: the iteration-0 kernels, a kernel that
// sets the loop condition, then a WHILE node whose body runs push or pull
// (each kernel returns at once when the other mode is selected), the
// frontier compaction and the condition kernel, which also picks the next
// iteration's mode.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <climits>
#include <cstring>
#include <vector>

#include "gas.h"
#include "gas_device.cuh"
#include "gas_engine_impl.h"
#include "gas_internal.h"
#include "gas_sched.h"
#include "gas_features.h"
#include "gas_learn.h"

using gasdev::kNT;
using gasdev::SegSource;

namespace {

inline cudaStream_t S(void *s) { return (cudaStream_t)s; }

enum { kModePush = 0, kModePull = 1 };

// ---------------------------------------------------------------------------
// iteration 0 -> the changed set
// ---------------------------------------------------------------------------
__global__ void k_seed_changed(const int32_t *act, const uint8_t *ret,
                               const gas_counters *cnt, uint32_t *cbits) {
  const int n = cnt->n_active;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    if (ret[i]) {
      const uint32_t v = (uint32_t)act[i];
      atomicOr(cbits + (v >> 5), 1u << (v & 31));
    }
  }
}

// Iteration 0 from the full vertex range, without folding every in-edge:
// with A_0 = V, a vertex u whose value is not below Program::gatherZero
// contributes min(gatherZero, d_u + w) = gatherZero >= d_v to every
// out-neighbour, so only S = {u : d_u < gatherZero} can change anything.
// Pushing (or dense-pulling) from S is iteration 0 exactly; for SSSP from
// one source S = {source}.
__global__ void k_seed_finite(const int32_t *vd, int nV, int32_t zero_cap,
                              uint32_t *cbits) {
  const int nW = (nV + 31) / 32;
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nW;
       w += gridDim.x * blockDim.x) {
    uint32_t m = 0;
    const int v0 = w * 32;
    const int n = nV - v0 < 32 ? nV - v0 : 32;
    for (int b = 0; b < n; ++b)
      if (vd[v0 + b] < zero_cap) m |= 1u << b;
    cbits[w] = m;
  }
}

// ---------------------------------------------------------------------------
// frontier compaction: changed bitmap -> queue of the members with out-edges,
// in two parts.  Heavy rows [0, q_heavy) (more than kLightDeg out-edges) are
// pushed by the warp slabs and hold (value at the end of the iteration, end
// of the out-edge range in the heavy rows' edge space, CSR position offset);
// light rows [q_heavy, n_changed) are pushed by warp-cooperative runs and
// hold (value, CSR start, out-degree).  Both parts are in vertex order.
// When the next iteration is a dense pull, also the snapshots of all members
// and the members' ids (by which the snapshots are reset afterwards).  One lane per vertex:
// each warp takes a run of 16 bitmap words (lane l < 16 holds word w0 + l)
// and walks it in two rounds of 8 words whose out-degree loads are in
// flight together, skipping a round whose words are all clear; a word's 32
// lanes read their out-degrees coalesced, ballots give queue positions, a
// warp scan gives edge offsets.  The count pass also keeps each warp's
// totals, so the write pass takes its offsets without counting again.
// (8 words per warp, one round, ran CC on R-MAT 22 + islands 6 % slower --
// 4 times as many blocks per pass; 32 words, four rounds, ran single-source
// SSSP 4 % slower -- longer serial chains in its dense iterations.)
// ---------------------------------------------------------------------------
constexpr int kQWordsPerWarp = 16;
constexpr int kQRound = 8;
constexpr int kQWarpsPerBlock = kNT / 32;
constexpr int kQWordsPerBlock = kQWordsPerWarp * kQWarpsPerBlock;  // 128 words
constexpr int kLightDeg = 8;  // rows with at most this many out-edges are light

__device__ __forceinline__ int warp_incl_sum_i(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int o = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += o;
  }
  return v;
}

__device__ __forceinline__ int4 add4(int4 a, int4 b) {
  return make_int4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

// One round: words w0 + r .. w0 + r + 7 of the warp's run (taken from the
// lanes' own words by shuffles); lane l takes vertex 32 w + l of each word,
// so the out-offset loads of a word are coalesced, and the 8 words' loads
// are issued before any of them is used.
struct QRound {
  int off[kQRound];
  int deg[kQRound];  // 0 when the bit is clear
};

__device__ __forceinline__ void q_round_load(uint32_t myword, const int32_t *csr_off, int w0,
                                             int r, QRound &q) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < kQRound; ++i) {
    const uint32_t word = __shfl_sync(0xffffffffu, myword, r + i);
    q.off[i] = 0;
    q.deg[i] = 0;
    if ((word >> lane) & 1u) {
      const int v = (w0 + r + i) * 32 + lane;
      q.off[i] = csr_off[v];
      q.deg[i] = csr_off[v + 1] - q.off[i];
    }
  }
}

// Adds a round's (heavy rows, heavy edges, light rows, light edges) to the
// lane's counts.
__device__ __forceinline__ void q_round_count(const QRound &q, int4 &c) {
#pragma unroll
  for (int i = 0; i < kQRound; ++i) {
    const int d = q.deg[i];
    if (d > kLightDeg) {
      ++c.x;
      c.y += d;
    } else if (d > 0) {
      ++c.z;
      c.w += d;
    }
  }
}

__device__ __forceinline__ int4 warp_sum4(int4 c) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    c.x += __shfl_xor_sync(0xffffffffu, c.x, o);
    c.y += __shfl_xor_sync(0xffffffffu, c.y, o);
    c.z += __shfl_xor_sync(0xffffffffu, c.z, o);
    c.w += __shfl_xor_sync(0xffffffffu, c.w, o);
  }
  return c;
}

// Counts per block (part, for the spine) and per warp (wpart, for the write
// pass), and the queue's out-degree histogram (schedule features).  The
// snapshots are written only for a queue that a dense pull reads: after a
// pull iteration (mode still says so here) the previous queue's snapshots
// (its length is still in the counters) go back to Program::gatherZero
// first.  BFS's bottom-up pass reads depths, never snapshots (bfs != 0:
// none are written or reset).
__global__ void __launch_bounds__(kNT)
    k_q_count(const uint32_t *cbits, const int32_t *csr_off, int nW,
              int4 *part, int4 *wpart, const int32_t *q_ids, int32_t *snap, int32_t zero,
              int32_t *hist, const gas_counters *cnt, int bfs) {
  if (!bfs && cnt->mode == kModePull) {
    const int n_old = cnt->n_changed;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_old;
         i += gridDim.x * blockDim.x)
      snap[q_ids[i]] = zero;
  }
  __shared__ int4 s_t[kQWarpsPerBlock];
  __shared__ int s_hist[8];
  if (threadIdx.x < 8) s_hist[threadIdx.x] = 0;
  if (hist) __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w0 = (blockIdx.x * kQWarpsPerBlock + warp) * kQWordsPerWarp;
  const uint32_t myword =
      lane < kQWordsPerWarp && w0 + lane < nW ? cbits[w0 + lane] : 0u;
  const unsigned nz = __ballot_sync(0xffffffffu, myword != 0u);
  int4 c = make_int4(0, 0, 0, 0);
#pragma unroll 1
  for (int r = 0; r < kQWordsPerWarp; r += kQRound) {
    if (!((nz >> r) & ((1u << kQRound) - 1u))) continue;  // warp-uniform
    QRound q;
    q_round_load(myword, csr_off, w0, r, q);
    q_round_count(q, c);
    if (hist) {
#pragma unroll
      for (int i = 0; i < kQRound; ++i)
        if (q.deg[i] > 0) atomicAdd(&s_hist[gasfeat::degree_bucket(q.deg[i])], 1);
    }
  }
  const int4 t = warp_sum4(c);
  if (lane == 0) {
    s_t[warp] = t;
    wpart[blockIdx.x * kQWarpsPerBlock + warp] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int4 b = make_int4(0, 0, 0, 0);
    for (int k = 0; k < kQWarpsPerBlock; ++k) b = add4(b, s_t[k]);
    part[blockIdx.x] = b;
  }
  if (hist && threadIdx.x < 8 && s_hist[threadIdx.x])
    atomicAdd(hist + threadIdx.x, s_hist[threadIdx.x]);
}

constexpr int kSpineNT = 1024;  // k_q_spine (with the loop control, below)
constexpr int kBfsPullDiv = 16;  // BFS pull_div of the counters (unused by its AUTO rule)
// BFS AUTO: the direction rule of Beamer, Asanovic & Patterson ("Direction-
// Optimizing Breadth-First Search", SC'12) with the paper's constants.  A
// top-down level is followed by a bottom-up one when the queue's out-edges
// exceed 1/alpha of the edges not yet explored (E minus the out-edges of
// every earlier level's queue); bottom-up levels continue while the queue
// grows or holds more than V/beta vertices.
constexpr int kBfsAlpha = 14;
constexpr int kBfsBeta = 24;
constexpr int kSpineRegs = 4;

// Queue positions of a warp's next rows: heavy row, heavy-edge offset,
// light row.
struct QPos {
  int bq, bd, lq;
};

// The queue entries of one round (its words' members in q, their values in
// val), from heavy position p.bq, heavy-edge offset p.bd and light position
// p.lq on; advances p.  chunk_row: the push's partition in (1 << cl)-edge
// chunks.
__device__ __forceinline__ void q_round_write(const QRound &q, const int *val, QPos &p,
                                              int wr, int cl, bool want_snap,
                                              int32_t *q_ids, int32_t *q_vals, int32_t *q_end,
                                              int32_t *q_delta, int32_t *snap,
                                              int32_t *chunk_row) {
  const int lane = threadIdx.x & 31;
  int bq = p.bq, bd = p.bd, lq = p.lq;
  const unsigned below = (1u << lane) - 1u;
#pragma unroll
  for (int i = 0; i < kQRound; ++i) {
    const int deg = q.deg[i];
    const bool heavy = deg > kLightDeg;
    const unsigned hb = __ballot_sync(0xffffffffu, heavy);
    const unsigned lb = __ballot_sync(0xffffffffu, deg > 0 && !heavy);
    if (!(hb | lb)) continue;  // warp-uniform
    const int v = (wr + i) * 32 + lane;
    if (hb) {  // warp-uniform
      const int incl = warp_incl_sum_i(heavy ? deg : 0);
      if (heavy) {
        const int pos = bq + __popc(hb & below);
        const int end = bd + incl;
        if (want_snap) q_ids[pos] = v;  // only a pull's snapshots are reset by id
        q_vals[pos] = val[i];
        q_end[pos] = end;
        q_delta[pos] = q.off[i] - (end - deg);
        // the push's chunk partition: every (1 << cl)-edge chunk that
        // starts inside this row's heavy-edge range starts in row pos
        for (int c = (end - deg + (1 << cl) - 1) >> cl; (c << cl) < end; ++c)
          chunk_row[c] = pos;
      }
      bq += __popc(hb);
      bd += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (deg > 0 && !heavy) {
      const int pos = lq + __popc(lb & below);
      if (want_snap) q_ids[pos] = v;
      q_vals[pos] = val[i];
      q_end[pos] = deg;
      q_delta[pos] = q.off[i];
    }
    lq += __popc(lb);
    if (want_snap && deg > 0) snap[v] = val[i];
  }
  p.bq = bq;
  p.bd = bd;
  p.lq = lq;
}

// (at most 48 registers: 5 CTAs per SM, so a sparse iteration's mostly
// empty bitmap runs pass in fewer waves)
__global__ void __launch_bounds__(kNT, 5)
    k_q_write(uint32_t *cbits, const int32_t *csr_off, int nW, const int4 *part,
              const int4 *wpart, const int32_t *vd, int32_t *q_ids, int32_t *q_vals,
              int32_t *q_end, int32_t *q_delta, int32_t *snap, int32_t *chunk_row,
              const gas_counters *cnt, int bfs) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w0 = (blockIdx.x * kQWarpsPerBlock + warp) * kQWordsPerWarp;
  const uint32_t myword =
      lane < kQWordsPerWarp && w0 + lane < nW ? cbits[w0 + lane] : 0u;
  if (bfs && cnt->mode == kModePull) {  // grid-uniform: the next BFS level is
    // bottom-up and reads depths, so only the changed bitmap is cleared
    if (myword) cbits[w0 + lane] = 0u;
    return;
  }
  const unsigned nz = __ballot_sync(0xffffffffu, myword != 0u);
  if (!nz) return;  // warp-uniform: no member, no word to clear
  int4 base = part[blockIdx.x];
  for (int k = 0; k < warp; ++k) base = add4(base, wpart[blockIdx.x * kQWarpsPerBlock + k]);
  QPos p{base.x, base.y, cnt->q_heavy + base.z};
  const int cl = cnt->push_chunk_log2;
  const bool want_snap = !bfs && cnt->mode == kModePull;  // the next iteration's mode
#pragma unroll 1
  for (int r = 0; r < kQWordsPerWarp; r += kQRound) {
    if (!((nz >> r) & ((1u << kQRound) - 1u))) continue;  // warp-uniform
    QRound q;
    q_round_load(myword, csr_off, w0, r, q);
    int val[kQRound];
#pragma unroll
    for (int i = 0; i < kQRound; ++i)
      val[i] = q.deg[i] > 0 ? vd[(w0 + r + i) * 32 + lane] : 0;
    q_round_write(q, val, p, w0 + r, cl, want_snap, q_ids, q_vals, q_end, q_delta, snap,
                  chunk_row);
  }
  if (myword) cbits[w0 + lane] = 0u;
}

// Edge-stream load that does not allocate in L1: the edge arrays are read
// once per iteration, and L1 is kept for the vertex state the pre-checks
// gather.
__device__ __forceinline__ int32_t ld_stream(const int32_t *p) {
  int32_t v;
  asm("ld.global.nc.L1::no_allocate.b32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}

// ---------------------------------------------------------------------------
// push (SSSP / CC) and BFS push
// ---------------------------------------------------------------------------
template <bool kWeighted>
struct PushPol {
  typedef int32_t Val;
  static constexpr bool kMapNeedsVertex = false;
  const int32_t *csr_dst;
  const int32_t *csr_w;
  const int32_t *q_vals;
  int32_t *vd;
  uint32_t *cbits;
  int32_t zero_cap;  // Program::gatherZero: gather results never exceed it
  __device__ Val zero() const { return 0; }
  __device__ Val reduce(Val a, Val) const { return a; }
  __device__ Val map(int, int, int) const { return 0; }
  __device__ void emit(int, int, Val) const {}
  // The pre-check is a plain (L1-cacheable) load: any value it returns was
  // held by the vertex during this iteration (L1 starts each kernel empty),
  // so it lies between the iteration's start value and the final one; cand
  // >= it means cand cannot lower the vertex, and cand < it means the vertex
  // ends the iteration below its start value -- it changed -- so the bit is
  // set without waiting for the atomic's result; both updates are
  // fire-and-forget reductions.
  struct Probe {
    int v, cand, cur;
  };
  __device__ __forceinline__ Probe probe(bool valid, int a, int, int pos) const {
    Probe p{0, 0, INT_MIN};
    if (valid) {
      p.v = ld_stream(csr_dst + pos);
      int cand = __ldg(q_vals + a);
      if (kWeighted) cand += ld_stream(csr_w + pos);
      p.cand = cand > zero_cap ? zero_cap : cand;
      p.cur = vd[p.v];
    }
    return p;
  }
  __device__ __forceinline__ void commit(const Probe &p) const {
    if (p.cand < p.cur) {
      atomicMin(vd + p.v, p.cand);
      atomicOr(cbits + ((uint32_t)p.v >> 5), 1u << (p.v & 31));
    }
  }
};

struct BfsPushPol {
  typedef int32_t Val;
  static constexpr bool kMapNeedsVertex = false;
  const int32_t *csr_dst;
  int32_t *depth;
  uint32_t *cbits;
  int32_t level;
  __device__ Val zero() const { return 0; }
  __device__ Val reduce(Val a, Val) const { return a; }
  __device__ Val map(int, int, int) const { return 0; }
  __device__ void emit(int, int, Val) const {}
  // Every writer of an iteration stores the same level, so a vertex seen
  // unreached (a plain load: a stale -1 only repeats the same store) is
  // claimed with a plain store and its bit set with a reduction.
  struct Probe {
    int v;
    bool unreached;
  };
  __device__ __forceinline__ Probe probe(bool valid, int, int, int pos) const {
    Probe p{0, false};
    if (valid) {
      p.v = ld_stream(csr_dst + pos);
      p.unreached = depth[p.v] == -1;
    }
    return p;
  }
  __device__ __forceinline__ void commit(const Probe &p) const {
    if (p.unreached) {
      __stcg(depth + p.v, level);
      atomicOr(cbits + ((uint32_t)p.v >> 5), 1u << (p.v & 31));
    }
  }
};

// Light queue rows [q_heavy, n_changed): a warp takes 32 consecutive rows
// (their CSR start and out-degree, at most kLightDeg, in registers; in the
// queue arrays a light row holds its CSR start in q_delta and its
// out-degree in q_end), lays their edges end to end -- at most 32 * kLightDeg
// of them -- and walks them 32 at a time, two rounds in flight: a ballot of
// the row starts gives each lane its row, a shuffle its CSR position.  When
// the rows are CSR neighbours (a dense frontier) the edge loads are
// coalesced; no per-edge global loads beyond the policy's own.
template <class Pol>
__device__ __forceinline__ void light_loop(const Pol &pol, const int32_t *q_start,
                                           const int32_t *q_deg, const gas_counters *cnt) {
  constexpr unsigned FULL = 0xffffffffu;
  const int n0 = cnt->q_heavy, n1 = cnt->n_changed;
  const int lane = threadIdx.x & 31;
  const int gwarp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  // the next batch's rows are loaded before this batch's edges are walked
  int nstart = 0, ndeg = 0;
  {
    const int i = n0 + gwarp * 32 + lane;
    if (i < n1) {
      nstart = __ldg(q_start + i);
      ndeg = __ldg(q_deg + i);
    }
  }
  for (int base = n0 + gwarp * 32; base < n1; base += nwarps * 32) {
    const int i = base + lane;
    const bool ok = i < n1;
    const int start = nstart;
    const int deg = ndeg;
    {
      const int j = i + nwarps * 32;
      nstart = j < n1 ? __ldg(q_start + j) : 0;
      ndeg = j < n1 ? __ldg(q_deg + j) : 0;
    }
    const int incl = warp_incl_sum_i(deg);
    const int excl = incl - deg;       // the row's first edge in the warp's run
    const int shift = start - excl;    // CSR position - run index, per row
    const int T = __shfl_sync(FULL, incl, 31);
    for (int r = 0; r < T; r += 64) {
      int pos[2], row[2];
      bool valid[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r0 = r + 32 * h;
        // row of edge r0: the last row starting at or before it
        const int row0 = __popc(__ballot_sync(FULL, ok && excl <= r0)) - 1;
        const int k = excl - r0;  // rows starting inside the round
        const unsigned starts =
            __reduce_or_sync(FULL, (ok && k >= 1 && k < 32) ? (1u << k) : 0u);
        int rw = row0 + __popc(starts & ((2u << lane) - 1u));
        rw = rw < 0 ? 0 : (rw > 31 ? 31 : rw);
        const int e = r0 + lane;
        valid[h] = e < T;
        row[h] = rw;
        pos[h] = e + __shfl_sync(FULL, shift, rw);
      }
      const typename Pol::Probe pa = pol.probe(valid[0], base + row[0], 0, pos[0]);
      const typename Pol::Probe pb = pol.probe(valid[1], base + row[1], 0, pos[1]);
      pol.commit(pa);
      pol.commit(pb);
    }
  }
}

// The queue's heavy rows by warp slabs, then its light rows.
template <class Pol>
__global__ void __launch_bounds__(kNT)
    k_push(Pol pol, gasdev::SlabSource src, const gas_counters *cnt) {
  if (cnt->mode != kModePush) return;
  gasdev::slab_loop<Pol, false>(pol, src, nullptr, nullptr, nullptr, nullptr, nullptr);
  light_loop(pol, src.delta, src.ends, cnt);
}

__global__ void __launch_bounds__(kNT)
    k_bfs_push(BfsPushPol pol, gasdev::SlabSource src, const gas_counters *cnt) {
  if (cnt->mode != kModePush) return;
  pol.level = cnt->iteration;
  gasdev::slab_loop<BfsPushPol, false>(pol, src, nullptr, nullptr, nullptr, nullptr,
                                       nullptr);
  light_loop(pol, src.delta, src.ends, cnt);
}

// Bottom-up BFS level: a thread per vertex; an unvisited vertex reads its
// first in-edge, then the rest four at a time (indices, then the sources'
// depths), and stops at the first source reached at the previous level.  A source claimed in this
// same pass reads as -1 or as the new level, never as the previous one, so
// the level set is exactly the push's.
__global__ void __launch_bounds__(kNT)
    k_bfs_pull(const int32_t *csc_off, const int32_t *csc_src, int32_t *depth,
               uint32_t *cbits, int nV, const gas_counters *cnt) {
  if (cnt->mode != kModePull) return;
  const int level = cnt->iteration, prev = level - 1;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    if (depth[v] != -1) continue;
    const int b = __ldg(csc_off + v), end = __ldg(csc_off + v + 1);
    // the first in-edge alone first: sources are in id order and low ids
    // are the hubs, so the first is the likeliest parent
    bool found = b < end && depth[ld_stream(csc_src + b)] == prev;
    for (int i = b + 1; i < end && !found; i += 4) {
      int u[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) u[j] = i + j < end ? ld_stream(csc_src + i + j) : -1;
#pragma unroll
      for (int j = 0; j < 4; ++j) found |= u[j] >= 0 && depth[u[j]] == prev;
    }
    if (found) {
      __stcg(depth + v, level);
      atomicOr(cbits + ((uint32_t)v >> 5), 1u << (v & 31));
    }
  }
}

// ---------------------------------------------------------------------------
// dense pull (SSSP / CC): every vertex folds the in-edges from C_k
// ---------------------------------------------------------------------------
template <bool kWeighted>
struct PullPol {
  typedef int32_t Val;
  static constexpr bool kMapNeedsVertex = false;
  static constexpr bool kIntMin = true;  // reduce is min over int
  const int32_t *csc_src;
  const int32_t *csc_w;
  const int32_t *snap;   // value of u at the end of iteration k if u is in
                         // C_k (and has out-edges), else Program::gatherZero
  int32_t *vd;
  uint32_t *cbits;
  int32_t zero_cap;
  __device__ Val zero() const { return INT_MAX; }
  __device__ __forceinline__ Val reduce(Val a, Val b) const { return a < b ? a : b; }
  __device__ __forceinline__ Val map(int, int, int pos) const {
    const int u = __ldg(csc_src + pos);
    int c = kWeighted ? __ldg(csc_w + pos) : 0;
    c += snap[u];  // a non-member gives gatherZero (+w), which changes nothing
    return c > zero_cap ? zero_cap : c;
  }
  __device__ __forceinline__ void emit(int, int v, Val g) const {
    if (g < vd[v]) {
      vd[v] = g;
      atomicOr(cbits + ((uint32_t)v >> 5), 1u << (v & 31));
    }
  }
};

template <class Pol>
__global__ void __launch_bounds__(kNT)
    k_pull(Pol pol, gasdev::SlabSource src, int32_t *cf, int32_t *cc, int32_t *ca0,
           int32_t *fix, int32_t *fix_n, const gas_counters *cnt) {
  if (cnt->mode != kModePull) return;
  gasdev::slab_loop<Pol, true>(pol, src, cf, cc, ca0, fix, fix_n);
}

template <class Pol>
__global__ void __launch_bounds__(kNT)
    k_pull_fixup(Pol pol, gasdev::SlabSource src, const int32_t *cf, const int32_t *cc,
                 const int32_t *ca0, const int32_t *fix, const int32_t *fix_n,
                 const gas_counters *cnt) {
  if (cnt->mode != kModePull) return;
  gasdev::slab_fixup_loop<Pol>(pol, src, cf, cc, ca0, fix, fix_n);
}

// ---------------------------------------------------------------------------
// loop control
// ---------------------------------------------------------------------------
// Loop-control state captured into the graph.
struct LoopCtl {
  cudaGraphConditionalHandle h;
  int in_graph;
  int nV;
  int nE;
  int weighted;
  int bfs;
  const __nv_bfloat16 *model;  // schedule head (LEARNED), or null
  gas_trace_record *trace;     // per-iteration records, or null
  int32_t *hist;               // degree histogram of the queue, or null
  int32_t *fix_n;
};

// The schedule head's weights (10.5 KB, BF16) staged in shared memory by
// the spine kernel at its start, while the block totals are still loading.
constexpr int kSchedW = (int)gaslearn::layout(GAS_SCHED_FEATURES, 2).total;
struct SchedSmem {
  __nv_bfloat16 w[kSchedW];
  float f[GAS_SCHED_FEATURES];
  float h1[gaslearn::kH];
  float h2p[4][gaslearn::kH];
  float h2[gaslearn::kH];
};

__device__ __forceinline__ void sched_stage_weights(SchedSmem &sm, const __nv_bfloat16 *model) {
  const uint4 *src = reinterpret_cast<const uint4 *>(model);
  uint4 *dst = reinterpret_cast<uint4 *>(sm.w);
  constexpr int kVec = kSchedW * 2 / 16;
  for (int i = threadIdx.x; i < kVec; i += blockDim.x) dst[i] = src[i];
  for (int i = kVec * 8 + threadIdx.x; i < kSchedW; i += blockDim.x) sm.w[i] = model[i];
}

// The head's two logits, evaluated by the whole CTA (at least 256 threads,
// every thread calls): layer 1 one unit per thread, layer 2 four partial
// sums per unit, the output layer by warp 0.  FP32 accumulation of the BF16
// weights; the result is in lg[] of warp 0.
__device__ __forceinline__ void sched_logits_cta(SchedSmem &sm, float *lg) {
  constexpr gaslearn::Layout L = gaslearn::layout(GAS_SCHED_FEATURES, 2);
  constexpr int kH = gaslearn::kH;
  const int t = threadIdx.x;
  if (t < kH) {
    float a = __bfloat162float(sm.w[L.b1 + t]);
#pragma unroll
    for (int i = 0; i < GAS_SCHED_FEATURES; ++i) a += sm.f[i] * __bfloat162float(sm.w[L.w1 + i * kH + t]);
    sm.h1[t] = a > 0.f ? a : 0.f;
  }
  __syncthreads();
  if (t < 4 * kH) {
    const int j = t % kH, q = t / kH;
    float a = 0.f;
#pragma unroll
    for (int i = q * (kH / 4); i < (q + 1) * (kH / 4); ++i)
      a += sm.h1[i] * __bfloat162float(sm.w[L.w2 + i * kH + j]);
    sm.h2p[q][j] = a;
  }
  __syncthreads();
  if (t < kH) {
    const float a = __bfloat162float(sm.w[L.b2 + t]) + sm.h2p[0][t] + sm.h2p[1][t] +
                    sm.h2p[2][t] + sm.h2p[3][t];
    sm.h2[t] = a > 0.f ? a : 0.f;
  }
  __syncthreads();
  if (t < 32) {
    float o0 = 0.f, o1 = 0.f;
#pragma unroll
    for (int j = t; j < kH; j += 32) {
      o0 += sm.h2[j] * __bfloat162float(sm.w[L.w3 + 2 * j]);
      o1 += sm.h2[j] * __bfloat162float(sm.w[L.w3 + 2 * j + 1]);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      o0 += __shfl_xor_sync(0xffffffffu, o0, d);
      o1 += __shfl_xor_sync(0xffffffffu, o1, d);
    }
    lg[0] = o0 + __bfloat162float(sm.w[L.b3]);
    lg[1] = o1 + __bfloat162float(sm.w[L.b3 + 1]);
  }
}

// Mode of the next iteration (every thread of the spine CTA calls; the
// counters of the new queue are written): forced push / pull, the learned
// head (weights already staged when `learned`), or the fixed heuristic --
// pull when the frontier's out-edges are more than 1/pull_div of all edges.
// With tracing, records the iteration.
// The loop state schedule_next decides from, as thread 0 of the spine holds
// it in registers (the new queue's counts and the counters it read once at
// the kernel's start).
struct LoopVals {
  int sched;  // 0 auto, 1 push, 2 pull, 3 learned
  int it;     // the iteration being scheduled
  int n_changed, n_scatter_edges, pull_div, cond;
  int mode;                     // the mode of the iteration that built the queue
  int seen_edges, prev_changed;  // BFS: see gas_counters
};

__device__ void schedule_next(gas_counters *cnt, const LoopCtl &c, long long now,
                              SchedSmem &sm, bool learned, const LoopVals &v) {
  const int t = threadIdx.x;
  float lg[2] = {0.f, 0.f};
  if (learned) {  // CTA-uniform
    if (t == 0)
      gasfeat::schedule_features(v.n_changed, v.n_scatter_edges, c.hist, v.it, c.nV, c.nE,
                                 c.weighted, sm.f);
    __syncthreads();
    sched_logits_cta(sm, lg);
  }
  if (t == 0) {
    int mode;
    if (v.sched == 1)
      mode = kModePush;
    else if (v.sched == 2)
      mode = kModePull;
    else if (learned)
      mode = lg[1] > lg[0] ? kModePull : kModePush;
    else if (c.bfs && v.mode == kModePush)
      mode = (long long)v.n_scatter_edges * kBfsAlpha > (long long)c.nE - v.seen_edges
                 ? kModePull : kModePush;
    else if (c.bfs)
      mode = (v.n_changed >= v.prev_changed || (long long)v.n_changed * kBfsBeta > c.nV)
                 ? kModePull : kModePush;
    else
      mode = ((long long)v.n_scatter_edges * v.pull_div > (long long)c.nE) ? kModePull
                                                                           : kModePush;
    cnt->mode = mode;
    if (c.trace && v.it < GAS_TRACE_CAP && v.cond) {
      gas_trace_record &r = c.trace[v.it];
      r.iteration = v.it;
      r.mode = mode;
      r.n_queue = v.n_changed;
      r.n_edges_out = v.n_scatter_edges;
      for (int b = 0; b < 8; ++b) r.hist[b] = c.hist ? c.hist[b] : 0;
      r.t_start_ns = now;
      r.t_end_ns = 0;
    }
    if (c.hist)
      for (int b = 0; b < 8; ++b) c.hist[b] = 0;
    if (c.in_graph) cudaGraphSetConditional(c.h, v.cond);
  }
}

__device__ __forceinline__ long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return (long long)t;
}

// Exclusive scan of the block totals in one pass: 1024 threads, thread t
// holds a run of ceil(nb / 1024) consecutive blocks in registers (16-byte
// loads, all issued before the first is used), one CTA scan, then the runs
// are rewritten as prefixes.  Also picks the push's chunk size for the new
// queue: 512 heavy edges per warp chunk, halved (down to 64) while the heavy
// edges would give fewer than two chunks per push warp, so that a small
// frontier still spreads over the GPU instead of running as a few long
// per-warp chains of dependent loads.  Then the loop control, once per
// iteration: counters, the WHILE condition and the next iteration's mode.
// phase 0: the prologue's queue (seeded: iteration 0 itself runs in the
// loop, and always exists: A_0 = V is not empty); phase 1: the queue an
// iteration built.
__global__ void __launch_bounds__(kSpineNT)
    k_q_spine(int4 *part, int nb, gas_counters *cnt, int push_warps, LoopCtl c,
              int phase, int seeded) {
  const long long now = global_ns();
  __shared__ __align__(16) SchedSmem sm;
  const bool learned = cnt->sched == 3 && c.model != nullptr;
  if (learned) sched_stage_weights(sm, c.model);
  // thread 0: every counter the loop control reads, in five 16-byte loads
  // issued with the block totals' (gas_counters is 80 bytes at the start of
  // a cudaMalloc block), instead of one dependent load after each store
  gas_counters k;
  if (threadIdx.x == 0) {
    constexpr int kWords = (int)(sizeof(gas_counters) / sizeof(int4));
    static_assert(sizeof(gas_counters) == kWords * sizeof(int4), "gas_counters layout");
    const int4 *p = reinterpret_cast<const int4 *>(cnt);
    int4 r[kWords];
#pragma unroll
    for (int i = 0; i < kWords; ++i) r[i] = p[i];
    memcpy(&k, r, sizeof(k));
  }
  const int per = (nb + kSpineNT - 1) / kSpineNT;
  const int b0 = threadIdx.x * per, b1 = min(nb, b0 + per);
  const bool in_regs = per <= kSpineRegs;
  int4 x[kSpineRegs];
  int4 sum = make_int4(0, 0, 0, 0);
  if (in_regs) {
#pragma unroll
    for (int k = 0; k < kSpineRegs; ++k)
      x[k] = b0 + k < b1 ? part[b0 + k] : make_int4(0, 0, 0, 0);
#pragma unroll
    for (int k = 0; k < kSpineRegs; ++k) sum = add4(sum, x[k]);
  } else {
    for (int b = b0; b < b1; ++b) sum = add4(sum, part[b]);
  }
  // CTA exclusive scan of the four sums
  __shared__ int4 s_warp[kSpineNT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int4 incl = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int4 o;
    o.x = __shfl_up_sync(0xffffffffu, incl.x, d);
    o.y = __shfl_up_sync(0xffffffffu, incl.y, d);
    o.z = __shfl_up_sync(0xffffffffu, incl.z, d);
    o.w = __shfl_up_sync(0xffffffffu, incl.w, d);
    if (lane >= d) incl = add4(incl, o);
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  int4 pre = make_int4(incl.x - sum.x, incl.y - sum.y, incl.z - sum.z, incl.w - sum.w);
  int4 tot = make_int4(0, 0, 0, 0);
#pragma unroll 8
  for (int w = 0; w < kSpineNT / 32; ++w) {
    const int4 t = s_warp[w];
    if (w < warp) pre = add4(pre, t);
    tot = add4(tot, t);
  }
  if (in_regs) {
#pragma unroll
    for (int k = 0; k < kSpineRegs; ++k) {
      if (b0 + k < b1) {
        part[b0 + k] = pre;
        pre = add4(pre, x[k]);
      }
    }
  } else {
    for (int b = b0; b < b1; ++b) {
      const int4 y = part[b];
      part[b] = pre;
      pre = add4(pre, y);
    }
  }
  LoopVals v{};
  if (threadIdx.x == 0) {
    v.sched = k.sched;
    v.pull_div = k.pull_div;
    v.mode = phase == 0 ? kModePush : k.mode;
    v.n_changed = tot.x + tot.z;        // queue length (members with out-edges)
    v.n_scatter_edges = tot.y + tot.w;  // their out-edges
    // the queue just expanded joins the explored levels
    v.seen_edges = phase == 0 ? 0 : k.seen_edges + k.n_scatter_edges;
    v.prev_changed = phase == 0 ? 0 : k.n_changed;
    cnt->seen_edges = v.seen_edges;
    cnt->prev_changed = v.prev_changed;
    cnt->n_changed = v.n_changed;
    cnt->n_scatter_edges = v.n_scatter_edges;
    cnt->q_heavy = tot.x;
    cnt->q_heavy_edges = tot.y;
    int cl = gasdev::kSlabChunkLog2;
    while (cl > gasdev::kSlabChunkMinLog2 && (tot.y >> cl) < 2 * push_warps) --cl;
    cnt->push_chunk_log2 = cl;
    const bool edges = v.n_scatter_edges > 0;
    if (phase == 0) {
      const int done = seeded ? 0 : 1;  // iterations run by the prologue
      const bool more = seeded ? true : edges;
      if (more && done >= k.max_iter) cnt->error = GAS_ERR_ITER_CAP;
      v.it = done;
      v.cond = (more && done < k.max_iter) ? 1 : 0;
    } else {
      *c.fix_n = 0;  // the pull fixup of this iteration has run
      if (k.mode == kModePush)
        cnt->n_push = k.n_push + 1;
      else
        cnt->n_pull = k.n_pull + 1;
      if (c.trace && k.iteration < GAS_TRACE_CAP) c.trace[k.iteration].t_end_ns = now;
      v.it = k.iteration + 1;
      if (edges && v.it >= k.max_iter) cnt->error = GAS_ERR_ITER_CAP;
      v.cond = (edges && v.it < k.max_iter) ? 1 : 0;
    }
    cnt->iteration = v.it;
    cnt->cond = v.cond;
  }
  __syncthreads();  // the staged weights
  schedule_next(cnt, c, now, sm, learned, v);
}


__global__ void k_fast_reset(gas_counters *cnt, int max_iter, int forced,
                             int pull_div) {
  cnt->iteration = 0;
  cnt->error = 0;
  cnt->max_iter = max_iter;
  cnt->n_push = 0;
  cnt->n_pull = 0;
  cnt->sched = forced;
  cnt->pull_div = pull_div;
  cnt->mode = kModePush;
  cnt->n_changed = 0;  // no previous queue whose snapshots need resetting
}

__global__ void k_fast_finish(gas_counters *cnt) {
  // the reference's active set is empty after run()
  if (!cnt->error) cnt->n_active = 0;
}

struct FastCtx {
  int nW;
  int n_qblocks;
  int slab_grid;  // resident CTAs of the pull slab kernel
  int push_grid;  // resident CTAs of the push kernel
  bool seeded;  // iteration 0 from the full range via the finite-value seed
};

LoopCtl loop_ctl(const gas_engine *e, cudaGraphConditionalHandle h) {
  LoopCtl c;
  c.h = h;
  c.in_graph = e->in_graph ? 1 : 0;
  c.nV = e->nV;
  c.nE = e->nE;
  c.weighted = e->prog == GAS_PROG_SSSP ? 1 : 0;
  c.bfs = e->prog == GAS_PROG_BFS ? 1 : 0;
  c.model = static_cast<const __nv_bfloat16 *>(e->sched_model);
  c.trace = e->trace_on ? e->trace : nullptr;
  c.hist = (e->trace_on || e->sched_model) ? e->hist : nullptr;
  c.fix_n = e->slab_fix_n;
  return c;
}

int32_t snap_zero(const gas_engine *e) {
  return e->prog == GAS_PROG_SSSP ? INT_MAX - 100000 : INT_MAX;
}

// The queue of the changed set, then the loop control (phase as for
// k_q_spine).
gas_status_t compaction(gas_engine *e, cudaStream_t cs, const FastCtx &c,
                        cudaGraphConditionalHandle h, int phase) {
  int4 *part = reinterpret_cast<int4 *>(e->qpart);
  int4 *wpart = part + c.n_qblocks;  // per-warp totals after the block totals
  int32_t *hist = (e->trace_on || e->sched_model) ? e->hist : nullptr;
  const int bfs = e->prog == GAS_PROG_BFS ? 1 : 0;
  k_q_count<<<c.n_qblocks, kNT, 0, cs>>>(e->cbits, e->csr_off, c.nW, part, wpart, e->q_ids,
                                         e->snap, snap_zero(e), hist, e->cnt, bfs);
  k_q_spine<<<1, kSpineNT, 0, cs>>>(part, c.n_qblocks, e->cnt, c.push_grid * (kNT / 32),
                                    loop_ctl(e, h), phase, c.seeded ? 1 : 0);
  k_q_write<<<c.n_qblocks, kNT, 0, cs>>>(e->cbits, e->csr_off, c.nW, part, wpart,
                                         (const int32_t *)e->vd, e->q_ids, e->q_vals,
                                         e->q_end, e->q_delta, e->snap, e->slab_qpart,
                                         e->cnt, bfs);
  CUDA_TRY(cudaGetLastError());
  return GAS_OK;
}

gasdev::SlabSource dense_csc(const gas_engine *e) {
  return gasdev::slab_source(e->ne_end, e->ne_vid, nullptr, e->n_ne, e->nE, nullptr,
                             nullptr, e->slab_dpart);
}

__global__ void k_fill(int32_t *p, int32_t v, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = v;
}

gas_status_t prologue(gas_engine *e, cudaStream_t cs, cudaGraphConditionalHandle h,
                      void *vctx) {
  const FastCtx &c = *static_cast<const FastCtx *>(vctx);
  k_fill<<<2 * e->num_sms, kNT, 0, cs>>>(e->snap, snap_zero(e), e->nV);
  if (c.seeded) {
    const int32_t zero_cap = e->prog == GAS_PROG_SSSP ? INT_MAX - 100000 : INT_MAX;
    k_seed_finite<<<2 * e->num_sms, kNT, 0, cs>>>((const int32_t *)e->vd, e->nV,
                                                  zero_cap, e->cbits);
    CUDA_TRY(cudaGetLastError());
    gasdev::k_slab_partition<><<<2 * e->num_sms, 256, 0, cs>>>(dense_csc(e), e->slab_dpart);
    return compaction(e, cs, c, h, 0);
  }
  // iteration 0: the generic kernels on the caller's active set
  e->level_from_counters = true;
  if (e->prog == GAS_PROG_BFS) {
    GAS_TRY(gas::engine_apply_only(e, cs));
  } else {
    GAS_TRY(gas::engine_gather_apply(e, cs));
    GAS_TRY(gas::engine_commit(e, cs));
  }
  e->level_from_counters = false;
  k_seed_changed<<<8 * e->num_sms, kNT, 0, cs>>>(e->act, e->ret, e->cnt, e->cbits);
  CUDA_TRY(cudaGetLastError());
  if (e->prog != GAS_PROG_BFS)  // chunk boundaries of the dense pull
    gasdev::k_slab_partition<><<<2 * e->num_sms, 256, 0, cs>>>(dense_csc(e), e->slab_dpart);
  return compaction(e, cs, c, h, 0);
}

gas_status_t body(gas_engine *e, cudaStream_t cs, cudaGraphConditionalHandle h,
                  void *vctx) {
  const FastCtx &c = *static_cast<const FastCtx *>(vctx);
  const gasdev::SlabSource qsrc = gasdev::slab_source(
      e->q_end, e->q_ids, e->q_delta, 0, 0, &e->cnt->q_heavy,
      &e->cnt->q_heavy_edges, e->slab_qpart, &e->cnt->push_chunk_log2);
  const int grid = c.slab_grid;  // resident CTAs only (persistent warps)
  const int pgrid = c.push_grid;
  const int32_t zero_cap = e->prog == GAS_PROG_SSSP ? INT_MAX - 100000 : INT_MAX;
  const gasdev::SlabSource dsrc = dense_csc(e);
  int32_t *cf = (int32_t *)e->slab_first, *cc = (int32_t *)e->slab_carry;
  // profiling (host loop only): the mode of this iteration was read back
  // with the counters before the launch
  const bool prof_pull = e->profiling && !e->in_graph && e->h_cnt->mode == kModePull;
  const int64_t wbytes = e->prog == GAS_PROG_SSSP ? 4 : 0;
  if (e->profiling && !e->in_graph) {
    if (prof_pull && e->prog == GAS_PROG_BFS)  // bottom-up: the dense depth and
      // offset reads only (the in-edges inspected before each early exit are
      // not counted, so this is a lower bound)
      gas::prof_begin(e, cs, gas::kProfPull, 12LL * e->nV);
    else if (prof_pull)  // per edge index (+ weight) + state or bitmap; per row 16 B
      gas::prof_begin(e, cs, gas::kProfPull, (8 + wbytes) * e->nE + 16LL * e->n_ne);
    else  // per pushed edge dst (+ weight) + state; per queue entry 16 B
      gas::prof_begin(e, cs, gas::kProfPush,
                      (8 + wbytes) * (int64_t)e->h_cnt->n_scatter_edges +
                          16LL * e->h_cnt->n_changed);
  }
  if (e->prog == GAS_PROG_BFS) {
    BfsPushPol pol{e->csr_dst, (int32_t *)e->vd, e->cbits, 0};
    k_bfs_push<<<pgrid, kNT, 0, cs>>>(pol, qsrc, e->cnt);
    k_bfs_pull<<<grid, kNT, 0, cs>>>(e->csc_off, e->csc_src, (int32_t *)e->vd, e->cbits,
                                     e->nV, e->cnt);
  } else if (e->prog == GAS_PROG_SSSP) {
    PushPol<true> pol{e->csr_dst, (const int32_t *)e->csr_ed, e->q_vals,
                      (int32_t *)e->vd, e->cbits, zero_cap};
    k_push<decltype(pol)><<<pgrid, kNT, 0, cs>>>(pol, qsrc, e->cnt);
    PullPol<true> pp{e->csc_src, (const int32_t *)e->csc_ed, e->snap, (int32_t *)e->vd,
                     e->cbits, zero_cap};
    k_pull<PullPol<true>><<<grid, kNT, 0, cs>>>(pp, dsrc, cf, cc, e->slab_a0, e->slab_fix,
                                                e->slab_fix_n, e->cnt);
    k_pull_fixup<PullPol<true>><<<2 * e->num_sms, kNT, 0, cs>>>(
        pp, dsrc, cf, cc, e->slab_a0, e->slab_fix, e->slab_fix_n, e->cnt);
  } else {
    PushPol<false> pol{e->csr_dst, nullptr, e->q_vals, (int32_t *)e->vd, e->cbits,
                       zero_cap};
    k_push<decltype(pol)><<<pgrid, kNT, 0, cs>>>(pol, qsrc, e->cnt);
    PullPol<false> pp{e->csc_src, nullptr, e->snap, (int32_t *)e->vd, e->cbits, zero_cap};
    k_pull<PullPol<false>><<<grid, kNT, 0, cs>>>(pp, dsrc, cf, cc, e->slab_a0, e->slab_fix,
                                                 e->slab_fix_n, e->cnt);
    k_pull_fixup<PullPol<false>><<<2 * e->num_sms, kNT, 0, cs>>>(
        pp, dsrc, cf, cc, e->slab_a0, e->slab_fix, e->slab_fix_n, e->cnt);
  }
  CUDA_TRY(cudaGetLastError());
  gas::prof_end(e, cs);
  return compaction(e, cs, c, h, 1);
}

gas_status_t ensure_fast_buffers(gas_engine *e) {
  if (e->q_ids) return GAS_OK;
  const size_t V = (size_t)e->nV, nW = (V + 31) / 32;
  const size_t nqb = (nW + kQWordsPerBlock - 1) / kQWordsPerBlock;
  CUDA_TRY(cudaMalloc(&e->q_ids, (V ? V : 1) * 4));
  CUDA_TRY(cudaMalloc(&e->q_vals, (V ? V : 1) * 4));
  CUDA_TRY(cudaMalloc(&e->q_end, (V ? V : 1) * 4));
  CUDA_TRY(cudaMalloc(&e->q_delta, (V ? V : 1) * 4));
  CUDA_TRY(cudaMalloc(&e->snap, (V ? V : 1) * 4));
  CUDA_TRY(cudaMalloc(&e->cbits, (nW ? nW : 1) * 4));
  // block totals, then the blocks' per-warp totals
  CUDA_TRY(cudaMalloc(&e->qpart, (nqb ? nqb : 1) * (1 + kQWarpsPerBlock) * sizeof(int4)));
  CUDA_TRY(cudaMemset(e->cbits, 0, (nW ? nW : 1) * 4));
  return GAS_OK;
}

}  // namespace

namespace gas {

// WHILE graph with a captured prologue before the loop node.
static gas_status_t build_fast_graph(gas_engine *e, FastCtx *ctx,
                                     cudaGraphExec_t *out) {
  cudaGraph_t g = nullptr;
  cudaStream_t cs = nullptr;
  gas_status_t st = GAS_OK;
  CUDA_TRY(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle h;
  cudaError_t ce = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  std::vector<cudaGraphNode_t> deps;
  if (ce == cudaSuccess)
    ce = cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (ce != cudaSuccess) {
    if (cs) cudaStreamDestroy(cs);
    cudaGraphDestroy(g);
    return fail(GAS_ERR_CUDA, "fast graph setup: %s", cudaGetErrorString(ce));
  }
  e->capturing = true;
  e->in_graph = true;
  st = prologue(e, cs, h, ctx);
  if (st == GAS_OK) {
    cudaStreamCaptureStatus cst;
    const cudaGraphNode_t *d = nullptr;
    size_t nd = 0;
    ce = cudaStreamGetCaptureInfo(cs, &cst, nullptr, nullptr, &d, nullptr, &nd);
    if (ce == cudaSuccess) deps.assign(d, d + nd);
    else st = fail(GAS_ERR_CUDA, "capture info: %s", cudaGetErrorString(ce));
  }
  e->capturing = false;
  e->in_graph = false;
  cudaGraph_t cap = nullptr;
  ce = cudaStreamEndCapture(cs, &cap);
  if (st == GAS_OK && ce != cudaSuccess)
    st = fail(GAS_ERR_CUDA, "end capture: %s", cudaGetErrorString(ce));
  if (st == GAS_OK) {
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    ce = cudaGraphAddNode(&node, g, deps.data(), nullptr, deps.size(), &p);
    if (ce != cudaSuccess) {
      st = fail(GAS_ERR_CUDA, "add while node: %s", cudaGetErrorString(ce));
    } else {
      cudaGraph_t bodyg = p.conditional.phGraph_out[0];
      ce = cudaStreamBeginCaptureToGraph(cs, bodyg, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeRelaxed);
      if (ce != cudaSuccess) {
        st = fail(GAS_ERR_CUDA, "body capture: %s", cudaGetErrorString(ce));
      } else {
        e->capturing = true;
        e->in_graph = true;
        st = body(e, cs, h, ctx);
        e->capturing = false;
        e->in_graph = false;
        cudaGraph_t bc = nullptr;
        ce = cudaStreamEndCapture(cs, &bc);
        if (st == GAS_OK && ce != cudaSuccess)
          st = fail(GAS_ERR_CUDA, "end body capture: %s", cudaGetErrorString(ce));
      }
    }
  }
  if (st == GAS_OK) {
    ce = cudaGraphInstantiate(out, g, 0);
    if (ce != cudaSuccess) st = fail(GAS_ERR_CUDA, "instantiate: %s", cudaGetErrorString(ce));
  }
  cudaStreamDestroy(cs);
  cudaGraphDestroy(g);
  return st;
}

gas_status_t run_fast(gas_engine *e, gas_schedule_t schedule,
                      int32_t max_iterations, gas_run_stats *stats,
                      void *stream) {
  if (e->prog == GAS_PROG_PAGERANK)  // not monotone: the generic kernels
    return gas_engine_run_schedule(e, GAS_SCHED_GENERIC, max_iterations, stats, stream);
  // BFS: push or the bottom-up pull per level; AUTO and LEARNED both take
  // the direction rule below (the schedule head's features do not tell BFS
  // from CC, whose pull costs far more)
  if (e->prog == GAS_PROG_BFS && schedule == GAS_SCHED_LEARNED) schedule = GAS_SCHED_AUTO;
  if (schedule == GAS_SCHED_LEARNED && !e->sched_model)
    return fail(GAS_ERR_STATE, "LEARNED schedule without a schedule model");
  if (bfs_small_eligible(e, schedule))
    return run_bfs_small(e, schedule, max_iterations, stats, stream);
  GAS_TRY(ensure_fast_buffers(e));
  FastCtx ctx;
  ctx.nW = (e->nV + 31) / 32;
  ctx.n_qblocks = (ctx.nW + kQWordsPerBlock - 1) / kQWordsPerBlock;
  if (ctx.n_qblocks < 1) ctx.n_qblocks = 1;
  {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pull<PullPol<true>>, kNT, 0);
    ctx.slab_grid = e->num_sms * (per_sm > 0 ? per_sm : 1);
    per_sm = 0;
    if (e->prog == GAS_PROG_BFS)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bfs_push, kNT, 0);
    else if (e->prog == GAS_PROG_SSSP)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_push<PushPol<true>>, kNT, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_push<PushPol<false>>, kNT, 0);
    ctx.push_grid = e->num_sms * (per_sm > 0 ? per_sm : 1);
    // the pushes use no shared memory: all of the SM's L1/shared storage
    // as L1 for the state gathers
    cudaFuncSetAttribute(k_bfs_push, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    cudaFuncSetAttribute(k_push<PushPol<true>>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         0);
    cudaFuncSetAttribute(k_push<PushPol<false>>,
                         cudaFuncAttributePreferredSharedMemoryCarveout, 0);
  }
  ctx.seeded = e->prog != GAS_PROG_BFS && e->active_full && !e->counts_dirty &&
               e->n_active == e->nV;
  const int slot = kGraphFast0 + (ctx.seeded ? 1 : 0);
  const bool host_loop = host_loop_for(e);
  if (!host_loop && !e->graphs[slot]) GAS_TRY(build_fast_graph(e, &ctx, &e->graphs[slot]));
  const int forced = schedule == GAS_SCHED_PUSH ? 1 : schedule == GAS_SCHED_PULL ? 2
                     : schedule == GAS_SCHED_LEARNED ? 3 : 0;
  // BFS pulls while the frontier's out-edges exceed 1/16 of the edges
  const int pull_div = e->prog == GAS_PROG_BFS ? kBfsPullDiv : e->pull_div;
  k_fast_reset<<<1, 1, 0, S(stream)>>>(e->cnt, max_iterations, forced, pull_div);
  cudaError_t ce = cudaGetLastError();
  if (host_loop) {
    if (ce == cudaSuccess) {
      e->capturing = true;
      e->in_graph = false;
      gas_status_t pst = prologue(e, S(stream), 0, &ctx);
      e->capturing = false;
      if (pst != GAS_OK) return pst;
      if (ce == cudaSuccess) GAS_TRY(run_host_loop(e, body, &ctx, stream));
    }
  } else if (ce == cudaSuccess) {
    ce = cudaGraphLaunch(e->graphs[slot], S(stream));
  }
  if (ce == cudaSuccess) {
    k_fast_finish<<<1, 1, 0, S(stream)>>>(e->cnt);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(S(stream));
  if (ce != cudaSuccess) return fail(GAS_ERR_CUDA, "fast run: %s", cudaGetErrorString(ce));
  gas_counters c;
  GAS_TRY(engine_sync_counts(e, stream));
  c = *e->h_cnt;
  if (stats) {
    stats->iterations = c.iteration;
    stats->push_iters = c.n_push;
    stats->pull_iters = c.n_pull;
    // prologue (snapshot fill; gather/apply, fixup, commit | bfs apply;
    // seed; partition of the dense pull; 3 compaction, the last two also
    // the loop control and the next push's partition) + per iteration
    // (push, pull, pull fixup | bfs push, bfs pull; 3 compaction) + reset
    // + finish
    const int pro = e->prog == GAS_PROG_BFS ? 6 : (ctx.seeded ? 6 : 10);
    const int per = e->prog == GAS_PROG_BFS ? 5 : 6;
    const int loop_iters = ctx.seeded ? c.iteration : (c.iteration > 0 ? c.iteration - 1 : 0);
    stats->kernel_launches = pro + per * loop_iters + 2;
    stats->graph_launches = host_loop ? 0 : 1;
  }
  e->level = c.iteration;
  e->active_full = false;
  return loop_status(e, c, stream);
}

}  // namespace gas

// ---------------------------------------------------------------------------
// traces and the schedule model
// ---------------------------------------------------------------------------
namespace {
void drop_fast_graphs(gas_engine *e) {
  for (int i = kGraphFast0; i < kGraphSlots; ++i) {
    if (e->graphs[i]) cudaGraphExecDestroy(e->graphs[i]);
    e->graphs[i] = nullptr;
  }
}
}  // namespace

extern "C" gas_status_t gas_engine_set_trace(gas_engine *e, int32_t on) {
  if (!e) return gas::fail(GAS_ERR_INVALID, "null engine");
  if ((on != 0) != e->trace_on) drop_fast_graphs(e);  // captured with the old setting
  e->trace_on = on != 0;
  return GAS_OK;
}

extern "C" gas_status_t gas_engine_get_trace(gas_engine *e, gas_trace_record *out,
                                             int32_t cap, int32_t *n) {
  if (!e || !out || !n || cap < 0) return gas::fail(GAS_ERR_INVALID, "bad arguments");
  if (!e->has_graph) return gas::fail(GAS_ERR_STATE, "no graph");
  gas_counters c;
  GAS_TRY(gas_engine_read_counters(e, &c, nullptr));
  int32_t k = c.iteration < GAS_TRACE_CAP ? c.iteration : GAS_TRACE_CAP;
  if (k > cap) k = cap;
  if (k > 0)
    CUDA_TRY(cudaMemcpy(out, e->trace, sizeof(gas_trace_record) * (size_t)k,
                        cudaMemcpyDeviceToHost));
  *n = k;
  return GAS_OK;
}

extern "C" gas_status_t gas_engine_set_schedule_model(gas_engine *e, const gas_mlp *m) {
  if (!e) return gas::fail(GAS_ERR_INVALID, "null engine");
  if (m && (gaslearn::mlp_inputs(m) != GAS_SCHED_FEATURES || gaslearn::mlp_outputs(m) != 2))
    return gas::fail(GAS_ERR_INVALID, "schedule model must be %d -> 2", GAS_SCHED_FEATURES);
  const void *w = m ? gaslearn::mlp_bf16(m) : nullptr;
  if (w != e->sched_model) drop_fast_graphs(e);
  e->sched_model = w;
  return GAS_OK;
}

extern "C" void gas_schedule_features(const gas_trace_record *rec, int32_t nV, int64_t nE,
                                      int32_t weighted, float *out) {
  if (!rec || !out) return;
  gasfeat::schedule_features(rec->n_queue, rec->n_edges_out, rec->hist, rec->iteration, nV,
                             nE, weighted, out);
}
