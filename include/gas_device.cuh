// gas_device.cuh -- device code shared by libgas and include/gpugas.h.
//
// The load-balanced gather of the reference (gpugas.h:714-786: a scan of
// in-degrees, MergePathPartitions, kGatherMap writing E-sized temporaries,
// then ReduceByKey) becomes one tiled kernel here:
//
//   * merge path over "segment ends + edges": the active list with its
//     exclusive in-degree scan is merged with the edge index range, and every
//     CTA tile takes kTile merge items, so hubs and zero-degree vertices are
//     balanced alike;
//   * the tile's row offsets are staged in shared memory, its edges are read
//     cooperatively (consecutive threads -> consecutive CSC entries) and
//     mapped with Program::gatherMap into shared memory;
//   * each thread folds kVT items with Program::gatherReduce, a warp-shuffle
//     segmented scan joins segments split across threads, and the segment's
//     epilogue runs Program::apply (apply fused into the gather);
//   * segments split across tiles leave a per-tile carry, folded by
//     k_fixup_tiles in tile order (deterministic).
//
// The same walk, without the reduction, drives the scatter-side expansion
// (frontier activation, gpugas.h:942-1013 + scatter_if_mgpu.h:130-157).
//
// Program::gatherZero is treated as the identity of Program::gatherReduce,
// as the reference's ReduceByKey does (gpugas.h:766-776).
#ifndef GAS_DEVICE_CUH_
#define GAS_DEVICE_CUH_

#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>
#include <string.h>

#include "gas.h"

namespace gasdev {

constexpr int kNT = 256;  // threads per CTA of the tiled kernels

// Merge items per thread for a reduction value of a given size (keeps the
// tile's shared memory under 48 KB).
template <int kValBytes>
struct TileShape {
  static constexpr int kVT = kValBytes <= 8 ? 8 : (kValBytes <= 16 ? 4 : 2);
  static constexpr int kTile = kNT * kVT;
};

// Shuffle of any trivially copyable value, in 32-bit pieces.
template <class T>
__device__ __forceinline__ T shfl_up_any(const T &v, int delta) {
  constexpr int W = (int)((sizeof(T) + 3) / 4);
  int w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int k = 0; k < W; ++k) w[k] = __shfl_up_sync(0xffffffffu, w[k], delta);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

template <class T>
__device__ __forceinline__ T shfl_down_any(const T &v, int delta) {
  constexpr int W = (int)((sizeof(T) + 3) / 4);
  int w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int k = 0; k < W; ++k)
    w[k] = __shfl_down_sync(0xffffffffu, w[k], delta);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

// Merge path over (segment ends, edge indices): the number of segment ends
// among the first `diag` merge items.  ends[i] = end of segment i (exclusive
// edge bound); an end is ordered before the edge with the same index.
__device__ __forceinline__ int merge_path(const int32_t *__restrict__ ends,
                                          int n_seg, int n_edge, int diag) {
  int lo = diag - n_edge > 0 ? diag - n_edge : 0;
  int hi = diag < n_seg ? diag : n_seg;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(ends + mid) <= diag - 1 - mid)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

template <class Val, int kTile>
struct TileSmem {
  int32_t end[kTile + 1];    // tile-local end of each touched segment
  int32_t delta[kTile + 1];  // array position - edge index, per segment
  int32_t vert[kTile + 1];   // vertex of each touched segment
  uint16_t seg[kTile];       // local segment of each tile edge
  Val val[kTile];            // mapped value of each tile edge
  Val wv[kNT / 32];
  int32_t wf[kNT / 32];
  int32_t bounds[4];
};

// Where a frontier's segments come from.
//   dense:  segment a = vertex a, edges off[a]..off[a+1]
//   listed: segment a = vertex act[a], edge index range scan[a]..scan[a+1],
//           array positions off[act[a]] + (edge - scan[a])
struct SegSource {
  const int32_t *act;
  const int32_t *scan;
  const int32_t *off;
  int32_t n_seg;             // sizes, unless read from device counters:
  int32_t n_edge;
  const int32_t *n_seg_p;    // device address of the segment count, or null
  const int32_t *n_edge_p;   // device address of the edge count, or null
  const int32_t *part;       // part[t] = segment ends before tile t (from
                             // k_partition), or null to search in the tile
};

__device__ __forceinline__ void seg_sizes(const SegSource &s, int &nA, int &E) {
  nA = s.n_seg_p ? *s.n_seg_p : s.n_seg;
  E = s.n_edge_p ? *s.n_edge_p : s.n_edge;
}

// Tile boundaries of a segment source, one thread per boundary, so that the
// binary searches of all tiles overlap instead of serialising in each CTA
// (moderngpu's MergePathPartitions step, gpugas.h:737-739).
template <int kTile, bool kDense>
__global__ void __launch_bounds__(256) k_partition(SegSource src, int32_t *part) {
  int nA, E;
  seg_sizes(src, nA, E);
  const int64_t M = (int64_t)nA + E;
  const int ntiles = (int)((M + kTile - 1) / kTile);
  const int32_t *ends = kDense ? src.off + 1 : src.scan + 1;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t <= ntiles;
       t += gridDim.x * blockDim.x) {
    const int64_t d = (int64_t)t * kTile < M ? (int64_t)t * kTile : M;
    part[t] = merge_path(ends, nA, E, (int)d);
  }
}

// One pass over all tiles of a segment source.  Pol provides
//   typedef Val; zero(); reduce(a, b); map(seg, vertex, pos) -> Val;
//   emit(seg, vertex, Val)                     (kReduce)
//   visit(seg, vertex, pos)                    (!kReduce)
// Tiles whose first segment started in an earlier tile and ends here leave
// tile_first[t] / tile_a0[t] for k_fixup_tiles; every tile leaves
// tile_carry[t], the fold of its trailing open segment.
template <class Pol, bool kDense, bool kReduce>
__device__ __forceinline__ void tile_loop(Pol &pol, const SegSource src,
                                          typename Pol::Val *tile_first,
                                          typename Pol::Val *tile_carry,
                                          int32_t *tile_a0) {
  using Val = typename Pol::Val;
  constexpr int kVT = TileShape<sizeof(Val)>::kVT;
  constexpr int kTile = TileShape<sizeof(Val)>::kTile;
  __shared__ TileSmem<Val, kTile> sm;

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  int nA, E;
  seg_sizes(src, nA, E);
  const int32_t *ends = kDense ? src.off + 1 : src.scan + 1;
  const int64_t M = (int64_t)nA + E;
  const int ntiles = (int)((M + kTile - 1) / kTile);

  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int d0 = t * kTile;
    const int d1 = (int)((int64_t)d0 + kTile < M ? (int64_t)d0 + kTile : M);
    if (src.part) {
      if (tid < 2) sm.bounds[tid] = __ldg(src.part + t + tid);
    } else {
      if (tid == 0) sm.bounds[0] = merge_path(ends, nA, E, d0);
      if (tid == 32) sm.bounds[1] = merge_path(ends, nA, E, d1);
    }
    __syncthreads();
    const int a0 = sm.bounds[0];
    const int a1 = sm.bounds[1];
    const int b0 = d0 - a0;
    const int b1 = d1 - a1;
    const int nX = a1 - a0;                  // segment ends inside the tile
    const int nS = nX + (a1 < nA ? 1 : 0);   // segments touched by the tile
    for (int i = tid; i < nS; i += kNT) {
      const int a = a0 + i;
      int v, beg, end, delta;
      if (kDense) {
        v = a;
        beg = __ldg(src.off + a);
        end = __ldg(src.off + a + 1);
        delta = 0;
      } else {
        v = __ldg(src.act + a);
        beg = __ldg(src.scan + a);
        end = __ldg(src.scan + a + 1);
        delta = __ldg(src.off + v) - beg;
      }
      sm.end[i] = end - b0;
      sm.delta[i] = delta;
      sm.vert[i] = v;
      if (i == 0) sm.bounds[2] = (beg < b0) ? 1 : 0;  // segment a0 open-start
    }
    if (nS == 0 && tid == 0) sm.bounds[2] = 0;
    __syncthreads();

    const int nItems = d1 - d0;
    const int nY = b1 - b0;
    const int dl = tid * kVT < nItems ? tid * kVT : nItems;
    const int dend = dl + kVT < nItems ? dl + kVT : nItems;
    int la;
    {
      int lo = dl - nY > 0 ? dl - nY : 0;
      int hi = dl < nX ? dl : nX;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (sm.end[mid] <= dl - 1 - mid)
          lo = mid + 1;
        else
          hi = mid;
      }
      la = lo;
    }
    const int lb = dl - la;
    {
      int a = la, b = lb;
      for (int k = dl; k < dend; ++k) {
        if (a < nX && sm.end[a] <= b) {
          ++a;
        } else {
          sm.seg[b] = (uint16_t)a;
          ++b;
        }
      }
    }
    __syncthreads();

    // Edges of the tile, consecutive threads on consecutive edges; fully
    // unrolled so that the kVT independent load chains of a thread overlap.
#pragma unroll
    for (int k = 0; k < kVT; ++k) {
      const int j = tid + k * kNT;
      if (j < nY) {
        const int ls = sm.seg[j];
        const int pos = b0 + j + sm.delta[ls];
        if constexpr (kReduce)
          sm.val[j] = pol.map(a0 + ls, sm.vert[ls], pos);
        else
          pol.visit(a0 + ls, sm.vert[ls], pos);
      }
    }
    __syncthreads();
    if constexpr (!kReduce) continue;

    Val acc = pol.zero();
    Val lead = pol.zero();
    int first = -1;
    {
      int a = la, b = lb;
      for (int k = dl; k < dend; ++k) {
        if (a < nX && sm.end[a] <= b) {
          if (first < 0) {
            first = a;
            lead = acc;
          } else {
            pol.emit(a0 + a, sm.vert[a], acc);
          }
          acc = pol.zero();
          ++a;
        } else {
          acc = pol.reduce(acc, sm.val[b]);
          ++b;
        }
      }
    }

    // CTA-wide exclusive segmented scan of (has_end, tail fold).
    Val incl = acc;
    int fi = first >= 0 ? 1 : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const Val ov = shfl_up_any(incl, d);
      const int of = __shfl_up_sync(0xffffffffu, fi, d);
      if (lane >= d) {
        if (!fi) incl = pol.reduce(ov, incl);
        fi |= of;
      }
    }
    if (lane == 31) {
      sm.wv[warp] = incl;
      sm.wf[warp] = fi;
    }
    __syncthreads();
    Val wp = pol.zero();
    for (int w = 0; w < warp; ++w) {
      if (sm.wf[w])
        wp = sm.wv[w];
      else
        wp = pol.reduce(wp, sm.wv[w]);
    }
    Val ex = shfl_up_any(incl, 1);
    int exf = __shfl_up_sync(0xffffffffu, fi, 1);
    if (lane == 0) {
      ex = pol.zero();
      exf = 0;
    }
    const Val carry = exf ? ex : pol.reduce(wp, ex);
    if (first >= 0) {
      const Val g = pol.reduce(carry, lead);
      if (first == 0 && sm.bounds[2]) {
        tile_first[t] = g;
      } else {
        pol.emit(a0 + first, sm.vert[first], g);
      }
    }
    if (tid == kNT - 1) tile_carry[t] = fi ? incl : pol.reduce(wp, incl);
    if (tid == 0) tile_a0[t] = (sm.bounds[2] && nX > 0) ? a0 : -1;
    __syncthreads();
  }
}

// Completes the segments that span tiles: fold tile_carry over the tiles the
// segment started in, then tile_first of the tile that ends it.  One warp
// per tile; the fold order is fixed, so results are deterministic.
template <class Pol, bool kDense>
__device__ __forceinline__ void fixup_loop(Pol &pol, const SegSource src,
                                           const typename Pol::Val *tile_first,
                                           const typename Pol::Val *tile_carry,
                                           const int32_t *tile_a0) {
  using Val = typename Pol::Val;
  constexpr int kTile = TileShape<sizeof(Val)>::kTile;
  int nA, E;
  seg_sizes(src, nA, E);
  const int64_t M = (int64_t)nA + E;
  const int ntiles = (int)((M + kTile - 1) / kTile);
  const int lane = threadIdx.x & 31;
  const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int t = gwarp; t < ntiles; t += nwarps) {
    const int a0 = tile_a0[t];
    if (a0 < 0) continue;
    const int beg = kDense ? __ldg(src.off + a0) : __ldg(src.scan + a0);
    const int s_first = (int)(((int64_t)beg + a0) / kTile);
    Val acc = pol.zero();
    for (int s = s_first; s < t; s += 32) {
      Val x = (s + lane < t) ? tile_carry[s + lane] : pol.zero();
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const Val y = shfl_down_any(x, d);
        if (lane + d < 32) x = pol.reduce(x, y);
      }
      acc = pol.reduce(acc, x);  // lane 0 holds the chunk's ordered fold
    }
    if (lane == 0) {
      const Val g = pol.reduce(acc, tile_first[t]);
      const int v = kDense ? a0 : __ldg(src.act + a0);
      pol.emit(a0, v, g);
    }
  }
}

// ---------------------------------------------------------------------------
// Policies for a user Program (the gather step of GASEngineGPU).
// ---------------------------------------------------------------------------

template <class P>
struct GenericGather {
  typedef typename P::VertexData VD;
  typedef typename P::EdgeData ED;
  typedef typename P::GatherResult Val;
  const int32_t *csc_src;
  const ED *csc_ed;
  const VD *vd;
  VD *slot;      // fused: new vertex data per active slot
  uint8_t *ret;  // fused: apply() result per active slot
  Val *gres;     // gather-only: gather result per active slot
  int fuse;

  __device__ __forceinline__ Val zero() const { return P::gatherZero; }
  __device__ __forceinline__ Val reduce(const Val &a, const Val &b) const {
    return P::gatherReduce(a, b);
  }
  __device__ __forceinline__ Val map(int, int dst, int pos) const {
    const int s = __ldg(csc_src + pos);
    return P::gatherMap(vd + dst, vd + s, csc_ed + pos);
  }
  __device__ __forceinline__ void emit(int a, int v, const Val &g) const {
    if (fuse) {
      VD tmp = vd[v];
      const bool r = P::apply(&tmp, g);
      slot[a] = tmp;
      ret[a] = r ? 1 : 0;
    } else {
      gres[a] = g;
    }
  }
};

template <class P>
__global__ void __launch_bounds__(kNT)
    k_gather_tiles(GenericGather<P> pol, SegSource src,
                   typename P::GatherResult *tile_first,
                   typename P::GatherResult *tile_carry, int32_t *tile_a0) {
  tile_loop<GenericGather<P>, false, true>(pol, src, tile_first, tile_carry,
                                           tile_a0);
}

template <class P>
__global__ void __launch_bounds__(kNT)
    k_gather_fixup(GenericGather<P> pol, SegSource src,
                   const typename P::GatherResult *tile_first,
                   const typename P::GatherResult *tile_carry,
                   const int32_t *tile_a0) {
  fixup_loop<GenericGather<P>, false>(pol, src, tile_first, tile_carry, tile_a0);
}

// A listed segment source whose sizes are the frontier counters.
__host__ __device__ inline SegSource frontier_source(const int32_t *act,
                                                     const int32_t *scan,
                                                     const int32_t *off,
                                                     const int32_t *n_seg_p,
                                                     const int32_t *n_edge_p,
                                                     const int32_t *part) {
  SegSource s;
  s.act = act;
  s.scan = scan;
  s.off = off;
  s.n_seg = 0;
  s.n_edge = 0;
  s.n_seg_p = n_seg_p;
  s.n_edge_p = n_edge_p;
  s.part = part;
  return s;
}

__host__ __device__ inline SegSource dense_source(const int32_t *off, int nV,
                                                  int nE, const int32_t *part) {
  SegSource s;
  s.act = nullptr;
  s.scan = nullptr;
  s.off = off;
  s.n_seg = nV;
  s.n_edge = nE;
  s.n_seg_p = nullptr;
  s.n_edge_p = nullptr;
  s.part = part;
  return s;
}

// Parity mode: one thread per active vertex folds its in-edges sequentially
// in CSC order, exactly like refgas.h:143-160.
template <class P>
__global__ void __launch_bounds__(kNT)
    k_gather_ordered(GenericGather<P> pol, const int32_t *act,
                     const int32_t *csc_off, const gas_counters *cnt) {
  const int n = cnt->n_active;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const int v = act[i];
    typename P::GatherResult acc = P::gatherZero;
    const int e1 = csc_off[v + 1];
    for (int e = csc_off[v]; e < e1; ++e)
      acc = P::gatherReduce(acc, pol.map(i, v, e));
    pol.emit(i, v, acc);
  }
}

// apply() without a preceding gather this iteration (BFS: gather(false)):
// the vertex is updated in place, since no gather reads it concurrently.
template <class P>
__global__ void __launch_bounds__(kNT)
    k_apply_only(const int32_t *act, const gas_counters *cnt,
                 typename P::VertexData *vd,
                 const typename P::GatherResult *gres, uint8_t *ret) {
  const int n = cnt->n_active;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const typename P::GatherResult g = gres ? gres[i] : P::gatherZero;
    ret[i] = P::apply(vd + act[i], g) ? 1 : 0;
  }
}

// Program::scatter on the GPU (refgas.h:175-196): for every active slot
// whose apply returned true, every out-edge in CSR order gets
// scatter(src, dst, edge) with the vertex data apply left.  One warp per
// active vertex; every edge belongs to one source, so no two threads touch
// the same edge record.  The CSR copy of the edge data is updated and
// mirrored into the CSC copy that the next gather reads.  Programs opt in
// with `static const bool runScatter = true;` (the reference GPU engine
// never calls scatter, gpugas.h:942, and the reference apps' scatter is
// empty).
template <class P, class = void>
struct RunsScatter { static constexpr bool value = false; };
template <class P>
struct RunsScatter<P, decltype((void)P::runScatter, void())> {
  static constexpr bool value = P::runScatter;
};

template <class P>
__global__ void __launch_bounds__(kNT)
    k_scatter_user(const int32_t *act, const gas_counters *cnt, const uint8_t *ret,
                   const int32_t *csr_off, const int32_t *csr_dst,
                   const typename P::VertexData *vd, typename P::EdgeData *csr_ed,
                   typename P::EdgeData *csc_ed, const int32_t *csr_to_csc) {
  typedef typename P::EdgeData ED;
  const int n = cnt->n_active;
  const int lane = threadIdx.x & 31;
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < n; i += nwarps) {
    if (!ret[i]) continue;
    const int sv = act[i];
    const int e1 = csr_off[sv + 1];
    for (int pos = csr_off[sv] + lane; pos < e1; pos += 32) {
      const int dv = csr_dst[pos];
      if (csr_ed) {
        ED ed = csr_ed[pos];
        P::scatter(vd + sv, vd + dv, &ed);
        csr_ed[pos] = ed;
        csc_ed[csr_to_csc[pos]] = ed;
      } else {
        ED ed{};
        P::scatter(vd + sv, vd + dv, &ed);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Warp-slab segmented passes (dense CSC pulls, PageRank, frontier pushes).
//
// The segments here are never empty (vertices without edges are handled
// apart), so a 32-edge slab contains at most 31 segment boundaries.  Each
// warp streams a contiguous chunk of kSlabChunk edges, 32 at a time: one
// coalesced load of the next 32 segment ends gives, through
// __reduce_or_sync + popc, the segment of every lane's edge; a 5-step
// shuffle segmented scan folds the slab; the last lane of each segment that
// ends in the slab emits it; a segment that runs past the slab is carried in
// registers.  No shared memory and no CTA barriers.  Segments split across
// chunks leave a per-chunk carry folded by slab_fixup_loop in chunk order.
// ---------------------------------------------------------------------------
constexpr int kSlabChunkLog2 = 9;
constexpr int kSlabChunk = 1 << kSlabChunkLog2;  // edges per warp chunk
constexpr int kSlabChunkMinLog2 = 6;             // the smallest chunk: one slab pair

struct SlabSource {
  const int32_t *ends;     // [n_seg] exclusive end of segment k in the virtual
                           // edge range, strictly increasing
  const int32_t *vid;      // [n_seg] vertex of segment k (null: k itself)
  const int32_t *delta;    // [n_seg] array position - virtual index (null: 0)
  int32_t n_seg;
  int32_t n_edge;
  const int32_t *n_seg_p;  // device counters, or null
  const int32_t *n_edge_p;
  const int32_t *part;     // [n_chunks] segment holding each chunk's first edge
  const int32_t *chunk_log2_p;  // device log2 of the chunk size, or null
                                // (kSlabChunk)
};

__device__ __forceinline__ int slab_chunk_log2(const SlabSource &s) {
  return s.chunk_log2_p ? *s.chunk_log2_p : kSlabChunkLog2;
}

__device__ __forceinline__ void slab_sizes(const SlabSource &s, int &nS, int &E) {
  nS = s.n_seg_p ? *s.n_seg_p : s.n_seg;
  E = s.n_edge_p ? *s.n_edge_p : s.n_edge;
}

// Segment of each chunk's first edge: the first k with ends[k] > e.
template <int kChunk = kSlabChunk>
__global__ void __launch_bounds__(256) k_slab_partition(SlabSource src, int32_t *part) {
  int nS, E;
  slab_sizes(src, nS, E);
  const int nchunks = (E + kChunk - 1) / kChunk;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nchunks;
       c += gridDim.x * blockDim.x) {
    const int e = c * kChunk;
    int lo = 0, hi = nS;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(src.ends + mid) <= e)
        lo = mid + 1;
      else
        hi = mid;
    }
    part[c] = lo;
  }
}

template <class T>
__device__ __forceinline__ T shfl_any(const T &v, int src_lane) {
  constexpr int W = (int)((sizeof(T) + 3) / 4);
  int w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int k = 0; k < W; ++k) w[k] = __shfl_sync(0xffffffffu, w[k], src_lane);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

// Policy traits of the slab passes (defaults: vertex ids loaded for map /
// visit, ordered shuffle scan).  A policy may declare
//   static constexpr bool kMapNeedsVertex = false;  // map/visit ignore it
//   static constexpr bool kIntMin = true;           // Val is int, reduce is min
template <class Pol, class = void>
struct NeedsVertex { static constexpr bool value = true; };
template <class Pol>
struct NeedsVertex<Pol, decltype((void)Pol::kMapNeedsVertex, void())> {
  static constexpr bool value = Pol::kMapNeedsVertex;
};
template <class Pol, class = void>
struct IntMin { static constexpr bool value = false; };
template <class Pol>
struct IntMin<Pol, decltype((void)Pol::kIntMin, void())> {
  static constexpr bool value = Pol::kIntMin;
};

// Visit policies may split visit() into probe() (the loads: returns a
// Probe) and commit(Probe) (the updates), so that slab_loop issues the loads
// of both slabs in flight before either slab's updates.
template <class Pol, class = void>
struct TwoPhase { static constexpr bool value = false; };
template <class Pol>
struct TwoPhase<Pol, decltype((void)sizeof(typename Pol::Probe), void())> {
  static constexpr bool value = true;
};

// Segment of every lane's edge in one 32-edge slab starting at s.
struct SlabRows {
  int row;
  bool valid;
  bool ends_here;  // this lane holds the last edge of its segment
  unsigned mask;   // bit l: lane l starts a new segment (l >= 1)
  int r_next;      // segment of the next slab's first edge
  bool end_last;   // the slab's last edge ends its segment
};

__device__ __forceinline__ SlabRows slab_rows(const SlabSource &src, int nS, int s,
                                              int e1, int r, int &wbase, int &b,
                                              int lane) {
  constexpr unsigned FULL = 0xffffffffu;
  int shift = r - wbase;
  const int b31 = __shfl_sync(FULL, b, 31);
  if (shift > 0 && b31 <= s + 31) {  // window used up: reload at r
    wbase = r;
    shift = 0;
    b = (r + lane < nS) ? __ldg(src.ends + r + lane) : INT_MAX;
  }
  SlabRows o;
  const int last = e1 - s - 1 < 31 ? e1 - s - 1 : 31;
  const int end_r = __shfl_sync(FULL, b, shift);  // end of segment r
  if (end_r > s + last) {
    // the whole slab lies in segment r (most slabs of high-degree rows)
    o.mask = 0u;
    o.row = r;
    o.valid = s + lane < e1;
    o.ends_here = o.valid && end_r == s + lane + 1;
    o.end_last = end_r == s + last + 1;
    o.r_next = o.end_last ? r + 1 : r;
    return o;
  }
  const int k = b - s;
  const unsigned bit = (lane >= shift && k >= 1 && k <= 31) ? (1u << k) : 0u;
  o.mask = __reduce_or_sync(FULL, bit);
  o.row = r + __popc(o.mask & ((2u << lane) - 1u));
  const int e = s + lane;
  o.valid = e < e1;
  const int row_end = __shfl_sync(FULL, b, o.row - wbase);
  o.ends_here = o.valid && row_end == e + 1;
  const int row_last = __shfl_sync(FULL, o.row, last);
  o.end_last = __shfl_sync(FULL, (int)o.ends_here, last) != 0;
  o.r_next = o.end_last ? row_last + 1 : row_last;
  return o;
}

// Inclusive fold of each segment's lanes (segment heads: lane 0 and the
// bits of mask); the last lane of a segment holds the segment's fold.
template <class Pol>
__device__ __forceinline__ typename Pol::Val slab_fold(const Pol &pol,
                                                       typename Pol::Val val,
                                                       unsigned mask, int lane) {
  const unsigned heads = mask | 1u;
  const int seg_start = 31 - __clz(heads & ((2u << lane) - 1u));
  if constexpr (IntMin<Pol>::value) {
    const unsigned above = heads & ~((2u << lane) - 1u);
    const int seg_end = above ? __ffs(above) - 2 : 31;
    const unsigned hi = seg_end == 31 ? 0xffffffffu : ((2u << seg_end) - 1u);
    const unsigned group = hi & ~((1u << seg_start) - 1u);
    return __reduce_min_sync(group, val);
  } else {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const typename Pol::Val t = shfl_up_any(val, d);
      if (lane - d >= seg_start) val = pol.reduce(t, val);
    }
    return val;
  }
}

// Policies whose Val carries compensation may declare a cheaper type for
// the scan inside a slab: `typedef ... Scan;` with to_scan(Val),
// from_scan(Scan) and scan_add(Scan, Scan).  A slab is then folded in that
// type, and the carry from earlier slabs joins its first segment through
// reduce() after the scan, so sums of many slabs stay compensated.
template <class Pol, class = void>
struct PlainScan { static constexpr bool value = false; };
template <class Pol>
struct PlainScan<Pol, decltype((void)sizeof(typename Pol::Scan), void())> {
  static constexpr bool value = true;
};

template <class Pol>
__device__ __forceinline__ typename Pol::Scan slab_fold_scan(const Pol &pol,
                                                             typename Pol::Scan val,
                                                             unsigned mask, int lane) {
  const unsigned heads = mask | 1u;
  const int seg_start = 31 - __clz(heads & ((2u << lane) - 1u));
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const typename Pol::Scan t = shfl_up_any(val, d);
    if (lane - d >= seg_start) val = pol.scan_add(t, val);
  }
  return val;
}

// Pol as for tile_loop: Val, zero(), reduce(), map(seg, vertex, pos),
// emit(seg, vertex, Val) when kReduce; visit(seg, vertex, pos) otherwise.
// Two slabs are in flight per iteration so that their load chains overlap.
// Chunks whose first segment started in an earlier chunk and ends here are
// appended to fix_list (row in ch_a0[c]) for slab_fixup_loop.
template <class Pol, bool kReduce>
__device__ __forceinline__ void slab_loop(Pol &pol, const SlabSource src,
                                          typename Pol::Val *ch_first,
                                          typename Pol::Val *ch_carry,
                                          int32_t *ch_a0, int32_t *fix_list,
                                          int32_t *fix_count) {
  using Val = typename Pol::Val;
  constexpr unsigned FULL = 0xffffffffu;
  constexpr bool kVert = NeedsVertex<Pol>::value;
  int nS, E;
  slab_sizes(src, nS, E);
  const int cl = slab_chunk_log2(src);
  const int nchunks = (int)(((long long)E + (1 << cl) - 1) >> cl);
  const int lane = threadIdx.x & 31;
  const int gwarp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  for (int c = gwarp; c < nchunks; c += nwarps) {
    const int e0 = c << cl;
    const int e1 = E - e0 > (1 << cl) ? e0 + (1 << cl) : E;
    int r = __ldg(src.part + c);
    const int r_first = r;
    bool open_first = false;
    if constexpr (kReduce) open_first = (r > 0 ? __ldg(src.ends + r - 1) : 0) < e0;
    int wbase = r;
    int b = (r + lane < nS) ? __ldg(src.ends + r + lane) : INT_MAX;
    Val carry = pol.zero();
    bool have_carry = false;
    bool first_done = false;
    for (int s = e0; s < e1; s += 64) {
      const bool two = s + 32 < e1;
      const SlabRows A = slab_rows(src, nS, s, e1, r, wbase, b, lane);
      SlabRows B = A;
      if (two) B = slab_rows(src, nS, s + 32, e1, A.r_next, wbase, b, lane);
      // positions and the (independent) loads of both slabs
      const int eA = s + lane, eB = s + 32 + lane;
      int posA = eA, posB = eB, vA = A.row, vB = B.row;
      if (A.valid) {
        if (src.delta) posA += __ldg(src.delta + A.row);
        if (kVert && src.vid) vA = __ldg(src.vid + A.row);
      }
      if (two && B.valid) {
        if (src.delta) posB += __ldg(src.delta + B.row);
        if (kVert && src.vid) vB = __ldg(src.vid + B.row);
      }
      if constexpr (!kReduce) {
        if constexpr (TwoPhase<Pol>::value) {
          // both slabs' loads first, then their (fire-and-forget) updates
          const typename Pol::Probe pa = pol.probe(A.valid, A.row, vA, posA);
          const typename Pol::Probe pb = pol.probe(two && B.valid, B.row, vB, posB);
          pol.commit(pa);
          pol.commit(pb);
        } else {
          if (A.valid) pol.visit(A.row, vA, posA);
          if (two && B.valid) pol.visit(B.row, vB, posB);
        }
        r = two ? B.r_next : A.r_next;
      } else {
        Val valA = A.valid ? pol.map(A.row, vA, posA) : pol.zero();
        Val valB = (two && B.valid) ? pol.map(B.row, vB, posB) : pol.zero();
        // slab A (its first segment is row r)
        if constexpr (PlainScan<Pol>::value) {
          valA = pol.from_scan(slab_fold_scan(pol, pol.to_scan(valA), A.mask, lane));
          if (have_carry && A.row == r) valA = pol.reduce(carry, valA);
        } else {
          if (lane == 0 && have_carry) valA = pol.reduce(carry, valA);
          valA = slab_fold(pol, valA, A.mask, lane);
        }
        {
          const bool to_first = A.ends_here && open_first && A.row == r_first;
          if (A.ends_here) {
            if (to_first) {
              ch_first[c] = valA;
            } else {
              const int v = (!kVert && src.vid) ? __ldg(src.vid + A.row) : vA;
              pol.emit(A.row, v, valA);
            }
          }
          first_done = first_done || __any_sync(FULL, to_first);
          const int last = e1 - s - 1 < 31 ? e1 - s - 1 : 31;
          const Val v_last = shfl_any(valA, last);
          have_carry = !A.end_last;
          if (have_carry) carry = v_last;
        }
        if (two) {
          if constexpr (PlainScan<Pol>::value) {
            valB = pol.from_scan(slab_fold_scan(pol, pol.to_scan(valB), B.mask, lane));
            if (have_carry && B.row == A.r_next) valB = pol.reduce(carry, valB);
          } else {
            if (lane == 0 && have_carry) valB = pol.reduce(carry, valB);
            valB = slab_fold(pol, valB, B.mask, lane);
          }
          const bool to_first = B.ends_here && open_first && B.row == r_first;
          if (B.ends_here) {
            if (to_first) {
              ch_first[c] = valB;
            } else {
              const int v = (!kVert && src.vid) ? __ldg(src.vid + B.row) : vB;
              pol.emit(B.row, v, valB);
            }
          }
          first_done = first_done || __any_sync(FULL, to_first);
          const int last = e1 - s - 33 < 31 ? e1 - s - 33 : 31;
          const Val v_last = shfl_any(valB, last);
          have_carry = !B.end_last;
          if (have_carry) carry = v_last;
        }
        r = two ? B.r_next : A.r_next;
      }
    }
    if constexpr (kReduce) {
      if (lane == 0) {
        ch_carry[c] = have_carry ? carry : pol.zero();
        if (open_first && first_done) {
          ch_a0[c] = r_first;
          fix_list[atomicAdd(fix_count, 1)] = c;
        }
      }
    }
  }
}

// Completes segments split across chunks: one warp per listed chunk folds
// the carries of the chunks the segment spans, in chunk order.
template <class Pol>
__device__ __forceinline__ void slab_fixup_loop(Pol &pol, const SlabSource src,
                                                const typename Pol::Val *ch_first,
                                                const typename Pol::Val *ch_carry,
                                                const int32_t *ch_a0,
                                                const int32_t *fix_list,
                                                const int32_t *fix_count) {
  using Val = typename Pol::Val;
  const int n = *fix_count;
  const int lane = threadIdx.x & 31;
  const int gwarp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  for (int i = gwarp; i < n; i += nwarps) {
    const int c = fix_list[i];
    const int row = ch_a0[c];
    const int start = row > 0 ? __ldg(src.ends + row - 1) : 0;
    const int c_first = start >> slab_chunk_log2(src);
    Val acc = pol.zero();
    for (int q = c_first; q < c; q += 32) {
      Val x = (q + lane < c) ? ch_carry[q + lane] : pol.zero();
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const Val y = shfl_down_any(x, d);
        if (lane + d < 32) x = pol.reduce(x, y);
      }
      acc = pol.reduce(acc, x);
    }
    if (lane == 0) {
      const int v = src.vid ? __ldg(src.vid + row) : row;
      pol.emit(row, v, pol.reduce(acc, ch_first[c]));
    }
  }
}

__host__ __device__ inline SlabSource slab_source(const int32_t *ends, const int32_t *vid,
                                                  const int32_t *delta, int n_seg,
                                                  int n_edge, const int32_t *n_seg_p,
                                                  const int32_t *n_edge_p,
                                                  const int32_t *part,
                                                  const int32_t *chunk_log2_p = nullptr) {
  SlabSource s;
  s.ends = ends;
  s.vid = vid;
  s.delta = delta;
  s.n_seg = n_seg;
  s.n_edge = n_edge;
  s.n_seg_p = n_seg_p;
  s.n_edge_p = n_edge_p;
  s.part = part;
  s.chunk_log2_p = chunk_log2_p;
  return s;
}

}  // namespace gasdev

#endif  // GAS_DEVICE_CUH_
