/*
 * gpugas.h -- drop-in replacement for the reference's GPU engine header
 * (gpugas.h:1025-1809, class GASEngineGPU), for one GB300 (sm_103a).
 *
 * The reference apps (bfs.cu, sssp.cu, pagerank.cu, connected_component.cu)
 * compile unchanged against this header when it sits beside them (or comes
 * first on the include path) and the program links libgas:
 *
 *   nvcc -gencode arch=compute_103a,code=sm_103a -std=c++17 \
 *        -I<repo>/include app.cu util.cu graphio.cpp -L<lib dir> -lgas -lz
 *
 * The Program-typed kernels (the load-balanced gather with Program::apply in
 * its epilogue, and apply without gather) are templates from gas_device.cuh
 * instantiated in the app's own translation unit, so user functors and the
 * app's __constant__ variables (bfs.cu:28) are visible to them.  Everything
 * that does not depend on the Program -- CSR/CSC construction, the commit of
 * applied vertex data, frontier expansion and compaction -- is libgas code
 * reached through the C ABI of gas.h.
 *
 * Semantics kept from the reference: bulk-synchronous iterations (gather
 * reads the vertex data of the previous iteration), active lists in
 * ascending vertex id, setGraph re-callable on one engine (sssp.cu:85),
 * all work on the legacy default stream (the apps write __constant__ data
 * with cudaMemcpyToSymbol between steps), errors printed as
 * "file(line): ..." followed by abort() (gpugas.h:1105-1112).
 * Differences: getResults() really copies the vertex data back (at the
 * reference's HEAD its body is compiled out, gpugas.h:1778-1787); there are
 * no shards, because the whole graph stays resident in HBM.
 */
#ifndef GPUGAS_H__
#define GPUGAS_H__

#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "gas.h"
#include "gas_device.cuh"

template <typename Program, typename Int = int32_t,
          bool sortEdgesForGather = true>
class GASEngineGPU {
 public:
  typedef typename Program::VertexData VertexData;
  typedef typename Program::EdgeData EdgeData;
  typedef typename Program::GatherResult GatherResult;

 private:
  gas_engine *m_engine;
  gas_engine_view m_view;
  bool m_haveGraph;
  bool m_pendingGather;  // gather() called, kernels not launched yet
  bool m_haveGatherTmp;  // gather_tmp holds this iteration's gather results
  int m_gatherGrid;
  int m_applyGrid;
  gas_run_stats m_lastRun;  // what the last run() did (not in the reference)

  void check(gas_status_t s, const char *file, int line) {
    if (s != GAS_OK) {
      printf("%s(%d): gas error %d (%s): %s\n", file, line, (int)s,
             gas_status_string(s), gas_last_error());
      abort();
    }
  }
  void checkCuda(cudaError_t err, const char *file, int line) {
    if (err != cudaSuccess) {
      printf("%s(%d): cuda error %d (%s)\n", file, line, (int)err,
             cudaGetErrorString(err));
      abort();
    }
  }
#define GPUGAS_CHECK(X) check((X), __FILE__, __LINE__)
#define GPUGAS_CUDA(X) checkCuda((X), __FILE__, __LINE__)

  gasdev::GenericGather<Program> policy(bool fuse) const {
    gasdev::GenericGather<Program> p;
    p.csc_src = m_view.csc_src;
    p.csc_ed = static_cast<const EdgeData *>(m_view.csc_ed);
    p.vd = static_cast<const VertexData *>(m_view.vertex_data);
    p.slot = static_cast<VertexData *>(m_view.slot);
    p.ret = m_view.apply_ret;
    p.gres = static_cast<GatherResult *>(m_view.gather_tmp);
    p.fuse = fuse ? 1 : 0;
    return p;
  }

  // The load-balanced gather over the current active list; with fuse, apply
  // runs in the epilogue and the new vertex data waits in per-slot storage
  // until scatterActivate commits it.  With fixedGrids the launch reads no
  // host-side count (every kernel loops over what the device counters say),
  // so that it can be captured into run()'s device loop.
  cudaError_t launchGatherOn(cudaStream_t stream, bool fuse, bool fixedGrids) {
    typedef gasdev::TileShape<sizeof(GatherResult)> Shape;
    long long tiles = 0;
    if (!fixedGrids) {
      gas_counters c;
      GPUGAS_CHECK(gas_engine_read_counters(m_engine, &c, stream));
      if (c.n_active == 0) return cudaSuccess;
      const long long items = (long long)c.n_active + c.n_edges;
      tiles = (items + Shape::kTile - 1) / Shape::kTile;
    }
    const gasdev::SegSource src = gasdev::frontier_source(
        m_view.active, m_view.active_scan, m_view.csc_off,
        &m_view.counters->n_active, &m_view.counters->n_edges, m_view.tile_part);
    const long long pblocks = fixedGrids ? 2LL * m_view.num_sms : (tiles + 1 + 255) / 256;
    gasdev::k_partition<Shape::kTile, false>
        <<<(int)(pblocks < 2 * m_view.num_sms ? pblocks : 2 * m_view.num_sms), 256, 0,
           stream>>>(src, m_view.tile_part);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    const int grid = fixedGrids ? m_gatherGrid
                                : (int)(tiles < m_gatherGrid ? tiles : m_gatherGrid);
    gasdev::k_gather_tiles<Program><<<grid, gasdev::kNT, 0, stream>>>(
        policy(fuse), src, static_cast<GatherResult *>(m_view.tile_first),
        static_cast<GatherResult *>(m_view.tile_carry), m_view.tile_a0);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    const long long fix = fixedGrids ? 32LL * m_view.num_sms : (tiles + 7) / 8;
    const int fgrid = (int)(fix < 4 * m_view.num_sms ? fix : 4 * m_view.num_sms);
    gasdev::k_gather_fixup<Program><<<fgrid > 0 ? fgrid : 1, gasdev::kNT, 0, stream>>>(
        policy(fuse), src, static_cast<GatherResult *>(m_view.tile_first),
        static_cast<GatherResult *>(m_view.tile_carry), m_view.tile_a0);
    return cudaGetLastError();
  }

  void launchGather(bool fuse) { GPUGAS_CUDA(launchGatherOn(0, fuse, false)); }

  // run()'s loop body, Program-typed part: gather with apply fused, fixed
  // grids, on the stream libgas is capturing.
  static gas_status_t deviceLoopStep(void *self, void *stream) {
    GASEngineGPU *me = static_cast<GASEngineGPU *>(self);
    return me->launchGatherOn(static_cast<cudaStream_t>(stream), true, true) == cudaSuccess
               ? GAS_OK
               : GAS_ERR_CUDA;
  }

  void launchScatter() {
    gas_counters c;
    GPUGAS_CHECK(gas_engine_read_counters(m_engine, &c, 0));
    if (c.n_active == 0) return;
    const int32_t *map = 0;
    GPUGAS_CHECK(gas_engine_prepare_scatter(m_engine, &map, 0));
    const long long warps = c.n_active;
    const long long blocks = (warps * 32 + gasdev::kNT - 1) / gasdev::kNT;
    const int grid = (int)(blocks < 8 * m_view.num_sms ? blocks : 8 * m_view.num_sms);
    EdgeData *csr_ed = map ? static_cast<EdgeData *>(const_cast<void *>(m_view.csr_ed)) : 0;
    gasdev::k_scatter_user<Program><<<grid, gasdev::kNT>>>(
        m_view.active, m_view.counters, m_view.apply_ret, m_view.csr_off, m_view.csr_dst,
        static_cast<const VertexData *>(m_view.vertex_data), csr_ed,
        static_cast<EdgeData *>(const_cast<void *>(m_view.csc_ed)), map);
    GPUGAS_CUDA(cudaGetLastError());
  }

  void flushGather() {
    if (!m_pendingGather) return;
    m_pendingGather = false;
    launchGather(false);
    m_haveGatherTmp = true;
  }

 public:
  GASEngineGPU()
      : m_engine(0), m_haveGraph(false), m_pendingGather(false),
        m_haveGatherTmp(false), m_gatherGrid(1), m_applyGrid(1), m_lastRun() {
    static_assert(sizeof(Int) == 4, "libgas indexes vertices and edges with 32 bits");
    GPUGAS_CHECK(gas_engine_create_user(sizeof(VertexData), sizeof(GatherResult),
                                        sizeof(EdgeData), &m_engine));
  }

  ~GASEngineGPU() { gas_engine_destroy(m_engine); }

  // gpugas.h:1314-1503
  void setGraph(Int nVertices, VertexData *vertexData, Int nEdges,
                EdgeData *edgeData, const Int *edgeListSrcs,
                const Int *edgeListDsts) {
    GPUGAS_CHECK(gas_engine_set_graph(m_engine, nVertices, vertexData, nEdges,
                                      edgeData, edgeListSrcs, edgeListDsts, 0));
    GPUGAS_CHECK(gas_engine_view_get(m_engine, &m_view));
    int perSm = 0;
    GPUGAS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &perSm, gasdev::k_gather_tiles<Program>, gasdev::kNT, 0));
    m_gatherGrid = m_view.num_sms * (perSm > 0 ? perSm : 1);
    m_applyGrid = 8 * m_view.num_sms;
    m_haveGraph = true;
    m_pendingGather = false;
    m_haveGatherTmp = false;
  }

  // gpugas.h:1524-1546
  void setActive(Int vertexStart, Int vertexEnd) {
    flushGather();
    GPUGAS_CHECK(gas_engine_set_active(m_engine, vertexStart, vertexEnd, 0));
  }

  // gpugas.h:1548-1551
  Int countActive() {
    int32_t n = 0;
    GPUGAS_CHECK(gas_engine_count_active(m_engine, &n));
    return n;
  }

  // gpugas.h:1553-1619.  The launch is deferred to apply() so that gather and
  // apply run as one kernel.
  void gather(bool haveGather = true) {
    m_haveGatherTmp = false;
    m_pendingGather = haveGather;
  }

  // gpugas.h:1621-1648
  void apply() {
    if (m_pendingGather) {
      m_pendingGather = false;
      launchGather(true);
      GPUGAS_CHECK(gas_engine_note_applied(m_engine, 1));
      return;
    }
    gas_counters c;
    GPUGAS_CHECK(gas_engine_read_counters(m_engine, &c, 0));
    if (c.n_active == 0) return;
    const int g = (c.n_active + gasdev::kNT - 1) / gasdev::kNT;
    gasdev::k_apply_only<Program><<<g < m_applyGrid ? g : m_applyGrid, gasdev::kNT>>>(
        m_view.active, m_view.counters, static_cast<VertexData *>(m_view.vertex_data),
        m_haveGatherTmp ? static_cast<const GatherResult *>(m_view.gather_tmp) : 0,
        m_view.apply_ret);
    GPUGAS_CUDA(cudaGetLastError());
    GPUGAS_CHECK(gas_engine_note_applied(m_engine, 0));
  }

  // gpugas.h:1650-1759.  Program::scatter runs on the GPU when the program
  // asks for it with `static const bool runScatter = true;`; otherwise, as
  // in the reference GPU engine, only the activation happens.
  void scatterActivate(bool haveScatter = true) {
    flushGather();
    if (haveScatter && gasdev::RunsScatter<Program>::value) launchScatter();
    GPUGAS_CHECK(gas_engine_scatter_activate(m_engine, haveScatter ? 1 : 0, 0));
    m_haveGatherTmp = false;
  }

  // gpugas.h:1761-1772
  Int nextIter() {
    int32_t n = 0;
    GPUGAS_CHECK(gas_engine_next_iter(m_engine, &n, 0));
    return n;
  }

  // gpugas.h:1778-1787 (with the copy-back its comment describes)
  void getResults() {
    flushGather();
    GPUGAS_CHECK(gas_engine_get_results(m_engine, 0));
  }

  // gpugas.h:1792-1807: iterate until no vertex is active, then print the
  // count.  The loop runs on the device -- one CUDA-graph launch whose WHILE
  // node holds an iteration's kernels (this Program's gather with apply
  // fused, then libgas's commit, scatter-activate and compaction) and tests
  // the frontier there -- so no host round trip happens per iteration.
  // Programs that run Program::scatter on the GPU take the step loop.
  void run() {
    if (gasdev::RunsScatter<Program>::value) {
      m_lastRun = gas_run_stats();
      int i = 1;
      while (countActive()) {
        gather();
        apply();
        scatterActivate();
        nextIter();
        ++i;
      }
      printf("Iterations: %d\n", i - 1);
      return;
    }
    flushGather();
    GPUGAS_CHECK(gas_engine_run_user(m_engine, &GASEngineGPU::deviceLoopStep, this, 1, 0,
                                     &m_lastRun, 0));
    m_haveGatherTmp = false;
    printf("Iterations: %d\n", m_lastRun.iterations);
  }

  // Not in the reference: iterations and launches of the last run() (all
  // zero after a run() that took the step loop).
  const gas_run_stats &lastRun() const { return m_lastRun; }

#undef GPUGAS_CHECK
#undef GPUGAS_CUDA
};

#endif  // GPUGAS_H__
