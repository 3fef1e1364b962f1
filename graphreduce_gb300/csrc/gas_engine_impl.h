// gas_engine_impl.h -- the engine object shared by libgas translation units
// (not installed).
#ifndef GAS_ENGINE_IMPL_H_
#define GAS_ENGINE_IMPL_H_

#include <cuda_runtime.h>

#include <vector>

#include "gas.h"
#include "gas_internal.h"

#define CUDA_TRY(call)                                                       \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      return gas::fail(GAS_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__,     \
                       #call, cudaGetErrorString(e_));                       \
  } while (0)

#define GAS_TRY(call)                  \
  do {                                 \
    gas_status_t s_ = (call);          \
    if (s_ != GAS_OK) return s_;       \
  } while (0)

// ---------------------------------------------------------------------------
// The engine object.
// ---------------------------------------------------------------------------
// Instantiated CUDA graphs cached per engine (valid until the next
// set_graph, since their kernels capture the engine's buffers).
// BFS runs on graphs up to this many vertices take the one-kernel path.
constexpr int kBfsSmallMaxV = 1 << 18;

enum { kGraphGeneric = 0, kGraphOrdered = 1, kGraphPagerank = 2, kGraphUser = 3,
       kGraphFast0 = 4, kGraphSlots = 12 };

struct gas_engine {
  gas_program_t prog = GAS_PROG_USER;
  size_t vbytes = 0, gbytes = 0, ebytes = 0;
  int32_t nV = 0, nE = 0;
  void *host_vd = nullptr;
  void *host_ed = nullptr;             // caller's edge data (user engines)
  std::vector<int32_t> h_csr_perm;     // edge-list index of each CSR edge
  std::vector<int32_t> h_csr_to_csc;   // CSC position of each CSR edge
  int32_t *csr_to_csc = nullptr;       // device copy (on first scatter)
  bool edges_dirty = false;            // a user scatter may have changed edge data
  int edge_place = GAS_EDGES_DEVICE;   // placement for the next set_graph
  bool edges_on_host = false;          // csc_src/csr_dst/csc_ed/csr_ed are pinned host memory
  std::vector<int32_t> h_csc_off;  // for host-side counts in setActive

  // device graph
  int32_t *csc_off = nullptr, *csc_src = nullptr, *csr_off = nullptr,
          *csr_dst = nullptr;
  void *csc_ed = nullptr, *csr_ed = nullptr;

  // device vertex + frontier state
  void *vd = nullptr;
  int32_t *act = nullptr, *scan = nullptr, *sscan = nullptr;
  uint8_t *ret = nullptr;
  void *slot = nullptr, *gres = nullptr;
  uint32_t *bits = nullptr;
  void *tile_first = nullptr, *tile_carry = nullptr;
  int32_t *tile_a0 = nullptr;
  int32_t tile_cap = 0;
  int32_t *tpart = nullptr;  // tile partitions of the current frontier pass
  int32_t *dpart = nullptr;  // tile partitions of the dense CSC (pull passes)
  int32_t *ppart = nullptr;  // predicated-scan partials
  int32_t *cpart = nullptr;  // compaction partials (pairs)
  int32_t n_cblocks = 0;
  gas_counters *cnt = nullptr;
  gas_counters *h_cnt = nullptr;  // pinned

  // precision PageRank buffers (lazily allocated)
  float *pr_rank[2] = {nullptr, nullptr};
  float *pr_contrib[2] = {nullptr, nullptr};
  int32_t *pr_seed = nullptr;  // personalization seed of the run (-1: none)
  float *pr_inv_deg = nullptr;  // [V] RN(1 / out-degree) (0: none)
  double *pr_l1 = nullptr;
  int32_t pr_l1_cap = 0;
  // merge-path tiles of the CSC: start rows [tiles + 1], head and tail
  // carry records [tiles]
  int32_t *pr_tile_row = nullptr;
  void *pr_head = nullptr, *pr_tail = nullptr;
  int32_t pr_tile_cap = 0;
  double pr_damping = 0.0;

  // fast-schedule state (lazily allocated): frontier queue of C_k with the
  // values its members had at the end of iteration k, out-degree scan,
  // changed bitmap (being built), membership bitmap of C_k, snapshots
  int32_t *q_ids = nullptr, *q_vals = nullptr, *q_end = nullptr, *q_delta = nullptr;
  int32_t *snap = nullptr, *qpart = nullptr;
  uint32_t *cbits = nullptr;
  int32_t pull_div = 4;

  // non-empty in-edge rows of the CSC (dense slab passes)
  int32_t *ne_vid = nullptr, *ne_end = nullptr;
  int32_t n_ne = 0;
  // warp-slab chunk state: partitions of the dense CSC and of the push
  // queue, per-chunk carries (8-byte values) and fixup rows
  int32_t *slab_dpart = nullptr, *slab_qpart = nullptr, *slab_a0 = nullptr;
  // traces and the learned schedule
  gas_trace_record *trace = nullptr;  // [GAS_TRACE_CAP] device
  int32_t *hist = nullptr;            // [8] degree histogram of the queue
  bool trace_on = false;
  const void *sched_model = nullptr;  // BF16 weights of the schedule head
  int32_t *slab_fix = nullptr;      // chunks needing a fixup, [slab_cap]
  int32_t *slab_fix_n = nullptr;    // their count (reset after each fixup)
  void *slab_first = nullptr, *slab_carry = nullptr;
  int32_t slab_cap = 0;

  // host view of the step API state
  int32_t n_active = 0, n_edges = 0;
  bool counts_dirty = false;
  bool pending_gather = false;
  bool have_gres = false;
  bool slots_pending = false;
  int32_t level = 0;
  int num_sms = 0;
  bool has_graph = false;
  // kernel profiling (gas_engine_set_profiling)
  bool profiling = false;
  cudaEvent_t prof_ev[2] = {nullptr, nullptr};
  int prof_kind = -1;           // kernel bracketed in the current iteration
  int64_t prof_bytes_pending = 0;
  gas_kernel_profile prof = {};
  bool active_full = false;          // active set is [0, nV) from set_active
  bool capturing = false;            // fixed grids (graph capture / host loop)
  bool in_graph = false;             // loop kernels set a graph condition
  cudaGraphExec_t graphs[kGraphSlots] = {};
  bool level_from_counters = false;  // BFS level = counters.iteration
  // small-graph BFS (gas_small.cu): three frontier bitmaps, the control
  // word, the level's members with many out-edges
  uint32_t *sb_bits = nullptr;
  void *sb_ctl = nullptr;
  int32_t *sb_heavy = nullptr;
  bool sb_clean = false;  // the kernel left them clear for the next run
  // what graphs[kGraphUser] was captured with (gas_engine_run_user)
  gas_user_step_fn user_step = nullptr;
  void *user_ctx = nullptr;
  int32_t user_wrote_slots = -1;
};

namespace gas {
// commit pending slots + expansion + compaction of the next frontier
gas_status_t engine_scatter(gas_engine *e, void *stream);
// one bulk-synchronous iteration of the generic (step API) kernels
gas_status_t engine_generic_iteration(gas_engine *e, bool ordered, void *stream);
// pieces of it: fused gather+apply into slots / apply only / commit slots
gas_status_t engine_gather_apply(gas_engine *e, void *stream);
gas_status_t engine_apply_only(gas_engine *e, void *stream);
gas_status_t engine_commit(gas_engine *e, void *stream);
// host copy of the counters (synchronises the stream)
gas_status_t engine_sync_counts(gas_engine *e, void *stream);
int engine_grid(int64_t work_items, int per_block, int cap);
// CSR/CSC on the device (gas_build.cu): fills csc_off/csc_src/csr_off/
// csr_dst (+ csc_ed/csr_ed), which must be allocated, and h_csc_off; the
// permutations (edge-list index per CSC / CSR position) when asked for.
gas_status_t build_graph_device(gas_engine *e, const int32_t *srcs, const int32_t *dsts,
                                const void *edge_data, std::vector<int32_t> *csc_perm,
                                std::vector<int32_t> *csr_perm, void *stream);
// Whether set_graph builds on the device: GAS_GRAPH_BUILD=host|device, else
// from 1M edges up.
bool device_build_for(int64_t n_edges);
// grid of a k_partition launch (fixed while capturing)
int engine_partition_grid(gas_engine *e, int64_t items, int tile);
// GAS_HOST_LOOP=1: device loops run as direct launches with one host read
// of the condition per iteration (the kernels are the same; ncu cannot
// profile kernels inside graphs with conditional nodes).
bool host_loop_requested();
// Profiling hooks: bracket one kernel of the current iteration (host loop
// only) and fold its time into the profile once the iteration has run.
enum { kProfPush = 0, kProfPull = 1, kProfPagerank = 2 };
void prof_begin(gas_engine *e, cudaStream_t s, int kind, int64_t bytes);
void prof_end(gas_engine *e, cudaStream_t s);
void prof_collect(gas_engine *e);
}  // namespace gas

#endif  // GAS_ENGINE_IMPL_H_
