// gas_sched.h -- fast schedules of the built-in programs (not installed).
#ifndef GAS_SCHED_H_
#define GAS_SCHED_H_

#include <cuda_runtime.h>

#include "gas.h"

struct gas_engine;

namespace gas {

// WHILE(cond) { body } as an instantiated CUDA graph; body captures one
// iteration on the given stream and ends with a kernel that calls
// cudaGraphSetConditional on the handle.
gas_status_t build_while_graph(
    gas_engine *e,
    gas_status_t (*body)(gas_engine *, cudaStream_t, cudaGraphConditionalHandle,
                         void *),
    void *ctx, cudaGraphExec_t *out);

// PUSH / PULL / AUTO schedules of BFS, SSSP, CC (and PageRank falls back to
// the generic kernels): same iteration count and vertex data as run().
gas_status_t run_fast(gas_engine *e, gas_schedule_t schedule,
                      int32_t max_iterations, gas_run_stats *stats,
                      void *stream);

bool host_loop_for(const gas_engine *e);

// BFS on a graph of at most kBfsSmallMaxV vertices as one cooperative
// kernel (gas_small.cu): same depths and iteration count as run_fast.
bool bfs_small_eligible(const gas_engine *e, gas_schedule_t schedule);
gas_status_t run_bfs_small(gas_engine *e, gas_schedule_t schedule, int32_t max_iterations,
                           gas_run_stats *stats, void *stream);

// The loop of build_while_graph as direct launches (GAS_HOST_LOOP=1).
gas_status_t run_host_loop(
    gas_engine *e,
    gas_status_t (*body)(gas_engine *, cudaStream_t, cudaGraphConditionalHandle,
                         void *),
    void *ctx, void *stream);

// Status of a finished device loop from its counters (clears the error word).
gas_status_t loop_status(gas_engine *e, const gas_counters &c, void *stream);

}  // namespace gas

#endif  // GAS_SCHED_H_
