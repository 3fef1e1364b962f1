// gas_sched.cu -- fast schedules of the built-in programs.
#include <cuda_runtime.h>

#include "gas.h"
#include "gas_engine_impl.h"
#include "gas_internal.h"
#include "gas_sched.h"

namespace gas {

gas_status_t run_fast(gas_engine *e, gas_schedule_t schedule,
                      int32_t max_iterations, gas_run_stats *stats,
                      void *stream) {
  (void)schedule;
  return gas_engine_run_schedule(e, GAS_SCHED_GENERIC, max_iterations, stats,
                                 stream);
}

}  // namespace gas
