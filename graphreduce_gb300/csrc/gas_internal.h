// gas_internal.h -- helpers shared by libgas translation units (not installed).
#ifndef GAS_INTERNAL_H_
#define GAS_INTERNAL_H_

#include <stdint.h>

#include "gas.h"

namespace gas {

// Records a printf-style message as this thread's last error and returns s.
gas_status_t fail(gas_status_t s, const char *fmt, ...)
    __attribute__((format(printf, 2, 3)));

// Clears this thread's last error / returns it.
void clear_error();
const char *g_err_ptr();

// Stable CSR construction on the host (util.cuh:80-111 semantics).
gas_status_t build_csr_host(int32_t nV, int64_t nE, const int32_t *keys,
                            const int32_t *vals, int32_t *offsets,
                            int32_t *out, int32_t *perm);

}  // namespace gas

#endif  // GAS_INTERNAL_H_
