// gas_features.h -- the schedule head's input features, evaluated the same
// way on the host (training data) and in the device loop (not installed).
#ifndef GAS_FEATURES_H_
#define GAS_FEATURES_H_

#include <math.h>
#include <stdint.h>

#include "gas.h"

namespace gasfeat {

// Degree-histogram bucket of a frontier vertex with out-degree d >= 1.
__host__ __device__ inline int degree_bucket(int d) {
  int l = 0;
  while ((d >> (l + 1)) > 0 && l < 30) ++l;  // floor(log2 d)
  const int b = l / 2;
  return b < 7 ? b : 7;
}

__host__ __device__ inline void schedule_features(int n_queue, int n_edges_out,
                                                  const int32_t *hist, int iteration,
                                                  int nV, long long nE, int weighted,
                                                  float *f) {
  f[0] = log2f(1.0f + (float)n_queue) / 32.0f;
  f[1] = log2f(1.0f + (float)n_edges_out) / 32.0f;
  f[2] = log2f(1.0f + (float)nV) / 32.0f;
  f[3] = log2f(1.0f + (float)nE) / 32.0f;
  f[4] = nE > 0 ? (float)n_edges_out / (float)nE : 0.0f;
  f[5] = nV > 0 ? (float)n_queue / (float)nV : 0.0f;
  for (int b = 0; b < 8; ++b)
    f[6 + b] = n_queue > 0 ? (float)hist[b] / (float)n_queue : 0.0f;
  f[14] = (float)(iteration < 64 ? iteration : 64) / 64.0f;
  f[15] = weighted ? 1.0f : 0.0f;
}

// PageRank warm-start input of a vertex.
__host__ __device__ inline void warm_features(float log_in, float log_out, int nV,
                                              long long nE, float *f) {
  f[0] = log_in / 32.0f;
  f[1] = log_out / 32.0f;
  f[2] = log2f(1.0f + (float)nV) / 32.0f;
  f[3] = log2f(1.0f + (nV > 0 ? (float)nE / (float)nV : 0.0f)) / 8.0f;
}

}  // namespace gasfeat

#endif  // GAS_FEATURES_H_
