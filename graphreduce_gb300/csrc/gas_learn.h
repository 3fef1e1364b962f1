// gas_learn.h -- device pieces of the learned schedule / warm start shared
// by libgas translation units (not installed).
#ifndef GAS_LEARN_H_
#define GAS_LEARN_H_

#include <cuda_bf16.h>
#include <stddef.h>

#include "gas.h"

namespace gaslearn {

constexpr int kH = GAS_MLP_HIDDEN;

// Offsets of the flat parameter layout of gas_mlp.
struct Layout {
  int n_in, n_out;
  size_t w1, b1, w2, b2, w3, b3, total;
};

__host__ __device__ constexpr Layout layout(int n_in, int n_out) {
  Layout l{};
  l.n_in = n_in;
  l.n_out = n_out;
  l.w1 = 0;
  l.b1 = l.w1 + (size_t)n_in * kH;
  l.w2 = l.b1 + kH;
  l.b2 = l.w2 + (size_t)kH * kH;
  l.w3 = l.b2 + kH;
  l.b3 = l.w3 + (size_t)kH * n_out;
  l.total = l.b3 + n_out;
  return l;
}

// Forward pass of one sample, FP32 weights (the BF16 values) in the flat
// layout; FP32 accumulation.
__device__ inline void mlp_eval(const float *wf, int n_in, int n_out, const float *x,
                                float *out) {
  const Layout L = layout(n_in, n_out);
  float h1[kH];
#pragma unroll 4
  for (int j = 0; j < kH; ++j) {
    float a = wf[L.b1 + j];
    for (int i = 0; i < n_in; ++i) a += x[i] * wf[L.w1 + i * kH + j];
    h1[j] = a > 0.f ? a : 0.f;
  }
  float o0 = wf[L.b3], o1 = n_out > 1 ? wf[L.b3 + 1] : 0.f;
  for (int j = 0; j < kH; ++j) {
    float a = wf[L.b2 + j];
#pragma unroll 8
    for (int i = 0; i < kH; ++i) a += h1[i] * wf[L.w2 + i * kH + j];
    const float h2 = a > 0.f ? a : 0.f;
    o0 += h2 * wf[L.w3 + j * n_out];
    if (n_out > 1) o1 += h2 * wf[L.w3 + j * n_out + 1];
  }
  out[0] = o0;
  if (n_out > 1) out[1] = o1;
}

const void *mlp_bf16(const gas_mlp *m);
int mlp_inputs(const gas_mlp *m);
int mlp_outputs(const gas_mlp *m);

}  // namespace gaslearn

#endif  // GAS_LEARN_H_
