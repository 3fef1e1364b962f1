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

// One warp evaluates a two-output model on one feature vector (BF16
// weights in global memory): lane l owns hidden units 2l and 2l+1, so every
// weight row is one coalesced 4-byte load per lane, and the rows are
// unrolled by 8 so that their loads overlap; every lane returns both
// logits.
template <int n_in>
__device__ inline void mlp_warp_logits(const __nv_bfloat16 *w, const float *x,
                                       float *logits) {
  constexpr Layout L = layout(n_in, 2);
  const int lane = threadIdx.x & 31;
  const __nv_bfloat162 *w2v = reinterpret_cast<const __nv_bfloat162 *>(w);
  // element offsets of the layout are even, so row r, units (2l, 2l+1) is
  // the bf16 pair at (offset + r * 64) / 2 + l
  float2 h1 = __bfloat1622float2(w2v[L.b1 / 2 + lane]);
#pragma unroll
  for (int i = 0; i < n_in; ++i) {  // x stays in registers
    const float2 wv = __bfloat1622float2(w2v[(L.w1 + (size_t)i * kH) / 2 + lane]);
    h1.x += x[i] * wv.x;
    h1.y += x[i] * wv.y;
  }
  h1.x = h1.x > 0.f ? h1.x : 0.f;
  h1.y = h1.y > 0.f ? h1.y : 0.f;
  float2 h2 = __bfloat1622float2(w2v[L.b2 / 2 + lane]);
#pragma unroll 8
  for (int i = 0; i < kH; ++i) {
    const float hi = __shfl_sync(0xffffffffu, (i & 1) ? h1.y : h1.x, i >> 1);
    const float2 wv = __bfloat1622float2(w2v[(L.w2 + (size_t)i * kH) / 2 + lane]);
    h2.x += hi * wv.x;
    h2.y += hi * wv.y;
  }
  h2.x = h2.x > 0.f ? h2.x : 0.f;
  h2.y = h2.y > 0.f ? h2.y : 0.f;
  // w3 rows are (unit j: logit 0, logit 1): units 2l, 2l+1 are 4 values
  const float2 a = __bfloat1622float2(w2v[L.w3 / 2 + 2 * lane]);
  const float2 b = __bfloat1622float2(w2v[L.w3 / 2 + 2 * lane + 1]);
  float o0 = h2.x * a.x + h2.y * b.x;
  float o1 = h2.x * a.y + h2.y * b.y;
  for (int d = 16; d > 0; d >>= 1) {
    o0 += __shfl_xor_sync(0xffffffffu, o0, d);
    o1 += __shfl_xor_sync(0xffffffffu, o1, d);
  }
  logits[0] = o0 + __bfloat162float(w[L.b3]);
  logits[1] = o1 + __bfloat162float(w[L.b3 + 1]);
}

const void *mlp_bf16(const gas_mlp *m);
int mlp_inputs(const gas_mlp *m);
int mlp_outputs(const gas_mlp *m);

}  // namespace gaslearn

#endif  // GAS_LEARN_H_
