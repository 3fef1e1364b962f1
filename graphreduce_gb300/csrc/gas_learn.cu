// gas_learn.cu -- the learned parts of the engine (no reference counterpart):
//
//   * a small MLP (n_in -> 64 -> 64 -> n_out, ReLU) with BF16 weights used
//     for inference and FP32 master weights, trained on the GPU by the
//     hand-written forward/backward and Adam kernels below (FP32
//     accumulation throughout);
//   * the schedule head: features of the frontier at the end of an
//     iteration -> {push, dense pull} for the next one, evaluated by one warp
//     inside the device loop (gas_sched.cu);
//   * the PageRank warm-start head: per-vertex degree features -> an initial
//     rank, evaluated by one thread per vertex.
//
// Parameter layout (flat, FP32 master / BF16 copy):
//   W1[n_in][H] b1[H] W2[H][H] b2[H] W3[H][n_out] b3[n_out]
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "gas.h"
#include "gas_internal.h"
#include "gas_engine_impl.h"
#include "gas_features.h"
#include "gas_learn.h"

namespace {

constexpr int H = GAS_MLP_HIDDEN;

inline cudaStream_t S(void *s) { return (cudaStream_t)s; }

#define LCUDA(call)                                                           \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess)                                                    \
      return gas::fail(GAS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

size_t n_params(int n_in, int n_out) {
  return (size_t)n_in * H + H + (size_t)H * H + H + (size_t)H * n_out + n_out;
}

// splitmix-based uniform in [-1, 1) for the initial weights
inline float uni(uint64_t seed, uint64_t i) {
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + i + 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (float)((double)(z >> 11) * (1.0 / 9007199254740992.0)) * 2.0f - 1.0f;
}

// One CTA of H threads per sample: forward, loss, backward; gradients are
// accumulated into g (FP32) with atomics.  kind: 0 = softmax cross-entropy
// over n_out classes with per-sample weights, 1 = squared error on output 0.
__global__ void __launch_bounds__(H)
    k_mlp_train(const __nv_bfloat16 *w, int n_in, int n_out, const float *x,
                const int32_t *y, const float *t, const float *sw, float inv_norm,
                int kind, float *g, float *loss) {
  __shared__ float s_x[GAS_MLP_MAX_IN];
  __shared__ float s_h1[H], s_h2[H], s_d2[H], s_out[GAS_MLP_MAX_OUT],
      s_dout[GAS_MLP_MAX_OUT];
  const gaslearn::Layout L = gaslearn::layout(n_in, n_out);
  const int b = blockIdx.x, j = threadIdx.x;
  if (j < n_in) s_x[j] = x[(size_t)b * n_in + j];
  __syncthreads();
  float a = __bfloat162float(w[L.b1 + j]);
  for (int i = 0; i < n_in; ++i) a += s_x[i] * __bfloat162float(w[L.w1 + (size_t)i * H + j]);
  const float h1 = a > 0.f ? a : 0.f;
  s_h1[j] = h1;
  __syncthreads();
  a = __bfloat162float(w[L.b2 + j]);
  for (int i = 0; i < H; ++i) a += s_h1[i] * __bfloat162float(w[L.w2 + (size_t)i * H + j]);
  const float h2 = a > 0.f ? a : 0.f;
  s_h2[j] = h2;
  __syncthreads();
  if (j < n_out) {
    float o = __bfloat162float(w[L.b3 + j]);
    for (int i = 0; i < H; ++i) o += s_h2[i] * __bfloat162float(w[L.w3 + (size_t)i * n_out + j]);
    s_out[j] = o;
  }
  __syncthreads();
  if (j == 0) {
    const float wt = sw ? sw[b] : 1.0f;
    if (kind == 0) {
      float m = s_out[0];
      for (int o = 1; o < n_out; ++o) m = fmaxf(m, s_out[o]);
      float z = 0.f;
      for (int o = 0; o < n_out; ++o) z += expf(s_out[o] - m);
      const int yb = y[b];
      atomicAdd(loss, wt * inv_norm * (logf(z) + m - s_out[yb]));
      for (int o = 0; o < n_out; ++o) {
        const float p = expf(s_out[o] - m) / z;
        s_dout[o] = wt * inv_norm * (p - (o == yb ? 1.f : 0.f));
      }
    } else {
      const float d = s_out[0] - t[b];
      atomicAdd(loss, wt * inv_norm * d * d);
      s_dout[0] = 2.f * wt * inv_norm * d;
      for (int o = 1; o < n_out; ++o) s_dout[o] = 0.f;
    }
  }
  __syncthreads();
  // output layer
  float d2 = 0.f;
  for (int o = 0; o < n_out; ++o) {
    atomicAdd(g + L.w3 + (size_t)j * n_out + o, h2 * s_dout[o]);
    d2 += __bfloat162float(w[L.w3 + (size_t)j * n_out + o]) * s_dout[o];
  }
  if (j < n_out) atomicAdd(g + L.b3 + j, s_dout[j]);
  d2 = h2 > 0.f ? d2 : 0.f;
  s_d2[j] = d2;
  __syncthreads();
  // hidden layer 2: W2[i][j] gets h1[i] * d2[j]
  atomicAdd(g + L.b2 + j, d2);
  for (int i = 0; i < H; ++i) atomicAdd(g + L.w2 + (size_t)i * H + j, s_h1[i] * d2);
  float d1 = 0.f;
  for (int k = 0; k < H; ++k) d1 += __bfloat162float(w[L.w2 + (size_t)j * H + k]) * s_d2[k];
  d1 = h1 > 0.f ? d1 : 0.f;
  atomicAdd(g + L.b1 + j, d1);
  for (int i = 0; i < n_in; ++i) atomicAdd(g + L.w1 + (size_t)i * H + j, s_x[i] * d1);
}

__global__ void k_adam(float *p, float *g, float *m, float *v, __nv_bfloat16 *wb,
                       size_t n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    wb[i] = __float2bfloat16(pi);
    g[i] = 0.f;
  }
}

__global__ void k_to_bf16(const float *p, __nv_bfloat16 *wb, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    wb[i] = __float2bfloat16(p[i]);
}

// One thread per sample, weights staged in shared memory as FP32 (they are
// BF16 values, so the products are exact in FP32; sums accumulate in FP32).
__global__ void __launch_bounds__(128)
    k_mlp_forward(const __nv_bfloat16 *w, int n_in, int n_out, const float *x,
                  int n, float *out) {
  extern __shared__ float s_w[];
  const gaslearn::Layout L = gaslearn::layout(n_in, n_out);
  for (size_t i = threadIdx.x; i < L.total; i += blockDim.x) s_w[i] = __bfloat162float(w[i]);
  __syncthreads();
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
    float xi[GAS_MLP_MAX_IN];
    for (int i = 0; i < n_in; ++i) xi[i] = x[(size_t)b * n_in + i];
    float o[GAS_MLP_MAX_OUT];
    gaslearn::mlp_eval(s_w, L.n_in, L.n_out, xi, o);
    for (int k = 0; k < n_out; ++k) out[(size_t)b * n_out + k] = o[k];
  }
}

}  // namespace

struct gas_mlp {
  int n_in = 0, n_out = 0;
  size_t n = 0;
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr, *loss = nullptr;
  __nv_bfloat16 *wb = nullptr;
  int64_t step = 0;
};

namespace gaslearn {
const void *mlp_bf16(const gas_mlp *m) { return m ? m->wb : nullptr; }
int mlp_inputs(const gas_mlp *m) { return m ? m->n_in : 0; }
int mlp_outputs(const gas_mlp *m) { return m ? m->n_out : 0; }
}  // namespace gaslearn

extern "C" {

gas_status_t gas_mlp_create(int32_t n_in, int32_t n_out, uint64_t seed, gas_mlp **out) {
  if (!out || n_in < 1 || n_in > GAS_MLP_MAX_IN || n_out < 1 || n_out > GAS_MLP_MAX_OUT)
    return gas::fail(GAS_ERR_INVALID, "mlp_create: n_in in [1,%d], n_out in [1,%d]",
                     GAS_MLP_MAX_IN, GAS_MLP_MAX_OUT);
  gas_mlp *m = new (std::nothrow) gas_mlp;
  if (!m) return gas::fail(GAS_ERR_NOMEM, "mlp_create");
  m->n_in = n_in;
  m->n_out = n_out;
  m->n = n_params(n_in, n_out);
  const gaslearn::Layout L = gaslearn::layout(n_in, n_out);
  std::vector<float> host(m->n, 0.f);
  // He-uniform initial weights, zero biases
  const float s1 = sqrtf(6.f / n_in), s2 = sqrtf(6.f / H), s3 = sqrtf(6.f / H);
  for (size_t i = 0; i < (size_t)n_in * H; ++i) host[L.w1 + i] = s1 * uni(seed, i);
  for (size_t i = 0; i < (size_t)H * H; ++i) host[L.w2 + i] = s2 * uni(seed + 1, i);
  for (size_t i = 0; i < (size_t)H * n_out; ++i) host[L.w3 + i] = 0.5f * s3 * uni(seed + 2, i);
  cudaError_t ce = cudaMalloc(&m->p, m->n * 4);
  if (ce == cudaSuccess) ce = cudaMalloc(&m->g, m->n * 4);
  if (ce == cudaSuccess) ce = cudaMalloc(&m->m, m->n * 4);
  if (ce == cudaSuccess) ce = cudaMalloc(&m->v, m->n * 4);
  if (ce == cudaSuccess) ce = cudaMalloc(&m->loss, 4);
  if (ce == cudaSuccess) ce = cudaMalloc(&m->wb, m->n * 2);
  if (ce == cudaSuccess) ce = cudaMemcpy(m->p, host.data(), m->n * 4, cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemset(m->g, 0, m->n * 4);
  if (ce == cudaSuccess) ce = cudaMemset(m->m, 0, m->n * 4);
  if (ce == cudaSuccess) ce = cudaMemset(m->v, 0, m->n * 4);
  if (ce == cudaSuccess) {
    k_to_bf16<<<64, 256>>>(m->p, m->wb, m->n);
    ce = cudaDeviceSynchronize();
  }
  if (ce != cudaSuccess) {
    gas_mlp_destroy(m);
    return gas::fail(GAS_ERR_CUDA, "mlp_create: %s", cudaGetErrorString(ce));
  }
  *out = m;
  return GAS_OK;
}

void gas_mlp_destroy(gas_mlp *m) {
  if (!m) return;
  cudaFree(m->p); cudaFree(m->g); cudaFree(m->m); cudaFree(m->v);
  cudaFree(m->loss); cudaFree(m->wb);
  delete m;
}

int64_t gas_mlp_num_params(const gas_mlp *m) { return m ? (int64_t)m->n : 0; }

gas_status_t gas_mlp_get_params(const gas_mlp *m, float *host) {
  if (!m || !host) return gas::fail(GAS_ERR_INVALID, "null argument");
  LCUDA(cudaMemcpy(host, m->p, m->n * 4, cudaMemcpyDeviceToHost));
  return GAS_OK;
}

gas_status_t gas_mlp_set_params(gas_mlp *m, const float *host) {
  if (!m || !host) return gas::fail(GAS_ERR_INVALID, "null argument");
  LCUDA(cudaMemcpy(m->p, host, m->n * 4, cudaMemcpyHostToDevice));
  k_to_bf16<<<64, 256>>>(m->p, m->wb, m->n);
  LCUDA(cudaDeviceSynchronize());
  return GAS_OK;
}

gas_status_t gas_mlp_gradients(gas_mlp *m, const float *x, const int32_t *y,
                               const float *t, const float *w, int32_t batch,
                               float *grad_host, float *loss_host, void *stream) {
  if (!m || !x || batch < 1 || (!y && !t))
    return gas::fail(GAS_ERR_INVALID, "mlp_gradients: bad arguments");
  float wsum = (float)batch;
  LCUDA(cudaMemsetAsync(m->g, 0, m->n * 4, S(stream)));
  LCUDA(cudaMemsetAsync(m->loss, 0, 4, S(stream)));
  k_mlp_train<<<batch, H, 0, S(stream)>>>(m->wb, m->n_in, m->n_out, x, y, t, w,
                                          1.0f / wsum, y ? 0 : 1, m->g, m->loss);
  LCUDA(cudaGetLastError());
  if (grad_host) LCUDA(cudaMemcpyAsync(grad_host, m->g, m->n * 4, cudaMemcpyDeviceToHost, S(stream)));
  if (loss_host) LCUDA(cudaMemcpyAsync(loss_host, m->loss, 4, cudaMemcpyDeviceToHost, S(stream)));
  LCUDA(cudaStreamSynchronize(S(stream)));
  LCUDA(cudaMemsetAsync(m->g, 0, m->n * 4, S(stream)));
  return GAS_OK;
}

gas_status_t gas_mlp_train_step(gas_mlp *m, const float *x, const int32_t *y,
                                const float *t, const float *w, int32_t batch,
                                float lr, float *loss_host, void *stream) {
  if (!m || !x || batch < 1 || (!y && !t))
    return gas::fail(GAS_ERR_INVALID, "mlp_train_step: bad arguments");
  LCUDA(cudaMemsetAsync(m->loss, 0, 4, S(stream)));
  k_mlp_train<<<batch, H, 0, S(stream)>>>(m->wb, m->n_in, m->n_out, x, y, t, w,
                                          1.0f / (float)batch, y ? 0 : 1, m->g, m->loss);
  ++m->step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)m->step), c2 = 1.f - powf(b2, (float)m->step);
  k_adam<<<64, 256, 0, S(stream)>>>(m->p, m->g, m->m, m->v, m->wb, m->n, lr, b1, b2,
                                    1e-8f, c1, c2);
  LCUDA(cudaGetLastError());
  if (loss_host) {
    LCUDA(cudaMemcpyAsync(loss_host, m->loss, 4, cudaMemcpyDeviceToHost, S(stream)));
    LCUDA(cudaStreamSynchronize(S(stream)));
  }
  return GAS_OK;
}

gas_status_t gas_mlp_forward(const gas_mlp *m, const float *x, int32_t n, float *out,
                             void *stream) {
  if (!m || !x || !out || n < 0) return gas::fail(GAS_ERR_INVALID, "mlp_forward: bad arguments");
  if (n == 0) return GAS_OK;
  const size_t smem = m->n * sizeof(float);
  const int grid = (n + 127) / 128 < 1024 ? (n + 127) / 128 : 1024;
  LCUDA(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem));
  k_mlp_forward<<<grid, 128, smem, S(stream)>>>(m->wb, m->n_in, m->n_out, x, n, out);
  LCUDA(cudaGetLastError());
  return GAS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// PageRank warm start
// ---------------------------------------------------------------------------
namespace {

constexpr int kWarmGrid = 64;  // log2(1 + degree) in steps of 1/2: 0 .. 31.5

// Bilinear interpolation of the head's prediction over the log-degree grid;
// init[v] = exp(prediction) / N.
__global__ void k_warm_init(const int32_t *csr_off, const int32_t *csc_off, int nV,
                            const float *grid, float *init) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV;
       v += gridDim.x * blockDim.x) {
    const float li = 2.0f * log2f(1.0f + (float)(csc_off[v + 1] - csc_off[v]));
    const float lo = 2.0f * log2f(1.0f + (float)(csr_off[v + 1] - csr_off[v]));
    const float ci = fminf(li, kWarmGrid - 1.001f), co = fminf(lo, kWarmGrid - 1.001f);
    const int i0 = (int)ci, o0 = (int)co;
    const float fi = ci - i0, fo = co - o0;
    const float y00 = grid[i0 * kWarmGrid + o0], y01 = grid[i0 * kWarmGrid + o0 + 1];
    const float y10 = grid[(i0 + 1) * kWarmGrid + o0], y11 = grid[(i0 + 1) * kWarmGrid + o0 + 1];
    const float y = (1.f - fi) * ((1.f - fo) * y00 + fo * y01) + fi * ((1.f - fo) * y10 + fo * y11);
    init[v] = expf(fminf(y, 30.f)) / (float)nV;
  }
}

// Per-block FP64 sums of init over all vertices and over vertices without
// out-edges (fixed order inside a block).
__global__ void __launch_bounds__(256)
    k_warm_mass(const int32_t *csr_off, const float *init, int nV, double *part) {
  __shared__ double s_all[256], s_dang[256];
  double all = 0.0, dang = 0.0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const double r = init[v];
    all += r;
    if (csr_off[v + 1] == csr_off[v]) dang += r;
  }
  s_all[threadIdx.x] = all;
  s_dang[threadIdx.x] = dang;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s_all[threadIdx.x] += s_all[threadIdx.x + o];
      s_dang[threadIdx.x] += s_dang[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s_all[0];
    part[2 * blockIdx.x + 1] = s_dang[0];
  }
}

__global__ void k_warm_scale(float *init, int nV, float scale) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x)
    init[v] = __fmul_rn(init[v], scale);
}

}  // namespace

extern "C" gas_status_t gas_engine_pagerank_warm_start(gas_engine *e, const gas_mlp *m,
                                                       double damping, float *init,
                                                       void *stream) {
  if (!e || !m || !init) return gas::fail(GAS_ERR_INVALID, "null argument");
  if (!e->has_graph) return gas::fail(GAS_ERR_STATE, "no graph");
  if (m->n_in != GAS_WARM_FEATURES || m->n_out != 1)
    return gas::fail(GAS_ERR_INVALID, "warm-start model must be %d -> 1", GAS_WARM_FEATURES);
  if (!(damping > 0.0 && damping < 1.0))
    return gas::fail(GAS_ERR_INVALID, "damping must be in (0,1)");
  const int nV = e->nV;
  if (nV == 0) return GAS_OK;
  std::vector<float> x((size_t)kWarmGrid * kWarmGrid * GAS_WARM_FEATURES);
  for (int i = 0; i < kWarmGrid; ++i)
    for (int o = 0; o < kWarmGrid; ++o)
      gasfeat::warm_features(0.5f * i, 0.5f * o, nV, e->nE,
                             &x[((size_t)i * kWarmGrid + o) * GAS_WARM_FEATURES]);
  float *dx = nullptr, *dy = nullptr, *dinit = nullptr;
  double *dpart = nullptr;
  const int mass_blocks = 2 * e->num_sms;
  std::vector<double> part(2 * (size_t)mass_blocks);
  cudaPointerAttributes attr;
  const bool on_device = cudaPointerGetAttributes(&attr, init) == cudaSuccess &&
                         attr.type == cudaMemoryTypeDevice;
  cudaError_t ce = cudaMalloc(&dx, x.size() * 4);
  if (ce == cudaSuccess) ce = cudaMalloc(&dy, (size_t)kWarmGrid * kWarmGrid * 4);
  if (ce == cudaSuccess && !on_device) ce = cudaMalloc(&dinit, (size_t)nV * 4);
  if (ce == cudaSuccess) ce = cudaMalloc(&dpart, part.size() * sizeof(double));
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(dx, x.data(), x.size() * 4, cudaMemcpyHostToDevice, S(stream));
  gas_status_t st = GAS_OK;
  if (ce == cudaSuccess) st = gas_mlp_forward(m, dx, kWarmGrid * kWarmGrid, dy, stream);
  if (ce == cudaSuccess && st == GAS_OK) {
    float *out = on_device ? init : dinit;
    k_warm_init<<<8 * e->num_sms, 256, 0, S(stream)>>>(e->csr_off, e->csc_off, nV, dy, out);
    ce = cudaGetLastError();
    // Mass correction: PageRank without dangling redistribution has total
    // mass m* = (1-d) / (1 - d (1 - delta)) at its fixed point, delta being
    // the share of the mass on vertices without out-edges; the error along
    // the fixed point itself decays only at rate d, so the start is scaled
    // to m* (delta estimated from the prediction).
    if (ce == cudaSuccess) {
      k_warm_mass<<<mass_blocks, 256, 0, S(stream)>>>(e->csr_off, out, nV, dpart);
      ce = cudaGetLastError();
    }
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(part.data(), dpart, part.size() * sizeof(double),
                           cudaMemcpyDeviceToHost, S(stream));
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(S(stream));
    if (ce == cudaSuccess) {
      double all = 0.0, dang = 0.0;
      for (int b = 0; b < mass_blocks; ++b) {
        all += part[2 * b];
        dang += part[2 * b + 1];
      }
      const double delta = all > 0.0 ? dang / all : 0.0;
      const double mstar = (1.0 - damping) / (1.0 - damping * (1.0 - delta));
      if (all > 0.0) {
        k_warm_scale<<<8 * e->num_sms, 256, 0, S(stream)>>>(out, nV, (float)(mstar / all));
        ce = cudaGetLastError();
      }
    }
    if (ce == cudaSuccess && !on_device)
      ce = cudaMemcpyAsync(init, dinit, (size_t)nV * 4, cudaMemcpyDeviceToHost, S(stream));
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(S(stream));
  }
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(dinit);
  cudaFree(dpart);
  if (st != GAS_OK) return st;
  if (ce != cudaSuccess)
    return gas::fail(GAS_ERR_CUDA, "warm start: %s", cudaGetErrorString(ce));
  return GAS_OK;
}
