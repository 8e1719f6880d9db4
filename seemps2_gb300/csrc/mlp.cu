// Rank predictor: a small MLP (GELU hidden layers) with hand-written forward,
// backward and Adam kernels for training on the GPU, and a BF16-weight
// inference kernel used inside the sweep to predict each split's kept rank.
//
// Parameters are one flat FP32 array, layer by layer: W_k (out_k x in_k,
// row-major) then b_k (out_k).  A layer computes Z = X W^T + b and, except for
// the last one, A = gelu(Z) with the tanh form
//   gelu(z) = 0.5 z (1 + tanh(c (z + 0.044715 z^3))),  c = sqrt(2 / pi).
// The training cache holds Z and A of every layer (B x out_k each).
//
// Split features (rank_features, SM_RANK_FEATURES = 37 values) describe the
// split about to be made: the 32 largest singular values of the previous split
// (the neighbouring bond in a sweep) as log10(s_i / s_0) (padding -20), the
// site position site / n, log10 of the tolerance, log2 of 1 + the previous
// kept rank, log2 of min(m, n) of this split and log2 of the bond cap.  The
// target is log2 of the kept rank.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "kernels.cuh"

namespace sm {

namespace {

constexpr int TB = 64, TK = 16, TNT = 256;

// C[M,N] = op(A)[M,K] op(B)[K,N], FP32, op 0 = as stored, 1 = transposed.
__global__ void __launch_bounds__(TNT) k_sgemm(int opA, int opB, int M, int N, int K,
                                               const float* __restrict__ A, int lda,
                                               const float* __restrict__ B, int ldb,
                                               float* __restrict__ C, int ldc) {
  __shared__ float As[TK][TB + 1];
  __shared__ float Bs[TK][TB + 1];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const int m0 = blockIdx.y * TB, n0 = blockIdx.x * TB;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += TK) {
#pragma unroll
    for (int e = 0; e < (TB * TK) / TNT; ++e) {
      const int idx = tid + e * TNT;
      int mm, kk;
      if (opA == 0) { mm = idx / TK; kk = idx % TK; } else { kk = idx / TB; mm = idx % TB; }
      const int gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < K) v = opA == 0 ? A[(size_t)gm * lda + gk] : A[(size_t)gk * lda + gm];
      As[kk][mm] = v;
    }
#pragma unroll
    for (int e = 0; e < (TB * TK) / TNT; ++e) {
      const int idx = tid + e * TNT;
      int nn, kk;
      if (opB == 0) { kk = idx / TB; nn = idx % TB; } else { nn = idx / TK; kk = idx % TK; }
      const int gn = n0 + nn, gk = k0 + kk;
      float v = 0.f;
      if (gn < N && gk < K) v = opB == 0 ? B[(size_t)gk * ldb + gn] : B[(size_t)gn * ldb + gk];
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx + 16 * j;
      if (gn < N) C[(size_t)gm * ldc + gn] = acc[i][j];
    }
  }
}

__device__ __forceinline__ float gelu_f(float z) {
  const float c = 0.7978845608028654f;
  const float t = tanhf(c * (z + 0.044715f * z * z * z));
  return 0.5f * z * (1.f + t);
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float c = 0.7978845608028654f;
  const float t = tanhf(c * (z + 0.044715f * z * z * z));
  return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * c * (1.f + 3.f * 0.044715f * z * z);
}

// Z += b (per column); A = gelu(Z) if A != nullptr
__global__ void k_bias_act(float* __restrict__ Z, const float* __restrict__ b, int M, int N,
                           float* __restrict__ A) {
  const size_t tot = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot;
       e += (size_t)gridDim.x * blockDim.x) {
    const float z = Z[e] + b[e % N];
    Z[e] = z;
    if (A) A[e] = gelu_f(z);
  }
}

// dZ = dA * gelu'(Z)
__global__ void k_gelu_back(const float* __restrict__ dA, const float* __restrict__ Z, size_t n,
                            float* __restrict__ dZ) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    dZ[e] = dA[e] * gelu_grad(Z[e]);
}

// db[j] = sum_i dZ[i][j], one thread per column, rows summed in order
__global__ void k_col_sum(const float* __restrict__ dZ, int M, int N, float* __restrict__ db) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  float a = 0.f;
  for (int i = 0; i < M; ++i) a += dZ[(size_t)i * N + j];
  db[j] = a;
}

// mean squared error: dy = 2 (yhat - y) / B; loss[0] = mean (one block)
__global__ void k_mse(const float* __restrict__ yhat, const float* __restrict__ y, int B,
                      float* __restrict__ dy, float* __restrict__ loss) {
  __shared__ float red[256];
  float a = 0.f;
  for (int i = threadIdx.x; i < B; i += blockDim.x) {
    const float r = yhat[i] - y[i];
    if (dy) dy[i] = 2.f * r / (float)B;
    a += r * r;
  }
  red[threadIdx.x] = a;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0 && loss) loss[0] = red[0] / (float)B;
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[e];
    const float mi = b1 * m[e] + (1.f - b1) * gi;
    const float vi = b2 * v[e] + (1.f - b2) * gi * gi;
    m[e] = mi;
    v[e] = vi;
    p[e] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_to_bf16(const float* __restrict__ x, size_t n, __nv_bfloat16* __restrict__ y) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    y[e] = __float2bfloat16_rn(x[e]);
}

// One inference layer: Y[r][o] = act(sum_i X[r][i] W[o][i] + b[o]); BF16
// weights, FP32 activations and accumulation; one warp per (r, o).
__global__ void k_infer_layer(const float* __restrict__ X, int B, int in, int out,
                              const __nv_bfloat16* __restrict__ W, const float* __restrict__ b,
                              int act, float* __restrict__ Y) {
  const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x % 32;
  if (warp >= (long)B * out) return;
  const int r = (int)(warp / out), o = (int)(warp % out);
  float a = 0.f;
  for (int i = lane; i < in; i += 32)
    a = fmaf(X[(size_t)r * in + i], __bfloat162float(W[(size_t)o * in + i]), a);
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) a += __shfl_xor_sync(0xffffffffu, a, s);
  if (lane == 0) {
    const float z = a + b[o];
    Y[(size_t)r * out + o] = act ? gelu_f(z) : z;
  }
}

inline int blocks_for(size_t n) {
  return (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 4096));
}

int sgemm(cudaStream_t st, int opA, int opB, int M, int N, int K, const float* A, int lda,
          const float* B, int ldb, float* C, int ldc) {
  if (M <= 0 || N <= 0) return SM_OK;
  dim3 grid((N + TB - 1) / TB, (M + TB - 1) / TB);
  k_sgemm<<<grid, TNT, 0, st>>>(opA, opB, M, N, K, A, lda, B, ldb, C, ldc);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

size_t param_count(int L, const int* dims) {
  size_t n = 0;
  for (int k = 0; k < L; ++k) n += (size_t)dims[k + 1] * dims[k] + dims[k + 1];
  return n;
}

int check_dims(int L, const int* dims) {
  if (L < 1 || L > 8 || !dims) {
    set_error("mlp: need 1..8 layers and a dims array");
    return SM_ERR_VALUE;
  }
  for (int k = 0; k <= L; ++k)
    if (dims[k] < 1 || dims[k] > 4096) {
      set_error("mlp: layer widths must be in 1..4096");
      return SM_ERR_VALUE;
    }
  return SM_OK;
}

// Layers of the installed model on rows X (device, batch x dims[0]) -> out
// (device, batch); two ping-pong buffers of batch x widest layer.
int infer(Ctx& c, cudaStream_t st, float* X, int batch, float* tmp, float** out) {
  RankModel& m = c.model;
  int wmax = 0;
  for (int k = 0; k <= m.layers; ++k) wmax = std::max(wmax, m.dims[k]);
  float* cur = X;
  float* bufs[2] = {tmp, tmp + (size_t)batch * wmax};
  size_t wo = 0, bo = 0;
  for (int l = 0; l < m.layers; ++l) {
    const int in = m.dims[l], outd = m.dims[l + 1];
    float* nxt = bufs[l & 1];
    const long warps = (long)batch * outd;
    k_infer_layer<<<(int)((warps * 32 + 255) / 256), 256, 0, st>>>(cur, batch, in, outd, m.w + wo,
                                                                  m.b + bo, l + 1 < m.layers, nxt);
    note_launch();
    wo += (size_t)in * outd;
    bo += outd;
    cur = nxt;
  }
  SM_CUDA_CHECK(cudaGetLastError());
  *out = cur;
  return SM_OK;
}

// The features of rank_features on the device: f[0..31] from the previous
// split's sorted values (len of them), then the host-known scalars.
__global__ void k_rank_features(const double* __restrict__ prev_s, int len, float site,
                                float ltol, float lprev, float lk, float lmaxb,
                                float* __restrict__ f) {
  const int i = threadIdx.x;
  if (i < 32) {
    float v = -20.f;
    if (prev_s && i < len) {
      const double s0 = prev_s[0], si = prev_s[i];
      if (s0 > 0.0 && si > 0.0) v = (float)fmax(-20.0, log10(si / s0));
    }
    f[i] = v;
  } else if (i == 32) {
    f[32] = site;
    f[33] = ltol;
    f[34] = lprev;
    f[35] = lk;
    f[36] = lmaxb;
  }
}

// The QR cap from the network's log2-rank output y: r = clamp(ceil(2^y), 1, k),
// cap = min(k, ceil(margin r) + extra), 0 when it exceeds useful k.
__global__ void k_rank_cap(const float* __restrict__ y, int k, double margin, int extra,
                           double useful, int* __restrict__ out) {
  const double r = fmin((double)k, fmax(1.0, ceil(exp2((double)y[0]))));
  int cap = (int)fmin((double)k, ceil(margin * r) + extra);
  if (cap > useful * k) cap = 0;
  out[0] = cap;
  out[1] = (int)r;
}

}  // namespace

// ---- rank features --------------------------------------------------------
void rank_features(const Ctx& ctx, int k, const sm_strategy& st, float* f) {
  const size_t ns = ctx.prev_s.size();
  const double s0 = ns ? ctx.prev_s[0] : 0.0;
  for (int i = 0; i < 32; ++i) {
    float v = -20.f;
    if (i < (int)ns && s0 > 0.0 && ctx.prev_s[i] > 0.0)
      v = (float)std::max(-20.0, std::log10(ctx.prev_s[i] / s0));
    f[i] = v;
  }
  f[32] = ctx.split_n > 0 ? (float)ctx.split_site / (float)ctx.split_n : 0.5f;
  f[33] = st.tolerance > 0.0 ? (float)std::log10(st.tolerance) : -20.f;
  f[34] = (float)std::log2(1.0 + ctx.prev_rank);
  f[35] = (float)std::log2((double)std::max(1, k));
  f[36] = (float)std::log2((double)std::min(std::max(1, st.max_bond_dimension), 1 << 20));
}

int rank_predict_dev(Ctx& ctx, cudaStream_t st, int k, const sm_strategy& strat, double useful,
                     int* out) {
  if (!ctx.model.loaded) {
    set_error("rank model not set");
    return SM_ERR_VALUE;
  }
  float* x;
  SM_CHECK(ctx.scratch("mlp.infer", (size_t)3 * 4096, &x));
  const float site = ctx.split_n > 0 ? (float)ctx.split_site / (float)ctx.split_n : 0.5f;
  const float ltol = strat.tolerance > 0.0 ? (float)std::log10(strat.tolerance) : -20.f;
  const float lprev = (float)std::log2(1.0 + ctx.prev_rank);
  const float lk = (float)std::log2((double)std::max(1, k));
  const float lmaxb =
      (float)std::log2((double)std::min(std::max(1, strat.max_bond_dimension), 1 << 20));
  k_rank_features<<<1, 64, 0, st>>>(ctx.prev_len_dev > 0 ? ctx.prev_s_dev : nullptr,
                                    ctx.prev_len_dev, site, ltol, lprev, lk, lmaxb, x);
  note_launch();
  float* y = nullptr;
  SM_CHECK(infer(ctx, st, x, 1, x + 4096, &y));
  k_rank_cap<<<1, 1, 0, st>>>(y, k, ctx.cap_margin, ctx.cap_extra, useful, out);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

// Kept rank of a split of size k predicted by the context's model (1..k).
int rank_predict(Ctx& ctx, cudaStream_t st, int k, const sm_strategy& strat, int* out) {
  if (!ctx.model.loaded) {
    set_error("rank model not set");
    return SM_ERR_VALUE;
  }
  float* h = reinterpret_cast<float*>(ctx.pinned) + 4096;  // past the split read-back words
  rank_features(ctx, k, strat, h);
  float* x;
  SM_CHECK(ctx.scratch("mlp.infer", (size_t)3 * 4096, &x));
  SM_CUDA_CHECK(cudaMemcpyAsync(x, h, sizeof(float) * SM_RANK_FEATURES, cudaMemcpyHostToDevice, st));
  float* y = nullptr;
  SM_CHECK(infer(ctx, st, x, 1, x + 4096, &y));
  SM_CUDA_CHECK(cudaMemcpyAsync(h, y, sizeof(float), cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  const double r = std::exp2((double)h[0]);
  *out = (int)std::max(1.0, std::min((double)k, std::ceil(r)));
  return SM_OK;
}

}  // namespace sm

using namespace sm;

static Ctx* mctx(void* c) { return reinterpret_cast<Ctx*>(c); }
static cudaStream_t mst(void* s) { return reinterpret_cast<cudaStream_t>(s); }

extern "C" {

int64_t sm_mlp_param_count(int n_layers, const int* dims) {
  if (check_dims(n_layers, dims) != SM_OK) return -1;
  return (int64_t)param_count(n_layers, dims);
}

int64_t sm_mlp_cache_count(int n_layers, const int* dims, int batch) {
  if (check_dims(n_layers, dims) != SM_OK || batch < 1) return -1;
  int64_t n = 0;
  for (int k = 1; k <= n_layers; ++k) n += 2 * (int64_t)batch * dims[k];
  return n;
}

int sm_mlp_forward(void* ctx, int n_layers, const int* dims, const float* params, const float* X,
                   int batch, float* Y, float* cache, void* stream) {
  if (!ctx) return SM_ERR_VALUE;
  SM_CHECK(check_dims(n_layers, dims));
  if (!params || !X || !Y || !cache || batch < 1) {
    set_error("sm_mlp_forward: null pointer or empty batch");
    return SM_ERR_VALUE;
  }
  cudaStream_t st = mst(stream);
  const float* in = X;
  size_t po = 0, co = 0;
  for (int k = 0; k < n_layers; ++k) {
    const int di = dims[k], dout = dims[k + 1];
    const float* W = params + po;
    const float* b = W + (size_t)dout * di;
    float* Z = cache + co;
    float* A = Z + (size_t)batch * dout;
    SM_CHECK(sgemm(st, 0, 1, batch, dout, di, in, di, W, di, Z, dout));
    const bool hidden = k + 1 < n_layers;
    k_bias_act<<<blocks_for((size_t)batch * dout), 256, 0, st>>>(Z, b, batch, dout,
                                                                 hidden ? A : nullptr);
    note_launch();
    if (!hidden)
      SM_CUDA_CHECK(cudaMemcpyAsync(A, Z, sizeof(float) * batch * dout, cudaMemcpyDeviceToDevice, st));
    in = A;
    po += (size_t)dout * di + dout;
    co += 2 * (size_t)batch * dout;
  }
  SM_CUDA_CHECK(cudaMemcpyAsync(Y, in, sizeof(float) * batch * dims[n_layers],
                                cudaMemcpyDeviceToDevice, st));
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

int sm_mlp_backward(void* ctx, int n_layers, const int* dims, const float* params, const float* X,
                    int batch, const float* cache, const float* dY, float* grads, void* stream) {
  if (!ctx) return SM_ERR_VALUE;
  SM_CHECK(check_dims(n_layers, dims));
  if (!params || !X || !cache || !dY || !grads || batch < 1) {
    set_error("sm_mlp_backward: null pointer or empty batch");
    return SM_ERR_VALUE;
  }
  Ctx& c = *mctx(ctx);
  cudaStream_t st = mst(stream);
  int wmax = 0;
  for (int k = 0; k <= n_layers; ++k) wmax = std::max(wmax, dims[k]);
  float *g0, *g1;
  SM_CHECK(c.scratch("mlp.grad", (size_t)2 * batch * wmax, &g0));
  g1 = g0 + (size_t)batch * wmax;
  std::vector<size_t> po(n_layers), co(n_layers);
  size_t p = 0, q = 0;
  for (int k = 0; k < n_layers; ++k) {
    po[k] = p;
    co[k] = q;
    p += (size_t)dims[k + 1] * dims[k] + dims[k + 1];
    q += 2 * (size_t)batch * dims[k + 1];
  }
  // dZ of the last layer = dY (no activation)
  SM_CUDA_CHECK(cudaMemcpyAsync(g0, dY, sizeof(float) * batch * dims[n_layers],
                                cudaMemcpyDeviceToDevice, st));
  for (int k = n_layers - 1; k >= 0; --k) {
    const int di = dims[k], dout = dims[k + 1];
    const float* W = params + po[k];
    float* gW = grads + po[k];
    float* gb = gW + (size_t)dout * di;
    const float* in = k == 0 ? X : cache + co[k - 1] + (size_t)batch * dims[k];  // A_{k-1}
    SM_CHECK(sgemm(st, 1, 0, dout, di, batch, g0, dout, in, di, gW, di));  // dW = dZ^T X
    k_col_sum<<<(dout + 127) / 128, 128, 0, st>>>(g0, batch, dout, gb);
    note_launch();
    if (k > 0) {
      SM_CHECK(sgemm(st, 0, 0, batch, di, dout, g0, dout, W, di, g1, di));  // dA = dZ W
      const float* Zp = cache + co[k - 1];
      k_gelu_back<<<blocks_for((size_t)batch * di), 256, 0, st>>>(g1, Zp, (size_t)batch * di, g0);
      note_launch();
    }
  }
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

int sm_mse_loss(void* ctx, const float* yhat, const float* y, int batch, float* dyhat, float* loss,
                void* stream) {
  if (!ctx || !yhat || !y || batch < 1) {
    set_error("sm_mse_loss: null pointer or empty batch");
    return SM_ERR_VALUE;
  }
  k_mse<<<1, 256, 0, mst(stream)>>>(yhat, y, batch, dyhat, loss);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

int sm_adam_step(void* ctx, float* p, const float* g, float* m, float* v, int64_t n, float lr,
                 float beta1, float beta2, float eps, int step, void* stream) {
  if (!ctx || !p || !g || !m || !v || n < 1 || step < 1) {
    set_error("sm_adam_step: null pointer, empty array or step < 1");
    return SM_ERR_VALUE;
  }
  const float c1 = 1.f - std::pow(beta1, (float)step), c2 = 1.f - std::pow(beta2, (float)step);
  k_adam<<<blocks_for((size_t)n), 256, 0, mst(stream)>>>(p, g, m, v, (size_t)n, lr, beta1, beta2,
                                                        eps, c1, c2);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

int sm_rank_model_set(void* ctx, int n_layers, const int* dims, const float* params) {
  if (!ctx) return SM_ERR_VALUE;
  Ctx& c = *mctx(ctx);
  if (!params) {  // clear
    c.model.loaded = false;
    return SM_OK;
  }
  SM_CHECK(check_dims(n_layers, dims));
  if (dims[0] != SM_RANK_FEATURES || dims[n_layers] != 1) {
    set_error("sm_rank_model_set: the model maps SM_RANK_FEATURES inputs to 1 output");
    return SM_ERR_VALUE;
  }
  size_t nw = 0, nb = 0;
  for (int k = 0; k < n_layers; ++k) {
    nw += (size_t)dims[k + 1] * dims[k];
    nb += dims[k + 1];
  }
  __nv_bfloat16* w;
  float* b;
  SM_CHECK(c.scratch("rank.w", nw * sizeof(__nv_bfloat16), reinterpret_cast<void**>(&w)));
  SM_CHECK(c.scratch("rank.b", nb, &b));
  size_t po = 0, wo = 0, bo = 0;
  for (int k = 0; k < n_layers; ++k) {
    const size_t n = (size_t)dims[k + 1] * dims[k];
    k_to_bf16<<<blocks_for(n), 256>>>(params + po, n, w + wo);
    note_launch();
    SM_CUDA_CHECK(cudaMemcpy(b + bo, params + po + n, sizeof(float) * dims[k + 1],
                             cudaMemcpyDeviceToDevice));
    po += n + dims[k + 1];
    wo += n;
    bo += dims[k + 1];
  }
  SM_CUDA_CHECK(cudaDeviceSynchronize());
  c.model.loaded = true;
  c.model.layers = n_layers;
  for (int k = 0; k <= n_layers; ++k) c.model.dims[k] = dims[k];
  c.model.w = w;
  c.model.b = b;
  return SM_OK;
}

int sm_rank_features_record(void* ctx, int on) {
  if (!ctx) return SM_ERR_VALUE;
  Ctx& c = *mctx(ctx);
  c.record = on != 0;
  c.rec_x.clear();
  c.rec_y.clear();
  return SM_OK;
}

int sm_rank_features_read(void* ctx, float* X, int* D, int cap, int* count) {
  if (!ctx || !count) return SM_ERR_VALUE;
  Ctx& c = *mctx(ctx);
  const int n = (int)c.rec_y.size();
  *count = n;
  if (X && D) {
    const int m = std::min(n, cap);
    std::memcpy(X, c.rec_x.data(), sizeof(float) * (size_t)m * SM_RANK_FEATURES);
    std::memcpy(D, c.rec_y.data(), sizeof(int) * (size_t)m);
  }
  return SM_OK;
}

int sm_rank_predict(void* ctx, const float* X, int batch, float* out, void* stream) {
  if (!ctx || !X || !out || batch < 1) {
    set_error("sm_rank_predict: null pointer or empty batch");
    return SM_ERR_VALUE;
  }
  Ctx& c = *mctx(ctx);
  if (!c.model.loaded) {
    set_error("sm_rank_predict: no rank model set");
    return SM_ERR_VALUE;
  }
  cudaStream_t st = mst(stream);
  int wmax = 0;
  for (int k = 0; k <= c.model.layers; ++k) wmax = std::max(wmax, c.model.dims[k]);
  float* buf;
  SM_CHECK(c.scratch("mlp.pred", (size_t)3 * batch * wmax, &buf));
  SM_CUDA_CHECK(cudaMemcpyAsync(buf, X, sizeof(float) * batch * c.model.dims[0],
                                cudaMemcpyHostToDevice, st));
  float* y = nullptr;
  SM_CHECK(infer(c, st, buf, batch, buf + (size_t)batch * wmax, &y));
  SM_CUDA_CHECK(cudaMemcpyAsync(out, y, sizeof(float) * batch, cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  return SM_OK;
}

}  // extern "C"
