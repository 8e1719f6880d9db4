// Randomized range finder for the learned split (Halko, Martinsson and Tropp,
// "Finding structure with randomness", SIAM Review 53 (2011), Algorithms 4.1
// and 4.4), real FP64 operands.
//
// For W (kw x l) and a predicted kept rank r, k = r + oversampling:
//   Y = W Omega                       Omega: l x k Gaussian (counter-based, fixed seed)
//   q times: Y <- orth(Y); Y <- W orth(W^T Y)   (subspace iteration)
//   Z = W^T Y                          (l x k)
//   G = Y^T Y = L L^T                  shifted Cholesky (one CTA, blocked)
//   BH = Z L^{-T} = W^T Q              Q = Y L^{-T} spans range(Y) orthonormally
// BH (l x k) holds the action of W on the captured subspace: with
// B = BH^T = U_B S V_B^T, W ~ (Q U_B) S V_B^T, so the rows of U_B^T B are W's
// right singular vectors within the subspace.  The caller factors BH with the
// FP32 cluster kernel (rows of length k instead of l) and refines the result
// against the exact W in FP64, where the exact discarded weight decides
// whether the subspace held everything the truncation keeps.
//
// The shift: with k above W's numerical rank, Y has directions at rounding
// level and G is singular to working precision; the Cholesky factor of
// G + s I (s = 1e-13 tr(G)) stays finite, those directions come out of Q with
// small norm, and the captured directions stay orthonormal to ~s / sigma^2.
#include <algorithm>
#include <cmath>

#include "kernels.cuh"

namespace sm {

namespace {

constexpr int kCholNB = 32;    // panel width
constexpr double kCholShift = 1e-13;

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// X[i] ~ N(0, 1), two per hash pair (Box-Muller on 53-bit uniforms).
__global__ void k_gaussian(double* __restrict__ X, size_t n, unsigned long long seed) {
  const size_t pairs = (n + 1) / 2;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < pairs;
       p += (size_t)gridDim.x * blockDim.x) {
    const unsigned long long h1 = splitmix64(seed ^ (2 * p));
    const unsigned long long h2 = splitmix64(seed ^ (2 * p + 1));
    const double u1 = ((double)(h1 >> 11) + 1.0) * 0x1.0p-53;  // (0, 1]
    const double u2 = (double)(h2 >> 11) * 0x1.0p-53;          // [0, 1)
    const double rad = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    X[2 * p] = rad * c;
    if (2 * p + 1 < n) X[2 * p + 1] = rad * s;
  }
}

// In-place lower Cholesky factor of G + s I (k x k, row-major, lower triangle
// read and written), s = shift_rel * trace(G), right-looking in 32-wide
// panels over the whole GPU (GB300's FP64 rate per SM is low, so no step stays
// on one SM longer than a 32 x 32 block): per panel, k_chol_diag factors the
// diagonal block in one warp, k_chol_panel solves the rows below it (thread
// per row), k_chol_syrk updates the trailing lower triangle in 32 x 32 tiles.
// *status = 1 if a pivot is not positive even after the shift.
__global__ void k_chol_shift(const double* __restrict__ G, int k, double shift_rel,
                             double* __restrict__ shift) {
  __shared__ double red[8];
  double t = 0.0;
  for (int i = threadIdx.x; i < k; i += blockDim.x) t += G[(size_t)i * k + i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    *shift = shift_rel * s;
  }
}

__global__ void k_chol_diag(double* __restrict__ G, int k, int j0, int nb,
                            const double* __restrict__ shift, int* status) {
  constexpr int LD = kCholNB + 1;
  __shared__ double D[kCholNB * LD];
  const int lane = threadIdx.x;  // one warp
  const double sh = *shift;
  for (int c = 0; c < nb; ++c) {
    double v = 0.0;
    if (lane < nb && c <= lane) v = G[(size_t)(j0 + lane) * k + j0 + c] + (lane == c ? sh : 0.0);
    D[lane * LD + c] = v;
  }
  __syncwarp();
  bool bad = false;
  for (int c = 0; c < nb; ++c) {
    if (lane == c) {
      const double d = D[c * LD + c];
      if (!(d > 0.0)) bad = true;
      D[c * LD + c] = d > 0.0 ? sqrt(d) : 1.0;
    }
    __syncwarp();
    const double piv = D[c * LD + c];
    if (lane > c && lane < nb) D[lane * LD + c] /= piv;
    __syncwarp();
    for (int cc = c + 1; cc < nb; ++cc)
      if (lane >= cc && lane < nb) D[lane * LD + cc] -= D[lane * LD + c] * D[cc * LD + c];
    __syncwarp();
  }
  if (lane < nb)
    for (int c = 0; c <= lane; ++c) G[(size_t)(j0 + lane) * k + j0 + c] = D[lane * LD + c];
  if (bad) *status = 1;
}

__global__ void k_chol_panel(double* __restrict__ G, int k, int j0, int nb) {
  constexpr int LD = kCholNB + 1;
  __shared__ double L11[kCholNB * LD];
  for (int e = threadIdx.x; e < kCholNB * kCholNB; e += blockDim.x) {
    const int r = e / kCholNB, c = e % kCholNB;
    L11[r * LD + c] = (r < nb && c <= r) ? G[(size_t)(j0 + r) * k + j0 + c] : 0.0;
  }
  __syncthreads();
  const int i = j0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k) return;
  double* gi = G + (size_t)i * k + j0;
  double x[kCholNB];
#pragma unroll
  for (int c = 0; c < kCholNB; ++c) x[c] = c < nb ? gi[c] : 0.0;
#pragma unroll
  for (int c = 0; c < kCholNB; ++c) {
    if (c < nb) {
      double v = x[c];
#pragma unroll
      for (int t = 0; t < c; ++t) v -= x[t] * L11[c * LD + t];
      x[c] = v / L11[c * LD + c];
    }
  }
#pragma unroll
  for (int c = 0; c < kCholNB; ++c)
    if (c < nb) gi[c] = x[c];
}

__global__ void k_chol_syrk(double* __restrict__ G, int k, int j0, int nb) {
  constexpr int LD = kCholNB + 1;
  __shared__ double Pi[kCholNB * LD], Pc[kCholNB * LD];
  const int r0 = j0 + nb;
  // tile (ti, tc), tc <= ti, from the linear block index
  int ti = (int)((sqrt(8.0 * blockIdx.x + 1.0) - 1.0) * 0.5);
  while ((ti + 1) * (ti + 2) / 2 <= (int)blockIdx.x) ++ti;
  while (ti * (ti + 1) / 2 > (int)blockIdx.x) --ti;
  const int tc = blockIdx.x - ti * (ti + 1) / 2;
  const int i0 = r0 + ti * 32, c0 = r0 + tc * 32;
  for (int e = threadIdx.x; e < 32 * kCholNB; e += blockDim.x) {
    const int r = e / kCholNB, t = e % kCholNB;
    Pi[r * LD + t] = (i0 + r < k && t < nb) ? G[(size_t)(i0 + r) * k + j0 + t] : 0.0;
    Pc[r * LD + t] = (c0 + r < k && t < nb) ? G[(size_t)(c0 + r) * k + j0 + t] : 0.0;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
    const int r = e / 32, c = e % 32;
    const int i = i0 + r, cc = c0 + c;
    if (i >= k || cc > i) continue;
    double acc = 0.0;
#pragma unroll 8
    for (int t = 0; t < nb; ++t) acc = fma(Pi[r * LD + t], Pc[c * LD + t], acc);
    G[(size_t)i * k + cc] -= acc;
  }
}

// X (rows x k, row-major) <- X L^{-T} for the lower factor L (k x k): each row
// x solves q L^T = x by forward substitution, q_c = (x_c - sum_{t<c} q_t L_ct)
// / L_cc.  One warp per row, lanes split the sums; the row in shared memory.
constexpr int kTrsmWarps = 8;
__global__ void __launch_bounds__(32 * kTrsmWarps) k_trsm_lt(double* __restrict__ X, int rows,
                                                             int k, const double* __restrict__ L) {
  extern __shared__ double sm_q[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int row = blockIdx.x * kTrsmWarps + warp;
  if (row >= rows) return;
  double* q = sm_q + (size_t)warp * k;
  double* x = X + (size_t)row * k;
  for (int c = lane; c < k; c += 32) q[c] = x[c];
  __syncwarp();
  for (int c = 0; c < k; ++c) {
    const double* lc = L + (size_t)c * k;
    double acc = 0.0;
    for (int t = lane; t < c; t += 32) acc = fma(q[t], lc[t], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) q[c] = (q[c] - acc) / lc[c];
    __syncwarp();
  }
  for (int c = lane; c < k; c += 32) x[c] = q[c];
}

// L = chol(G + s I) in place, then X (rows x k) <- X L^{-T}.
int chol_solve(Ctx& ctx, cudaStream_t st, double* G, int k, double* X, int rows, int* status) {
  double* shift;
  SM_CHECK(ctx.scratch("rf.shift", 1, &shift));
  k_chol_shift<<<1, 256, 0, st>>>(G, k, kCholShift, shift);
  note_launch();
  for (int j0 = 0; j0 < k; j0 += kCholNB) {
    const int nb = std::min(kCholNB, k - j0);
    const int nr = k - j0 - nb;
    k_chol_diag<<<1, 32, 0, st>>>(G, k, j0, nb, shift, status);
    note_launch();
    if (nr > 0) {
      k_chol_panel<<<(nr + 127) / 128, 128, 0, st>>>(G, k, j0, nb);
      const int nt = (nr + 31) / 32;
      k_chol_syrk<<<nt * (nt + 1) / 2, 256, 0, st>>>(G, k, j0, nb);
      note_launch(2);
    }
  }
  const size_t tsmem = sizeof(double) * (size_t)kTrsmWarps * k;
  if (tsmem > 48 * 1024) SM_CHECK(raise_smem_limit(k_trsm_lt, tsmem));
  k_trsm_lt<<<(rows + kTrsmWarps - 1) / kTrsmWarps, 32 * kTrsmWarps, tsmem, st>>>(X, rows, k, G);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

}  // namespace

int range_finder_max_k() { return 640; }

int range_finder_bh(Ctx& ctx, cudaStream_t st, const double* A, int m, int n, bool want_u, int k,
                    int power_iters, double* BH, int* status) {
  // W = A^T (kw = n, l = m) when want_u, else W = A (kw = m, l = n)
  const int kw = want_u ? n : m;
  const int l = want_u ? m : n;
  if (k < 1 || k > std::min(range_finder_max_k(), std::min(kw, l))) {
    set_error("range finder: k out of range");
    return SM_ERR_VALUE;
  }
  double *Om, *Y, *Gs;
  SM_CHECK(ctx.scratch("rf.omega", (size_t)l * k, &Om));
  SM_CHECK(ctx.scratch("rf.Y", (size_t)kw * k, &Y));
  SM_CHECK(ctx.scratch("rf.G", (size_t)k * k, &Gs));
  SM_CUDA_CHECK(cudaMemsetAsync(status, 0, sizeof(int), st));
  {
    const size_t total = (size_t)l * k;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((total / 2 + 255) / 256, 1024));
    k_gaussian<<<blocks, 256, 0, st>>>(Om, total, 0x5EE4A5ull * 1000003ull + (unsigned)k);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
  }
  // W X for an l x k X (into kw x k) and W^T X for a kw x k X (into l x k): the
  // subspace iterations' products at FP32 accuracy (3xTF32 on the tensor
  // cores), the products that define the final Y and BH FP64-accurate (an FP32
  // Y would carry directions outside W's range at 1e-7 of |Y|)
  auto w_times = [&](const double* X, double* out, bool fp64) -> int {
    if (want_u) {
      if (fp64) return gemm_ctx<double>(ctx, st, SM_OP_T, SM_OP_N, n, k, m, 1.0, A, n, X, k, 0.0, out, k);
      return gemm_ctx_f32<double>(ctx, st, SM_OP_T, SM_OP_N, n, k, m, 1.0, A, n, X, k, 0.0, out, k);
    }
    if (fp64) return gemm_ctx<double>(ctx, st, SM_OP_N, SM_OP_N, m, k, n, 1.0, A, n, X, k, 0.0, out, k);
    return gemm_ctx_f32<double>(ctx, st, SM_OP_N, SM_OP_N, m, k, n, 1.0, A, n, X, k, 0.0, out, k);
  };
  auto wt_times = [&](const double* X, double* out, bool fp64) -> int {
    if (want_u) {
      if (fp64) return gemm_ctx<double>(ctx, st, SM_OP_N, SM_OP_N, m, k, n, 1.0, A, n, X, k, 0.0, out, k);
      return gemm_ctx_f32<double>(ctx, st, SM_OP_N, SM_OP_N, m, k, n, 1.0, A, n, X, k, 0.0, out, k);
    }
    if (fp64) return gemm_ctx<double>(ctx, st, SM_OP_T, SM_OP_N, n, k, m, 1.0, A, n, X, k, 0.0, out, k);
    return gemm_ctx_f32<double>(ctx, st, SM_OP_T, SM_OP_N, n, k, m, 1.0, A, n, X, k, 0.0, out, k);
  };
  auto gram = [&](const double* X, int rows) -> int {
    return gemm_ctx<double>(ctx, st, SM_OP_T, SM_OP_N, k, k, rows, 1.0, X, k, X, k, 0.0, Gs, k);
  };
  SM_CHECK(w_times(Om, Y, power_iters == 0));
  for (int it = 0; it < power_iters; ++it) {
    SM_CHECK(gram(Y, kw));
    SM_CHECK(chol_solve(ctx, st, Gs, k, Y, kw, status));  // Y <- orth(Y)
    SM_CHECK(wt_times(Y, BH, false));
    SM_CHECK(gram(BH, l));
    SM_CHECK(chol_solve(ctx, st, Gs, k, BH, l, status));  // W^T Y <- orth(W^T Y)
    SM_CHECK(w_times(BH, Y, it + 1 == power_iters));
  }
  // BH = W^T Y L^{-T} with L = chol(Y^T Y)
  SM_CHECK(wt_times(Y, BH, true));
  SM_CHECK(gram(Y, kw));
  return chol_solve(ctx, st, Gs, k, BH, l, status);
}

}  // namespace sm
