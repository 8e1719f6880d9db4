// FP64 / complex128 GEMM for the contractions of the sweep (row-major).
//
//   C[M,N] = alpha * op(A)[M,K] * op(B)[K,N] + beta * C
//
// op = N (as stored), T (transpose) or C (conjugate transpose), the three
// GemmOrder flags of the reference (cython/gemm.pxi:17-20, :21-122).  GB300
// runs FP64 on the CUDA cores only, so this is a shared-memory tiled SIMT
// kernel: 64x64 output tile per CTA, 16-deep K slices, 256 threads holding a
// 4x4 register tile each; the FP64 pipe is the bound, not HBM (operands are
// re-read from L2 at most M/64 + N/64 times).  When the output has fewer
// tiles than the GPU has SMs (the 256..768-sized contractions of a sweep give
// 16-150 tiles), the K range is split over blockIdx.z: each slice writes its
// partial tile to a workspace and a second kernel sums the slices in a fixed
// order (deterministic) and applies alpha / beta.
#include <algorithm>

#include "kernels.cuh"

namespace sm {

namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

__device__ __forceinline__ double shfl_xor_T(double v, int o) {
  return __shfl_xor_sync(0xffffffffu, v, o);
}
__device__ __forceinline__ cplx shfl_xor_T(cplx v, int o) {
  return cplx{__shfl_xor_sync(0xffffffffu, v.re, o), __shfl_xor_sync(0xffffffffu, v.im, o)};
}

template <typename T>
__device__ __forceinline__ T load_op(const T* p, int op) {
  T v = __ldg(p);
  return op == SM_OP_C ? S<T>::conj(v) : v;
}
template <>
__device__ __forceinline__ cplx load_op<cplx>(const cplx* p, int op) {
  const double2 v = __ldg(reinterpret_cast<const double2*>(p));
  return op == SM_OP_C ? cplx{v.x, -v.y} : cplx{v.x, v.y};
}

template <typename T>
__global__ void __launch_bounds__(NT) k_gemm(int opA, int opB, int M, int N, int K, T alpha,
                                             const T* __restrict__ A, int lda,
                                             const T* __restrict__ B, int ldb, T beta,
                                             T* __restrict__ C, int ldc, int kchunk,
                                             T* __restrict__ part) {
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = S<T>::zero();

  const int kbeg = blockIdx.z * kchunk;
  const int kend = min(K, kbeg + kchunk);
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int e = 0; e < (BM * BK) / NT; ++e) {
      const int idx = tid + e * NT;
      int mm, kk;
      if (opA == SM_OP_N) { mm = idx / BK; kk = idx % BK; }
      else                { kk = idx / BM; mm = idx % BM; }
      const int gm = m0 + mm, gk = k0 + kk;
      T v = S<T>::zero();
      if (gm < M && gk < kend)
        v = opA == SM_OP_N ? load_op(A + (size_t)gm * lda + gk, opA)
                           : load_op(A + (size_t)gk * lda + gm, opA);
      As[kk][mm] = v;
    }
#pragma unroll
    for (int e = 0; e < (BN * BK) / NT; ++e) {
      const int idx = tid + e * NT;
      int nn, kk;
      if (opB == SM_OP_N) { kk = idx / BN; nn = idx % BN; }
      else                { nn = idx / BK; kk = idx % BK; }
      const int gn = n0 + nn, gk = k0 + kk;
      T v = S<T>::zero();
      if (gn < N && gk < kend)
        v = opB == SM_OP_N ? load_op(B + (size_t)gk * ldb + gn, opB)
                           : load_op(B + (size_t)gn * ldb + gk, opB);
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = S<T>::fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  if (part) {
    T* p = part + (size_t)blockIdx.z * M * N;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int gm = m0 + ty + 16 * i;
      if (gm >= M) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int gn = n0 + tx + 16 * j;
        if (gn < N) p[(size_t)gm * N + gn] = acc[i][j];
      }
    }
    return;
  }
  const bool use_beta = S<T>::abs2(beta) != 0.0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      T* c = C + (size_t)gm * ldc + gn;
      T v = alpha * acc[i][j];
      if (use_beta) v = S<T>::fma(beta, *c, v);
      *c = v;
    }
  }
}

// C = alpha * sum_z part[z] + beta * C, slices summed in order z = 0, 1, ...
// Small products (M N K below 2 Mi multiply-adds: the chain-end
// contractions and the small splits' refinements): one thread per output
// element, blocks of 64 threads along N so that even a 64 x 64 output spreads
// over 64 SMs; GB300's FP64 rate per SM (~2 FMA per cycle) makes spreading the
// work, not reusing it, what matters at these sizes.
template <typename T>
__global__ void __launch_bounds__(64) k_gemm_small(int opA, int opB, int M, int N, int K, T alpha,
                                                   const T* __restrict__ A, int lda,
                                                   const T* __restrict__ B, int ldb, T beta,
                                                   T* __restrict__ C, int ldc) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y;
  if (n >= N) return;
  T acc = S<T>::zero();
  for (int k = 0; k < K; ++k) {
    const T a = load_op(opA == SM_OP_N ? A + (size_t)m * lda + k : A + (size_t)k * lda + m, opA);
    const T b = load_op(opB == SM_OP_N ? B + (size_t)k * ldb + n : B + (size_t)n * ldb + k, opB);
    acc = S<T>::fma(a, b, acc);
  }
  T* c = C + (size_t)m * ldc + n;
  const bool zero_beta = S<T>::abs2(beta) == 0.0;
  *c = zero_beta ? alpha * acc : alpha * acc + beta * *c;
}

// Matrix-vector shapes (N = 1, or M = 1): the Lanczos projections and norms.
// N = 1, op(A) rows contiguous (op N): block (m, kb) sums K range kb of row m
// into part[m * nkb + kb]; k_gemv_final adds the partials in order.
template <typename T>
__global__ void k_gemv_rows(int opB, const T* __restrict__ A, int lda, const T* __restrict__ B,
                            int ldb, int K, int kchunk, T* __restrict__ part) {
  __shared__ T red[32];
  const int m = blockIdx.x, kb = blockIdx.y;
  const int k0 = kb * kchunk, k1 = min(K, k0 + kchunk);
  T acc = S<T>::zero();
  for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    const T b = load_op(opB == SM_OP_N ? B + (size_t)k * ldb : B + k, opB);
    acc = S<T>::fma(A[(size_t)m * lda + k], b, acc);
  }
  for (int o = 16; o > 0; o >>= 1) acc = acc + shfl_xor_T(acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    T t = S<T>::zero();
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = t + red[w];
    part[(size_t)m * gridDim.y + kb] = t;
  }
}

template <typename T>
__global__ void k_gemv_final(int M, int nkb, const T* __restrict__ part, T alpha, T beta,
                             T* __restrict__ C, int ldc) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  T acc = S<T>::zero();
  for (int kb = 0; kb < nkb; ++kb) acc = acc + part[(size_t)m * nkb + kb];
  T* c = C + (size_t)m * ldc;
  *c = S<T>::abs2(beta) == 0.0 ? alpha * acc : alpha * acc + beta * *c;
}

// N = 1 with op(A) = A^T / A^H (A stored K x M) or M = 1: one thread per output
// element, the K loop coalesced across threads.
template <typename T>
__global__ void k_gemv_cols(int opA, int opB, int M, int N, int K, T alpha,
                            const T* __restrict__ A, int lda, const T* __restrict__ B, int ldb,
                            T beta, T* __restrict__ C, int ldc) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)M * N) return;
  const int m = (int)(e / N), n = (int)(e % N);
  T acc = S<T>::zero();
  for (int k = 0; k < K; ++k) {
    const T a = load_op(opA == SM_OP_N ? A + (size_t)m * lda + k : A + (size_t)k * lda + m, opA);
    const T b = load_op(opB == SM_OP_N ? B + (size_t)k * ldb + n : B + (size_t)n * ldb + k, opB);
    acc = S<T>::fma(a, b, acc);
  }
  T* c = C + (size_t)m * ldc + n;
  *c = S<T>::abs2(beta) == 0.0 ? alpha * acc : alpha * acc + beta * *c;
}

template <typename T>
__global__ void k_splitk_reduce(int M, int N, int nz, const T* __restrict__ part, T alpha, T beta,
                                T* __restrict__ C, int ldc) {
  const bool use_beta = S<T>::abs2(beta) != 0.0;
  const size_t mn = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < mn;
       e += (size_t)gridDim.x * blockDim.x) {
    T acc = part[e];
    for (int z = 1; z < nz; ++z) acc = acc + part[(size_t)z * mn + e];
    const int gm = (int)(e / N), gn = (int)(e % N);
    T* c = C + (size_t)gm * ldc + gn;
    T v = alpha * acc;
    if (use_beta) v = S<T>::fma(beta, *c, v);
    *c = v;
  }
}

// ---- FP32-arithmetic variant (contractions of the mixed forms) --------------
// Same tiling as k_gemm; operands are rounded to FP32 (complex: two FP32) when
// staged in shared memory and the products accumulate in FP32; alpha, beta
// and the output stay FP64.  Relative error ~1e-7 |A||B| per entry.
template <typename T> struct C32;
template <> struct C32<double> {
  using type = float;
  __device__ static float from(double x) { return (float)x; }
  __device__ static double to(float x) { return (double)x; }
  __device__ static float zero() { return 0.f; }
  __device__ static float fma(float a, float b, float c) { return fmaf(a, b, c); }
};
template <> struct C32<cplx> {
  using type = float2;
  __device__ static float2 from(cplx x) { return make_float2((float)x.re, (float)x.im); }
  __device__ static cplx to(float2 x) { return cplx{(double)x.x, (double)x.y}; }
  __device__ static float2 zero() { return make_float2(0.f, 0.f); }
  __device__ static float2 fma(float2 a, float2 b, float2 c) {
    return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
  }
};

template <typename T>
__global__ void __launch_bounds__(NT) k_gemm32(int opA, int opB, int M, int N, int K, T alpha,
                                               const T* __restrict__ A, int lda,
                                               const T* __restrict__ B, int ldb, T beta,
                                               T* __restrict__ C, int ldc, int kchunk,
                                               T* __restrict__ part) {
  using F = typename C32<T>::type;
  __shared__ F As[BK][BM + 1];
  __shared__ F Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  F acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = C32<T>::zero();
  const int kbeg = blockIdx.z * kchunk;
  const int kend = min(K, kbeg + kchunk);
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int e = 0; e < (BM * BK) / NT; ++e) {
      const int idx = tid + e * NT;
      int mm, kk;
      if (opA == SM_OP_N) { mm = idx / BK; kk = idx % BK; }
      else                { kk = idx / BM; mm = idx % BM; }
      const int gm = m0 + mm, gk = k0 + kk;
      T v = S<T>::zero();
      if (gm < M && gk < kend)
        v = opA == SM_OP_N ? load_op(A + (size_t)gm * lda + gk, opA)
                           : load_op(A + (size_t)gk * lda + gm, opA);
      As[kk][mm] = C32<T>::from(v);
    }
#pragma unroll
    for (int e = 0; e < (BN * BK) / NT; ++e) {
      const int idx = tid + e * NT;
      int nn, kk;
      if (opB == SM_OP_N) { kk = idx / BN; nn = idx % BN; }
      else                { nn = idx / BK; kk = idx % BK; }
      const int gn = n0 + nn, gk = k0 + kk;
      T v = S<T>::zero();
      if (gn < N && gk < kend)
        v = opB == SM_OP_N ? load_op(B + (size_t)gk * ldb + gn, opB)
                           : load_op(B + (size_t)gn * ldb + gk, opB);
      Bs[kk][nn] = C32<T>::from(v);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      F a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = C32<T>::fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  const bool use_beta = S<T>::abs2(beta) != 0.0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      const T r = C32<T>::to(acc[i][j]);
      if (part) {
        part[(size_t)blockIdx.z * M * N + (size_t)gm * N + gn] = r;
      } else {
        T* c = C + (size_t)gm * ldc + gn;
        T v = alpha * r;
        if (use_beta) v = S<T>::fma(beta, *c, v);
        *c = v;
      }
    }
  }
}

}  // namespace

template <typename T>
int gemm(cudaStream_t st, int opA, int opB, int M, int N, int K, T alpha, const T* A, int lda,
         const T* B, int ldb, T beta, T* C, int ldc) {
  if (M < 0 || N < 0 || K < 0) {
    set_error("gemm: negative size");
    return SM_ERR_VALUE;
  }
  if (M == 0 || N == 0) return SM_OK;
  if (K == 0) {
    // C = beta C  (or zero)
    return scale_matrix<T>(st, M, N, beta, C, ldc);
  }
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
  if (grid.y > 65535) {
    set_error("gemm: M too large");
    return SM_ERR_VALUE;
  }
  k_gemm<T><<<grid, NT, 0, st>>>(opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, K,
                                 nullptr);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

// Split-K variant: `nz` K slices (nz > 1) through the workspace `part`
// (nz * M * N elements).
template <typename T>
int gemm_splitk(cudaStream_t st, int opA, int opB, int M, int N, int K, T alpha, const T* A,
                int lda, const T* B, int ldb, T beta, T* C, int ldc, int nz, T* part) {
  const int kchunk = ((K + nz - 1) / nz + BK - 1) / BK * BK;
  nz = (K + kchunk - 1) / kchunk;
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, nz);
  k_gemm<T><<<grid, NT, 0, st>>>(opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk,
                                 part);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  const size_t mn = (size_t)M * N;
  const int blocks = (int)std::min<size_t>((mn + 255) / 256, 4096);
  k_splitk_reduce<T><<<blocks, 256, 0, st>>>(M, N, nz, part, alpha, beta, C, ldc);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

// K slices for an M x N x K product on `sms` SMs: enough CTAs for about two
// waves, each slice at least 64 deep; 1 = no split.
int splitk_slices(int M, int N, int K, int sms) {
  const long tiles = (long)((M + BM - 1) / BM) * ((N + BN - 1) / BN);
  if (tiles >= sms || K < 128) return 1;
  const long want = (2L * sms + tiles - 1) / tiles;
  return (int)std::max(1L, std::min({want, (long)(K / 64), 32L}));
}

template <typename T>
int gemm_ctx(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, T alpha, const T* A,
             int lda, const T* B, int ldb, T beta, T* C, int ldc) {
  return gemm_ctx_sel(ctx, st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, true);
}

template <typename T>
int gemm_ctx_sel(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, T alpha,
                 const T* A, int lda, const T* B, int ldb, T beta, T* C, int ldc, bool allow_tc) {
  if (M == 0 || N == 0 || K == 0) return gemm<T>(st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  if constexpr (sizeof(T) == sizeof(double)) {
    // mixed forms: FP64-accurate products on the BF16 tensor cores
    if (allow_tc && ctx.precision != SM_PRECISION_FP64 && ctx.fp64_tc &&
        gemm_oz_eligible(M, N, K)) {
      ctx.stats.gemm_oz_launches += 1;
      ctx.stats.gemm_oz_flops += 2.0 * M * N * K;
      if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
      SM_CHECK(gemm_oz(ctx, st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc));
      if (ctx.timing) {
        SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
        SM_CUDA_CHECK(cudaEventSynchronize(ctx.ev1));
        float ms = 0.f;
        SM_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
        ctx.stats.gemm_oz_ms += ms;
      }
      return SM_OK;
    }
  } else {
    // mixed forms, complex operands: three real FP64-accurate products (3M)
    if (allow_tc && ctx.precision != SM_PRECISION_FP64 && ctx.fp64_tc &&
        gemm_cplx_oz_eligible(M, N, K)) {
      ctx.stats.gemm_oz_launches += 3;
      ctx.stats.gemm_oz_flops += 6.0 * M * N * K;
      if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
      SM_CHECK(gemm_cplx_3m(ctx, st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc,
                            true));
      if (ctx.timing) {
        SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
        SM_CUDA_CHECK(cudaEventSynchronize(ctx.ev1));
        float ms = 0.f;
        SM_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
        ctx.stats.gemm_oz_ms += ms;
      }
      return SM_OK;
    }
  }
  ctx.stats.gemm_launches += 1;
  ctx.stats.gemm_flops += 2.0 * M * N * K * (sizeof(T) == sizeof(double) ? 1.0 : 4.0);
  if (N == 1 && opA == SM_OP_N && K >= 1024 && M <= 65535) {
    // long dot products: K split over blocks, partials summed in order
    const int nkb = std::min(64, (K + 4095) / 4096);
    const int kchunk = (K + nkb - 1) / nkb;
    T* part;
    SM_CHECK(ctx.scratch("gemv.part", (size_t)M * nkb, &part));
    k_gemv_rows<T><<<dim3(M, nkb), 256, 0, st>>>(opB, A, lda, B, ldb, K, kchunk, part);
    k_gemv_final<T><<<(M + 127) / 128, 128, 0, st>>>(M, nkb, part, alpha, beta, C, ldc);
    note_launch(2);
    SM_CUDA_CHECK(cudaGetLastError());
    return SM_OK;
  }
  if ((N == 1 || M == 1) && K <= 4096) {
    const size_t mn = (size_t)M * N;
    k_gemv_cols<T><<<(unsigned)((mn + 127) / 128), 128, 0, st>>>(opA, opB, M, N, K, alpha, A, lda,
                                                                   B, ldb, beta, C, ldc);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    return SM_OK;
  }
  if ((double)M * N * K <= 2.0 * 1024 * 1024 && M <= 65535) {
    if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
    k_gemm_small<T><<<dim3((N + 63) / 64, M), 64, 0, st>>>(opA, opB, M, N, K, alpha, A, lda, B, ldb,
                                                           beta, C, ldc);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    if (ctx.timing) {
      SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
      SM_CUDA_CHECK(cudaEventSynchronize(ctx.ev1));
      float ms = 0.f;
      SM_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
      ctx.stats.gemm_ms += ms;
    }
    return SM_OK;
  }
  const int nz = splitk_slices(M, N, K, std::max(1, ctx.num_sms));
  T* part = nullptr;
  if (nz > 1) SM_CHECK(ctx.scratch("gemm.splitk", (size_t)nz * M * N, &part));
  auto run = [&]() -> int {
    if (nz > 1)
      return gemm_splitk<T>(st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, nz, part);
    return gemm<T>(st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  };
  if (!ctx.timing) return run();
  SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
  SM_CHECK(run());
  SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
  SM_CUDA_CHECK(cudaEventSynchronize(ctx.ev1));
  float ms = 0.f;
  SM_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
  ctx.stats.gemm_ms += ms;
  return SM_OK;
}

template <typename T>
int gemm_ctx_f32(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, T alpha,
                 const T* A, int lda, const T* B, int ldb, T beta, T* C, int ldc) {
  if (M == 0 || N == 0 || K == 0) return gemm<T>(st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  ctx.stats.gemm32_launches += 1;
  ctx.stats.gemm32_flops += 2.0 * M * N * K * (sizeof(T) == sizeof(double) ? 1.0 : 4.0);
  if constexpr (sizeof(T) == sizeof(double)) {
    if (gemm_tc_eligible(M, N, K)) {
      if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
      SM_CHECK(gemm_tc(ctx, st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc));
      ctx.stats.gemm_tc_launches += 1;
      ctx.stats.gemm_tc_flops += 2.0 * M * N * K;
      if (ctx.timing) {
        SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
        SM_CUDA_CHECK(cudaEventSynchronize(ctx.ev1));
        float ms = 0.f;
        SM_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
        ctx.stats.gemm32_ms += ms;
        ctx.stats.gemm_tc_ms += ms;
      }
      return SM_OK;
    }
  } else {
    // complex operands: three real 3xTF32 products on split planes (3M)
    if (gemm_cplx_tc_eligible(M, N, K)) {
      if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
      SM_CHECK(gemm_cplx_3m(ctx, st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc,
                            false));
      ctx.stats.gemm_tc_launches += 3;
      ctx.stats.gemm_tc_flops += 6.0 * M * N * K;
      if (ctx.timing) {
        SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
        SM_CUDA_CHECK(cudaEventSynchronize(ctx.ev1));
        float ms = 0.f;
        SM_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
        ctx.stats.gemm32_ms += ms;
        ctx.stats.gemm_tc_ms += ms;
      }
      return SM_OK;
    }
  }
  // FP32 runs 64x the FP64 rate: split K only when the output has very few tiles
  const int nz = splitk_slices(M, N, K, std::max(1, ctx.num_sms) / 2);
  T* part = nullptr;
  if (nz > 1) SM_CHECK(ctx.scratch("gemm.splitk", (size_t)nz * M * N, &part));
  const int kchunk = nz > 1 ? ((K + nz - 1) / nz + BK - 1) / BK * BK : K;
  const int nzz = nz > 1 ? (K + kchunk - 1) / kchunk : 1;
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, nzz);
  if (grid.y > 65535) {
    set_error("gemm: M too large");
    return SM_ERR_VALUE;
  }
  if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
  k_gemm32<T><<<grid, NT, 0, st>>>(opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk,
                                   nzz > 1 ? part : nullptr);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  if (nzz > 1) {
    const size_t mn = (size_t)M * N;
    const int blocks = (int)std::min<size_t>((mn + 255) / 256, 4096);
    k_splitk_reduce<T><<<blocks, 256, 0, st>>>(M, N, nzz, part, alpha, beta, C, ldc);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
  }
  if (ctx.timing) {
    SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
    SM_CUDA_CHECK(cudaEventSynchronize(ctx.ev1));
    float ms = 0.f;
    SM_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
    ctx.stats.gemm32_ms += ms;
  }
  return SM_OK;
}

template int gemm_ctx_f32<double>(Ctx&, cudaStream_t, int, int, int, int, int, double,
                                  const double*, int, const double*, int, double, double*, int);
template int gemm_ctx_f32<cplx>(Ctx&, cudaStream_t, int, int, int, int, int, cplx, const cplx*,
                                int, const cplx*, int, cplx, cplx*, int);

template int gemm_ctx<double>(Ctx&, cudaStream_t, int, int, int, int, int, double, const double*,
                              int, const double*, int, double, double*, int);
template int gemm_ctx_sel<double>(Ctx&, cudaStream_t, int, int, int, int, int, double,
                                  const double*, int, const double*, int, double, double*, int,
                                  bool);
template int gemm_ctx_sel<cplx>(Ctx&, cudaStream_t, int, int, int, int, int, cplx, const cplx*,
                                int, const cplx*, int, cplx, cplx*, int, bool);
template int gemm_ctx<cplx>(Ctx&, cudaStream_t, int, int, int, int, int, cplx, const cplx*, int,
                            const cplx*, int, cplx, cplx*, int);

template int gemm<double>(cudaStream_t, int, int, int, int, int, double, const double*, int,
                          const double*, int, double, double*, int);
template int gemm<cplx>(cudaStream_t, int, int, int, int, int, cplx, const cplx*, int,
                        const cplx*, int, cplx, cplx*, int);

}  // namespace sm
