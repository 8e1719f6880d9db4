// Two-site effective-Hamiltonian matvec of DMRG (the reference's
// QuadraticForm.two_site_operator._matvec, operators/quadratic.py:187-237):
//
//   out[a, ko, lo, g] = sum_{b,c,d,k,l,f} L[a, c, b] v[b, k, l, f] H[c, ko, k, lo, l, d] R[g, d, f]
//
// with L (bra bond a, MPO bond c, ket bond b), the two-site MPO H = O_i O_{i+1}
// (_contract_last_and_first) and R (bra g, MPO d, ket f).  Three steps:
//   1. X1[(a,c), (k,l,f)] = L[(a,c), b] v[b, (k,l,f)]            GEMM, 2 a c b k l f flops
//   2. X2[a, ko, lo, d, f] = sum_{c,k,l} X1[a,c,k,l,f] H[c,ko,k,lo,l,d]
//                                                               k_h12_apply, 2 a f (c k l)(ko lo d)
//   3. out[(a,ko,lo), g] = X2[(a,ko,lo), (d,f)] R[g, (d,f)]^T   GEMM reading R in place (op T)
// At chi = 256, D = 5, d = 2: 671 + 52 + 671 MFLOP.  The precision argument
// picks the products: FP64 SIMT, FP64-accurate on the BF16 tensor cores,
// FP32-accurate 3xTF32, or one BF16 product with FP32 accumulation (the
// precision pattern of the DMRG configuration); complex operands use the SIMT
// kernels (FP64, or FP32 for the two reduced precisions).
#include <algorithm>

#include "kernels.cuh"

namespace sm {

namespace {

// X2[a][ko][lo][dd][f] = sum_{c,k,l} X1[a][c][k][l][f] H[c][ko][k][lo][l][dd].
// One thread per (a, f), lanes along f (coalesced reads of X1 and writes of
// X2); H (c p1 p1 p2 p2 e entries) in shared memory.
// Acc is the accumulation type (T).
template <typename T, typename Acc>
__global__ void k_h12_apply(const T* __restrict__ X1, const T* __restrict__ H, int A, int Cc,
                            int p1, int p2, int E, int F, T* __restrict__ X2) {
  extern __shared__ unsigned char sraw[];
  T* Hs = reinterpret_cast<T*>(sraw);
  const int nh = Cc * p1 * p1 * p2 * p2 * E;
  for (int i = threadIdx.x + blockDim.x * threadIdx.y; i < nh; i += blockDim.x * blockDim.y)
    Hs[i] = H[i];
  __syncthreads();
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int a = blockIdx.y * blockDim.y + threadIdx.y;
  if (f >= F || a >= A) return;
  const size_t sx = (size_t)F;  // stride of l in X1
  const T* x = X1 + (size_t)a * Cc * p1 * p2 * F + f;
  T* out = X2 + (size_t)a * p1 * p2 * E * F + f;
  for (int ko = 0; ko < p1; ++ko)
    for (int lo = 0; lo < p2; ++lo)
      for (int dd = 0; dd < E; ++dd) {
        Acc acc{};
        for (int c = 0; c < Cc; ++c)
          for (int k = 0; k < p1; ++k)
            for (int l = 0; l < p2; ++l) {
              const T h = Hs[((((c * p1 + ko) * p1 + k) * p2 + lo) * p2 + l) * E + dd];
              if (S<T>::abs2(h) == 0.0) continue;  // zero blocks of the MPO (warp-uniform)
              const T xv = x[(((size_t)c * p1 + k) * p2 + l) * sx];
              if constexpr (sizeof(Acc) == sizeof(T)) acc = S<T>::fma(h, xv, acc);
              else acc = fmaf((float)S<T>::real(h), (float)S<T>::real(xv), acc);
            }
        if constexpr (sizeof(Acc) == sizeof(T)) out[(((size_t)ko * p2 + lo) * E + dd) * F] = acc;
        else out[(((size_t)ko * p2 + lo) * E + dd) * F] = S<T>::from_real((double)acc);
      }
}

template <typename T>
int product(Ctx& ctx, cudaStream_t st, int precision, int opA, int opB, int M, int N, int K,
            const T* A, int lda, const T* B, int ldb, T* C, int ldc) {
  const T one = S<T>::one(), zero = S<T>::zero();
  if constexpr (sizeof(T) == sizeof(double)) {
    if (precision == SM_MATVEC_FP64TC && gemm_oz_eligible(M, N, K)) {
      ctx.stats.gemm_oz_launches += 1;
      ctx.stats.gemm_oz_flops += 2.0 * M * N * K;
      return gemm_oz(ctx, st, opA, opB, M, N, K, one, A, lda, B, ldb, zero, C, ldc);
    }
    if ((precision == SM_MATVEC_TF32X3 || precision == SM_MATVEC_BF16) &&
        gemm_tc_eligible(M, N, K)) {
      ctx.stats.gemm_tc_launches += 1;
      ctx.stats.gemm_tc_flops += 2.0 * M * N * K;
      return gemm_tc(ctx, st, opA, opB, M, N, K, one, A, lda, B, ldb, zero, C, ldc,
                     precision == SM_MATVEC_BF16);
    }
  }
  if (precision == SM_MATVEC_TF32X3 || precision == SM_MATVEC_BF16)
    return gemm_ctx_f32<T>(ctx, st, opA, opB, M, N, K, one, A, lda, B, ldb, zero, C, ldc);
  return gemm_ctx_sel<T>(ctx, st, opA, opB, M, N, K, one, A, lda, B, ldb, zero, C, ldc, false);
}

}  // namespace

template <typename T>
int two_site_matvec(Ctx& ctx, cudaStream_t st, int a, int c, int b, int p1, int p2, int e, int g,
                    int f, const T* L, const T* H, const T* R, const T* v, T* out, int precision) {
  T *X1, *X2;
  SM_CHECK(ctx.scratch("mv.X1", (size_t)a * c * p1 * p2 * f, &X1));
  SM_CHECK(ctx.scratch("mv.X2", (size_t)a * p1 * p2 * e * f, &X2));
  SM_CHECK(product<T>(ctx, st, precision, SM_OP_N, SM_OP_N, a * c, p1 * p2 * f, b, L, b, v,
                      p1 * p2 * f, X1, p1 * p2 * f));
  const size_t hs = sizeof(T) * (size_t)c * p1 * p1 * p2 * p2 * e;
  const dim3 blk(32, 8), grd((f + 31) / 32, (a + 7) / 8);
  // FP64 arithmetic at every precision: the intermediates are FP64, and
  // converting them to FP32 costs GB300's FP64 pipe as much as the FMAs
  if (hs > 48 * 1024) SM_CHECK(raise_smem_limit(k_h12_apply<T, T>, hs));
  k_h12_apply<T, T><<<grd, blk, hs, st>>>(X1, H, a, c, p1, p2, e, f, X2);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return product<T>(ctx, st, precision, SM_OP_N, SM_OP_T, a * p1 * p2, g, e * f, X2, e * f, R,
                    e * f, out, g);
}

template int two_site_matvec<double>(Ctx&, cudaStream_t, int, int, int, int, int, int, int, int,
                                     const double*, const double*, const double*, const double*,
                                     double*, int);
template int two_site_matvec<cplx>(Ctx&, cudaStream_t, int, int, int, int, int, int, int, int,
                                   const cplx*, const cplx*, const cplx*, const cplx*, cplx*, int);

// ---------------------------------------------------------------------------
// Prepared form for a Lanczos run (real operands, TF32X3 / BF16): L and R do
// not change between matvecs, so they become tensor-core operand planes once.
// Per matvec only v is converted; the first product writes X1 in FP32, the
// MPO step reads it in FP32 and writes X2 straight into the second product's
// operand planes, and the second product writes the FP64 result.
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// X2[(a, ko, lo)][(dd, f)] = sum_{c,k,l} X1[a][c][k][l][f] H[c][ko][k][lo][l][dd]
// in FP32, written as K-contiguous operand rows of kp entries (the caller
// zeroes the columns past E F): one BF16 plane, or TF32 hi = rna(x) and
// lo = x - hi.  One thread per (a, f), lanes along f; H (FP64) converted into
// shared memory.
template <bool BF16>
__global__ void k_h12_planes(const float* __restrict__ X1, const double* __restrict__ H, int A,
                             int Cc, int p1, int p2, int E, int F, int kp, void* __restrict__ hi,
                             float* __restrict__ lo) {
  extern __shared__ float hs[];
  const int nh = Cc * p1 * p1 * p2 * p2 * E;
  for (int i = threadIdx.x + blockDim.x * threadIdx.y; i < nh; i += blockDim.x * blockDim.y)
    hs[i] = (float)H[i];
  __syncthreads();
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int a = blockIdx.y * blockDim.y + threadIdx.y;
  if (a >= A || f >= F) return;
  const float* x = X1 + (size_t)a * Cc * p1 * p2 * F + f;
  for (int ko = 0; ko < p1; ++ko)
    for (int lo2 = 0; lo2 < p2; ++lo2) {
      const size_t row = ((size_t)a * p1 + ko) * p2 + lo2;
      for (int dd = 0; dd < E; ++dd) {
        float acc = 0.f;
        for (int c = 0; c < Cc; ++c)
          for (int k = 0; k < p1; ++k)
            for (int l = 0; l < p2; ++l) {
              const float h = hs[((((c * p1 + ko) * p1 + k) * p2 + lo2) * p2 + l) * E + dd];
              if (h == 0.f) continue;  // zero blocks of the MPO (warp-uniform)
              acc = fmaf(h, x[(((size_t)c * p1 + k) * p2 + l) * F], acc);
            }
        const size_t o = row * kp + (size_t)dd * F + f;
        if (BF16) {
          reinterpret_cast<__nv_bfloat16*>(hi)[o] = __float2bfloat16_rn(acc);
        } else {
          const float h = tf32_round(acc);
          reinterpret_cast<float*>(hi)[o] = h;
          lo[o] = acc - h;
        }
      }
    }
}

}  // namespace

int two_site_prepare(Ctx& ctx, cudaStream_t st, int a, int c, int b, int p1, int p2, int e,
                     int g, int f, const double* L, const double* R, int precision) {
  if (precision != SM_MATVEC_TF32X3 && precision != SM_MATVEC_BF16) {
    set_error("two_site_prepare: the prepared matvec takes SM_MATVEC_TF32X3 or SM_MATVEC_BF16");
    return SM_ERR_VALUE;
  }
  MatvecPrep& mp = ctx.mvp;
  mp = MatvecPrep{};
  mp.precision = precision;
  mp.a = a, mp.c = c, mp.b = b, mp.p1 = p1, mp.p2 = p2, mp.e = e, mp.g = g, mp.f = f;
  mp.L = L;
  mp.R = R;
  const int n1 = p1 * p2 * f;
  mp.tc = gemm_tc_eligible(a * c, n1, b) && gemm_tc_eligible(a * p1 * p2, g, e * f);
  if (!mp.tc) return SM_OK;  // small shapes: the matvec runs the generic path
  const bool bf16 = precision == SM_MATVEC_BF16;
  const int TK = tc_kslab(bf16);
  mp.kpL = (b + TK - 1) / TK * TK;
  mp.kpR = (e * f + TK - 1) / TK * TK;
  const size_t es = bf16 ? 2 : 4;
  SM_CHECK(ctx.scratch("mvp.Lh", es * (size_t)a * c * mp.kpL, &mp.Lh));
  SM_CHECK(ctx.scratch("mvp.Rh", es * (size_t)g * mp.kpR, &mp.Rh));
  if (!bf16) {
    SM_CHECK(ctx.scratch("mvp.Ll", (size_t)a * c * mp.kpL, &mp.Ll));
    SM_CHECK(ctx.scratch("mvp.Rl", (size_t)g * mp.kpR, &mp.Rl));
  }
  // L[(a,c)][b] and R[g][(d,f)] are K-contiguous already
  SM_CHECK(tc_planes(ctx, st, L, b, a * c, b, mp.kpL, 0, bf16, mp.Lh, mp.Ll));
  SM_CHECK(tc_planes(ctx, st, R, e * f, g, e * f, mp.kpR, 0, bf16, mp.Rh, mp.Rl));
  return SM_OK;
}

int two_site_matvec_prepared(Ctx& ctx, cudaStream_t st, const double* H, const double* v,
                             double* out) {
  const MatvecPrep& mp = ctx.mvp;
  if (mp.precision < 0) {
    set_error("two_site_matvec_prepared: no prepared operator (sm_two_site_prepare)");
    return SM_ERR_VALUE;
  }
  const int a = mp.a, c = mp.c, b = mp.b, p1 = mp.p1, p2 = mp.p2, e = mp.e, g = mp.g, f = mp.f;
  if (!mp.tc)
    return two_site_matvec<double>(ctx, st, a, c, b, p1, p2, e, g, f, mp.L, H, mp.R, v, out,
                                   mp.precision);
  const bool bf16 = mp.precision == SM_MATVEC_BF16;
  const size_t es = bf16 ? 2 : 4;
  const int n1 = p1 * p2 * f, m3 = a * p1 * p2;
  void *vh, *x2h;
  float *vl = nullptr, *x2l = nullptr, *X1;
  SM_CHECK(ctx.scratch("mvp.vh", es * (size_t)n1 * mp.kpL, &vh));
  SM_CHECK(ctx.scratch("mvp.x2h", es * (size_t)m3 * mp.kpR, &x2h));
  SM_CHECK(ctx.scratch("mvp.X1", (size_t)a * c * n1, &X1));
  if (!bf16) {
    SM_CHECK(ctx.scratch("mvp.vl", (size_t)n1 * mp.kpL, &vl));
    SM_CHECK(ctx.scratch("mvp.x2l", (size_t)m3 * mp.kpR, &x2l));
  }
  // v[b][(k,l,f)]: op(B)^T rows are its columns
  SM_CHECK(tc_planes(ctx, st, v, n1, n1, b, mp.kpL, 1, bf16, vh, vl));
  ctx.stats.gemm_tc_launches += 2;
  ctx.stats.gemm_tc_flops += 2.0 * a * c * n1 * b + 2.0 * m3 * g * e * f;
  SM_CHECK(gemm_tc_planes<float>(ctx, st, a * c, n1, mp.kpL, bf16, mp.Lh, mp.Ll, vh, vl, 1.0,
                                 0.0, X1, n1));
  if (mp.kpR > e * f) {  // zero K padding of the second product's A operand
    SM_CUDA_CHECK(cudaMemsetAsync(x2h, 0, es * (size_t)m3 * mp.kpR, st));
    if (!bf16) SM_CUDA_CHECK(cudaMemsetAsync(x2l, 0, sizeof(float) * (size_t)m3 * mp.kpR, st));
  }
  const size_t hs = sizeof(float) * (size_t)c * p1 * p1 * p2 * p2 * e;
  const dim3 blk(32, 8), grd((f + 31) / 32, (a + 7) / 8);
  if (bf16) {
    if (hs > 48 * 1024) SM_CHECK(raise_smem_limit(k_h12_planes<true>, hs));
    k_h12_planes<true><<<grd, blk, hs, st>>>(X1, H, a, c, p1, p2, e, f, mp.kpR, x2h, x2l);
  } else {
    if (hs > 48 * 1024) SM_CHECK(raise_smem_limit(k_h12_planes<false>, hs));
    k_h12_planes<false><<<grd, blk, hs, st>>>(X1, H, a, c, p1, p2, e, f, mp.kpR, x2h, x2l);
  }
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return gemm_tc_planes<double>(ctx, st, m3, g, mp.kpR, bf16, x2h, x2l, mp.Rh, mp.Rl, 1.0, 0.0,
                                out, g);
}

}  // namespace sm
