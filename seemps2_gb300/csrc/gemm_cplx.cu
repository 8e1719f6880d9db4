// Complex products on the tensor cores as three real products (the 3M form).
//
// With op(A) = Ar + i Ai and op(B) = Br + i Bi held as split real planes,
//   T1 = Ar Br,  T2 = Ai Bi,  T3 = (Ar + Ai)(Br + Bi),
//   op(A) op(B) = (T1 - T2) + i (T3 - T1 - T2):
// three real GEMMs (6 M N K real flops) instead of the four of the direct form.
// k_cplx_planes writes op(X) (transposition and conjugation applied) as the
// three FP64 planes re, im and re + im in one pass; the real products run on
// the 3xTF32 tensor-core GEMM (FP32 accuracy, the mixed forms' contractions)
// or on the FP64-accurate BF16-slice GEMM (the mixed forms' FP64 products);
// k_cplx_combine forms alpha (T1 - T2 + i (T3 - T1 - T2)) + beta C.  The 3M
// form's cancellation in T3 - T1 - T2 keeps the error normwise: within a few
// units of the real products' own error times |A| |B|.
#include <algorithm>

#include "kernels.cuh"

namespace sm {

namespace {

// Y = op(X) (rows x cols) as three row-major FP64 planes; X is stored
// rows x cols (trans = 0) or cols x rows (trans = 1) with leading dimension
// ldx; conj negates the imaginary part.  32 x 32 tiles through shared memory
// keep both the read and the writes coalesced.
__global__ void k_cplx_planes(const cplx* __restrict__ X, int ldx, int rows, int cols, int trans,
                              int conj, double* __restrict__ re, double* __restrict__ im,
                              double* __restrict__ sum) {
  __shared__ cplx tile[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int j = ty; j < 32; j += 8) {
    cplx v{0.0, 0.0};
    if (trans) {  // stored cols x rows: read along r
      const int c = c0 + j, r = r0 + tx;
      if (c < cols && r < rows) v = X[(size_t)c * ldx + r];
    } else {
      const int r = r0 + j, c = c0 + tx;
      if (c < cols && r < rows) v = X[(size_t)r * ldx + c];
    }
    tile[j][tx] = v;
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int r = r0 + j, c = c0 + tx;
    if (r < rows && c < cols) {
      const cplx v = trans ? tile[tx][j] : tile[j][tx];
      const double vi = conj ? -v.im : v.im;
      const size_t o = (size_t)r * cols + c;
      re[o] = v.re;
      im[o] = vi;
      sum[o] = v.re + vi;
    }
  }
}

__global__ void k_cplx_combine(int M, int N, const double* __restrict__ T1,
                               const double* __restrict__ T2, const double* __restrict__ T3,
                               cplx alpha, cplx beta, cplx* __restrict__ C, int ldc) {
  const size_t mn = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < mn;
       e += (size_t)gridDim.x * blockDim.x) {
    const double t1 = T1[e], t2 = T2[e];
    const double pr = t1 - t2, pi = T3[e] - t1 - t2;
    cplx* p = C + (e / N) * ldc + (e % N);
    double cr = alpha.re * pr - alpha.im * pi;
    double ci = alpha.re * pi + alpha.im * pr;
    if (beta.re != 0.0 || beta.im != 0.0) {
      const cplx o = *p;
      cr += beta.re * o.re - beta.im * o.im;
      ci += beta.re * o.im + beta.im * o.re;
    }
    *p = cplx{cr, ci};
  }
}

int planes(cudaStream_t st, const cplx* X, int ldx, int rows, int cols, int trans, int conj,
           double* re, double* im, double* sum) {
  const dim3 blk(32, 8), grd((cols + 31) / 32, (rows + 31) / 32);
  k_cplx_planes<<<grd, blk, 0, st>>>(X, ldx, rows, cols, trans, conj, re, im, sum);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

}  // namespace

// A complex product does four real multiply-adds per element step, so the
// tensor-core thresholds apply to 4 M N K; the calls on fixed shapes at the
// threshold only check that the tensor-map encoder is available.
bool gemm_cplx_tc_eligible(int M, int N, int K) {
  return M >= 64 && N >= 64 && K >= 32 && 4.0 * M * N * K >= 4.0 * 1024 * 1024 &&
         gemm_tc_eligible(64, 64, 1024);
}

bool gemm_cplx_oz_eligible(int M, int N, int K) {
  return M >= 32 && N >= 32 && K >= 32 && 4.0 * M * N * K >= 2.0 * 1024 * 1024 &&
         gemm_oz_eligible(32, 32, 2048);
}

int gemm_cplx_3m(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, cplx alpha,
                 const cplx* A, int lda, const cplx* B, int ldb, cplx beta, cplx* C, int ldc,
                 bool fp64_accurate) {
  const size_t mk = (size_t)M * K, kn = (size_t)K * N, mn = (size_t)M * N;
  double *pa, *pb, *t;
  SM_CHECK(ctx.scratch("c3m.A", 3 * mk, &pa));
  SM_CHECK(ctx.scratch("c3m.B", 3 * kn, &pb));
  SM_CHECK(ctx.scratch("c3m.T", 3 * mn, &t));
  // op(A): M x K; op(B): K x N
  SM_CHECK(planes(st, A, lda, M, K, opA == SM_OP_N ? 0 : 1, opA == SM_OP_C ? 1 : 0, pa, pa + mk,
                  pa + 2 * mk));
  SM_CHECK(planes(st, B, ldb, K, N, opB == SM_OP_N ? 0 : 1, opB == SM_OP_C ? 1 : 0, pb, pb + kn,
                  pb + 2 * kn));
  for (int p = 0; p < 3; ++p) {
    const double* a = pa + p * mk;
    const double* b = pb + p * kn;
    double* c = t + p * mn;
    if (fp64_accurate)
      SM_CHECK(gemm_oz(ctx, st, SM_OP_N, SM_OP_N, M, N, K, 1.0, a, K, b, N, 0.0, c, N));
    else
      SM_CHECK(gemm_tc(ctx, st, SM_OP_N, SM_OP_N, M, N, K, 1.0, a, K, b, N, 0.0, c, N));
  }
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>((mn + 255) / 256, 4096));
  k_cplx_combine<<<blocks, 256, 0, st>>>(M, N, t, t + mn, t + 2 * mn, alpha, beta, C, ldc);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

}  // namespace sm
