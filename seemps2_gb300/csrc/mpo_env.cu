// Three-leg MPO environments of DMRG (the reference's update_left_mpo_environment /
// update_right_mpo_environment, state/environments.py:19-42):
//
//   left:  out[d, e, f] = sum conj(A[a, j, d]) rho[a, c, b] O[c, j, i, e] B[b, i, f]
//   right: out[a, c, b] = sum conj(A[a, j, d]) rho[d, e, f] O[c, j, i, e] B[b, i, f]
//
// with the bra site A (a, j, d), the MPO site O (c, j, i, e) and the ket site
// B (b, i, f).  Each is two GEMMs around one pass over the MPO site, which is
// tiny (D x d x d x D) and sparse, so it stays out of the GEMMs:
//   left   1. X[(a c), (i f)]  = rho[(a c), b] B[b, (i f)]                  GEMM
//          2. Y[a, j, e, f]    = sum_{c,i} X[a, c, i, f] O[c, j, i, e]      k_mpo_site_left
//          3. out[d, (e f)]    = A[(a j), d]^H Y[(a j), (e f)]              GEMM (op C)
//   right  1. X[(b i), (d e)]  = B[(b i), f] rho[(d e), f]^T                GEMM (op T)
//          2. Y[c, b, j, d]    = sum_{i,e} X[b, i, d, e] O[c, j, i, e]      k_mpo_site_right
//          3. Z[(c b), a]      = Y[(c b), (j d)] A[a, (j d)]^H              GEMM (op C)
//          4. out[a, (c b)]    = Z^T                                        transpose
// At chi = 256, D = 5, d = 2 the two GEMMs are 671 MFLOP each; the MPO pass
// reads and writes chi^2 D d values once.
#include <algorithm>

#include "kernels.cuh"

namespace sm {

namespace {

// Y[a][j][e][f] = sum_{c,i} X[a][c][i][f] O[c][j][i][e]; one thread per (a, f),
// lanes along f; O in shared memory; zero MPO entries skipped (warp-uniform).
template <typename T>
__global__ void k_mpo_site_left(const T* __restrict__ X, const T* __restrict__ O, int A, int Cc,
                                int J, int I, int E, int F, T* __restrict__ Y) {
  extern __shared__ unsigned char sraw[];
  T* Os = reinterpret_cast<T*>(sraw);
  const int no = Cc * J * I * E;
  for (int x = threadIdx.x + blockDim.x * threadIdx.y; x < no; x += blockDim.x * blockDim.y)
    Os[x] = O[x];
  __syncthreads();
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int a = blockIdx.y * blockDim.y + threadIdx.y;
  if (f >= F || a >= A) return;
  const T* x = X + (size_t)a * Cc * I * F + f;
  T* y = Y + (size_t)a * J * E * F + f;
  for (int j = 0; j < J; ++j)
    for (int e = 0; e < E; ++e) {
      T acc = S<T>::zero();
      for (int c = 0; c < Cc; ++c)
        for (int i = 0; i < I; ++i) {
          const T o = Os[((c * J + j) * I + i) * E + e];
          if (S<T>::abs2(o) == 0.0) continue;
          acc = S<T>::fma(o, x[((size_t)c * I + i) * F], acc);
        }
      y[((size_t)j * E + e) * F] = acc;
    }
}

// Y[c][b][j][d] = sum_{i,e} X[b][i][d][e] O[c][j][i][e]; one thread per (b, d),
// lanes along d.
template <typename T>
__global__ void k_mpo_site_right(const T* __restrict__ X, const T* __restrict__ O, int Bn,
                                 int Cc, int J, int I, int E, int Dn, T* __restrict__ Y) {
  extern __shared__ unsigned char sraw[];
  T* Os = reinterpret_cast<T*>(sraw);
  const int no = Cc * J * I * E;
  for (int x = threadIdx.x + blockDim.x * threadIdx.y; x < no; x += blockDim.x * blockDim.y)
    Os[x] = O[x];
  __syncthreads();
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y * blockDim.y + threadIdx.y;
  if (d >= Dn || b >= Bn) return;
  const T* x = X + (size_t)b * I * Dn * E + (size_t)d * E;
  for (int c = 0; c < Cc; ++c)
    for (int j = 0; j < J; ++j) {
      T acc = S<T>::zero();
      for (int i = 0; i < I; ++i)
        for (int e = 0; e < E; ++e) {
          const T o = Os[((c * J + j) * I + i) * E + e];
          if (S<T>::abs2(o) == 0.0) continue;
          acc = S<T>::fma(o, x[(size_t)i * Dn * E + e], acc);
        }
      Y[(((size_t)c * Bn + b) * J + j) * Dn + d] = acc;
    }
}

}  // namespace

template <typename T>
int mpo_env_left(Ctx& ctx, cudaStream_t st, const T* rho, const T* A, int a, int j, int d,
                 const T* O, int c, int i, int e, const T* B, int b, int f, T* out) {
  T *X, *Y;
  SM_CHECK(ctx.scratch("me.X", (size_t)a * c * i * f, &X));
  SM_CHECK(ctx.scratch("me.Y", (size_t)a * j * e * f, &Y));
  const T one = S<T>::one(), zero = S<T>::zero();
  SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_N, SM_OP_N, a * c, i * f, b, one, rho, b, B, i * f, zero, X,
                       i * f));
  const size_t smem = sizeof(T) * (size_t)c * j * i * e;
  if (smem > 48 * 1024) SM_CHECK(raise_smem_limit(k_mpo_site_left<T>, smem));
  const dim3 blk(32, 8), grd((f + 31) / 32, (a + 7) / 8);
  k_mpo_site_left<T><<<grd, blk, smem, st>>>(X, O, a, c, j, i, e, f, Y);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return gemm_ctx<T>(ctx, st, SM_OP_C, SM_OP_N, d, e * f, a * j, one, A, d, Y, e * f, zero, out,
                     e * f);
}

template <typename T>
int mpo_env_right(Ctx& ctx, cudaStream_t st, const T* rho, const T* A, int a, int j, int d,
                  const T* O, int c, int i, int e, const T* B, int b, int f, T* out) {
  T *X, *Y, *Z;
  SM_CHECK(ctx.scratch("me.X", (size_t)b * i * d * e, &X));
  SM_CHECK(ctx.scratch("me.Y", (size_t)c * b * j * d, &Y));
  SM_CHECK(ctx.scratch("me.Z", (size_t)c * b * a, &Z));
  const T one = S<T>::one(), zero = S<T>::zero();
  SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_N, SM_OP_T, b * i, d * e, f, one, B, f, rho, f, zero, X,
                       d * e));
  const size_t smem = sizeof(T) * (size_t)c * j * i * e;
  if (smem > 48 * 1024) SM_CHECK(raise_smem_limit(k_mpo_site_right<T>, smem));
  const dim3 blk(32, 8), grd((d + 31) / 32, (b + 7) / 8);
  k_mpo_site_right<T><<<grd, blk, smem, st>>>(X, O, b, c, j, i, e, d, Y);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_N, SM_OP_C, c * b, a, j * d, one, Y, j * d, A, j * d, zero, Z,
                       a));
  return transpose<T>(st, c * b, a, Z, a, out, c * b);
}

template int mpo_env_left<double>(Ctx&, cudaStream_t, const double*, const double*, int, int, int,
                                  const double*, int, int, int, const double*, int, int, double*);
template int mpo_env_left<cplx>(Ctx&, cudaStream_t, const cplx*, const cplx*, int, int, int,
                                const cplx*, int, int, int, const cplx*, int, int, cplx*);
template int mpo_env_right<double>(Ctx&, cudaStream_t, const double*, const double*, int, int,
                                   int, const double*, int, int, int, const double*, int, int,
                                   double*);
template int mpo_env_right<cplx>(Ctx&, cudaStream_t, const cplx*, const cplx*, int, int, int,
                                 const cplx*, int, int, int, const cplx*, int, int, cplx*);

}  // namespace sm
