// <O a | O b> of an MPO O applied to two MPS, computed from the factors.
//
// The reference forms the product MPS O|psi> (bond chi*D) and takes its norm
// with scprod (state/simplification.py:101, MPS.norm_squared in
// state/mps.py; environments.pxi:87-118), which costs 4 d (chi D)^3 flops per
// site.  Here the environment keeps the MPO legs apart,
//   E[x, alpha, beta, y]   (x: bond of a, alpha/beta: MPO bond on the bra/ket
//                           side, y: bond of b),
// and one site is two FP64 GEMMs of 2 d D^2 chi^3 flops each plus one small
// contraction with the double-layer MPO tensor
//   K4[alpha, beta, j, k, alpha', beta'] = sum_i conj(O[alpha,i,j,alpha']) O[beta,i,k,beta'].
// The value is the reference's to FP64 rounding (the same sum in a different
// order).  Sites alternate which state is contracted first so that every GEMM
// reads its operands in place (op T / op C on the MPS tensor) and the output's
// leading index is the one the next site contracts first:
//   even sites: E[x][a][b][y] -> U = a^H E -> W = K4 . U -> E' = b^T W = E'[y'][a'][b'][x']
//   odd sites:  E[y][a][b][x] -> P = b^T E -> Q = K4 . P -> E' = a^H Q = E'[x'][a'][b'][y']
#include <algorithm>

#include "kernels.cuh"

namespace sm {

namespace {

// K4[al][be][j][k][al2][be2] = sum_i conj(O[al,i,j,al2]) O[be,i,k,be2]
template <typename T>
__global__ void k_double_layer(const T* __restrict__ O, int Dl, int q, int p, int Dr,
                               T* __restrict__ K4) {
  const size_t total = (size_t)Dl * Dl * p * p * Dr * Dr;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    size_t r = e;
    const int be2 = (int)(r % Dr); r /= Dr;
    const int al2 = (int)(r % Dr); r /= Dr;
    const int k = (int)(r % p); r /= p;
    const int j = (int)(r % p); r /= p;
    const int be = (int)(r % Dl); r /= Dl;
    const int al = (int)r;
    T acc = S<T>::zero();
    for (int i = 0; i < q; ++i)
      acc = S<T>::cfma(O[(((size_t)al * q + i) * p + j) * Dr + al2],
                       O[(((size_t)be * q + i) * p + k) * Dr + be2], acc);
    K4[e] = acc;
  }
}

// Out[l][t][al2][be2][o] = sum_{al,be,s} K4[al][be][j][k][al2][be2] In[s][o][al][be][l]
// with (j, k) = (s, t), or (t, s) when `swap` is set.  One thread per (l, o)
// pair and output physical index t; lanes run along l, so the loads of In are
// contiguous; the K4 entries are warp-uniform (zero blocks of the MPO, common
// in banded operators, are skipped).
template <typename T>
__global__ void k_double_layer_apply(const T* __restrict__ K4, int Dl, int p, int Dr, int swap,
                                     const T* __restrict__ In, int no, int nl,
                                     T* __restrict__ Out) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  const int o = blockIdx.y * blockDim.y + threadIdx.y;
  if (l >= nl || o >= no) return;
  const size_t sIn = (size_t)no * Dl * Dl * nl;  // stride of s in In
  const T* in = In + (size_t)o * Dl * Dl * nl + l;
  for (int t = 0; t < p; ++t)
    for (int a2 = 0; a2 < Dr; ++a2)
      for (int b2 = 0; b2 < Dr; ++b2) {
        T acc = S<T>::zero();
        for (int s = 0; s < p; ++s) {
          const int j = swap ? t : s, k = swap ? s : t;
          for (int a = 0; a < Dl; ++a)
            for (int b = 0; b < Dl; ++b) {
              const T w = K4[(((((size_t)a * Dl + b) * p + j) * p + k) * Dr + a2) * Dr + b2];
              if (S<T>::abs2(w) == 0.0) continue;
              acc = S<T>::fma(w, in[(size_t)s * sIn + ((size_t)a * Dl + b) * nl], acc);
            }
        }
        Out[((((size_t)l * p + t) * Dr + a2) * Dr + b2) * no + o] = acc;
      }
}

}  // namespace

template <typename T>
int mpo_scprod_impl(Ctx& ctx, cudaStream_t st, int L, const int* dout, const int* din,
                    const int* Db, const void* const* Ov, const int* ab, const void* const* Av,
                    const int* bb, const void* const* Bv, double* out) {
  const T* const* O = reinterpret_cast<const T* const*>(Ov);
  const T* const* A = reinterpret_cast<const T* const*>(Av);
  const T* const* B = reinterpret_cast<const T* const*>(Bv);
  size_t me = 1, mu = 1, mk = 1;
  for (int i = 0; i <= L; ++i) me = std::max(me, (size_t)ab[i] * Db[i] * Db[i] * bb[i]);
  for (int i = 0; i < L; ++i) {
    const size_t p = din[i];
    mu = std::max(mu, p * ab[i + 1] * Db[i] * Db[i] * bb[i]);
    mu = std::max(mu, p * bb[i + 1] * Db[i] * Db[i] * ab[i]);
    mu = std::max(mu, p * bb[i] * Db[i + 1] * Db[i + 1] * ab[i + 1]);
    mu = std::max(mu, p * ab[i] * Db[i + 1] * Db[i + 1] * bb[i + 1]);
    mk = std::max(mk, (size_t)Db[i] * Db[i] * p * p * Db[i + 1] * Db[i + 1]);
  }
  T *E, *E2, *U, *W, *K4;
  SM_CHECK(ctx.scratch("mn.E", me, &E));
  SM_CHECK(ctx.scratch("mn.E2", me, &E2));
  SM_CHECK(ctx.scratch("mn.U", mu, &U));
  SM_CHECK(ctx.scratch("mn.W", mu, &W));
  SM_CHECK(ctx.scratch("mn.K4", mk, &K4));
  const T one = S<T>::one(), zero = S<T>::zero();
  SM_CHECK(set_identity<T>(st, 1, E, 1));
  for (int i = 0; i < L; ++i) {
    const int Dl = Db[i], Dr = Db[i + 1], p = din[i], q = dout[i];
    const int xa = ab[i], xa2 = ab[i + 1], yb = bb[i], yb2 = bb[i + 1];
    const size_t nk = (size_t)Dl * Dl * p * p * Dr * Dr;
    k_double_layer<T><<<(int)std::min<size_t>((nk + 255) / 256, 1024), 256, 0, st>>>(
        O[i], Dl, q, p, Dr, K4);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    const bool even = (i % 2) == 0;
    // first contraction: over the leading leg of E
    //   even: U[(j,x'),(a,b,y)] = sum_x conj(A[x][(j,x')]) E[x][(a,b,y)]
    //   odd:  U[(k,y'),(a,b,x)] = sum_y B[y][(k,y')] E[y][(a,b,x)]
    const int lead = even ? xa : yb, lead2 = even ? xa2 : yb2, other = even ? yb : xa;
    const int other2 = even ? yb2 : xa2;
    const int N1 = Dl * Dl * other;
    if (even)
      SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_C, SM_OP_N, p * lead2, N1, lead, one, A[i], p * lead2, E,
                           N1, zero, U, N1));
    else
      SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_T, SM_OP_N, p * lead2, N1, lead, one, B[i], p * lead2, E,
                           N1, zero, U, N1));
    // double layer: W[(l,t),(a',b',o')] with l = the other state's left bond
    dim3 blk(32, 8), grd((other + 31) / 32, (lead2 + 7) / 8);
    k_double_layer_apply<T><<<grd, blk, 0, st>>>(K4, Dl, p, Dr, even ? 0 : 1, U, lead2, other, W);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    // second contraction over (l, t) with the other state:
    //   even: E'[y'][(a',b',x')] = sum_{y,k} B[(y,k)][y'] W[(y,k)][...]
    //   odd:  E'[x'][(a',b',y')] = sum_{x,j} conj(A[(x,j)][x']) W[(x,j)][...]
    const int N2 = Dr * Dr * lead2;
    if (even)
      SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_T, SM_OP_N, other2, N2, other * p, one, B[i], other2, W,
                           N2, zero, E2, N2));
    else
      SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_C, SM_OP_N, other2, N2, other * p, one, A[i], other2, W,
                           N2, zero, E2, N2));
    std::swap(E, E2);
  }
  double* h = reinterpret_cast<double*>(ctx.pinned) + 64;
  SM_CUDA_CHECK(cudaMemcpyAsync(h, E, sizeof(T), cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  out[0] = h[0];
  out[1] = sizeof(T) == sizeof(double) ? 0.0 : h[1];
  if (ctx.precision != SM_PRECISION_FP64) SM_CHECK(tc_status_check(ctx, st));
  return SM_OK;
}

template int mpo_scprod_impl<double>(Ctx&, cudaStream_t, int, const int*, const int*, const int*,
                                     const void* const*, const int*, const void* const*,
                                     const int*, const void* const*, double*);
template int mpo_scprod_impl<cplx>(Ctx&, cudaStream_t, int, const int*, const int*, const int*,
                                   const void* const*, const int*, const void* const*, const int*,
                                   const void* const*, double*);

}  // namespace sm
