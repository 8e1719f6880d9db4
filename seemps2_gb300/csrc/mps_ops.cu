// Element-wise and reduction kernels of the MPS path: the MPO x MPS site
// product, transposes, scalings, block copies for MPSSum joins and the
// deterministic vdot used by the sweep's error estimate.  All of them are
// HBM/L2-bound element streams; grids are sized in multiples of the SM count.
#include <algorithm>

#include "kernels.cuh"

namespace sm {

namespace {

template <typename T>
__global__ void k_scale_matrix(int M, int N, T beta, T* C, int ldc, int zero) {
  const size_t total = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    T* c = C + (e / N) * ldc + (e % N);
    *c = zero ? S<T>::zero() : beta * *c;
  }
}

template <typename T>
__global__ void k_scale_vector(size_t n, double f, T* x) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    x[e] = S<T>::scale(x[e], f);
}

// C[(c*a_ + a), i, (d*b_ + b)] = sum_j B[c, j, d] O[a, i, j, b]
template <typename T>
__global__ void k_mpo_multiply(const T* __restrict__ O, int a_, int i_, int j_, int b_,
                               const T* __restrict__ B, int c_, int d_, T* __restrict__ C) {
  const size_t total = (size_t)c_ * a_ * i_ * d_ * b_;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    size_t r = e;
    const int b = (int)(r % b_); r /= b_;
    const int d = (int)(r % d_); r /= d_;
    const int i = (int)(r % i_); r /= i_;
    const int a = (int)(r % a_); r /= a_;
    const int c = (int)r;
    T acc = S<T>::zero();
    for (int j = 0; j < j_; ++j)
      acc = S<T>::fma(B[((size_t)c * j_ + j) * d_ + d], O[(((size_t)a * i_ + i) * j_ + j) * b_ + b],
                      acc);
    C[e] = acc;
  }
}

// Joined tensor of two MPOs applied one after the other (A first, then B):
// C[(a c), i, k, (b d)] = sum_j B[a, i, j, b] A[c, j, k, d]; one thread per output.
template <typename T>
__global__ void k_mpo_join(const T* __restrict__ B, int a_, int i_, int j_, int b_,
                           const T* __restrict__ A, int c_, int k_, int d_, T* __restrict__ C) {
  const size_t total = (size_t)a_ * c_ * i_ * k_ * b_ * d_;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    size_t r = e;
    const int d = (int)(r % d_); r /= d_;
    const int b = (int)(r % b_); r /= b_;
    const int k = (int)(r % k_); r /= k_;
    const int i = (int)(r % i_); r /= i_;
    const int c = (int)(r % c_); r /= c_;
    const int a = (int)r;
    T acc = S<T>::zero();
    for (int j = 0; j < j_; ++j)
      acc = S<T>::fma(B[(((size_t)a * i_ + i) * j_ + j) * b_ + b],
                      A[(((size_t)c * j_ + j) * k_ + k) * d_ + d], acc);
    C[e] = acc;
  }
}

// B[j, i] = A[i, j], 32x32 tiles through shared memory
template <typename T>
__global__ void k_transpose(int m, int n, const T* __restrict__ A, int lda, T* __restrict__ B,
                            int ldb) {
  __shared__ T tile[32][33];
  const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = i0 + r, j = j0 + threadIdx.x;
    if (i < m && j < n) tile[r][threadIdx.x] = A[(size_t)i * lda + j];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int j = j0 + r, i = i0 + threadIdx.x;
    if (i < m && j < n) B[(size_t)j * ldb + i] = tile[threadIdx.x][r];
  }
}

template <typename T>
__global__ void k_identity(int k, T* X, int ldx) {
  const size_t total = (size_t)k * k;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / k), j = (int)(e % k);
    X[(size_t)i * ldx + j] = i == j ? S<T>::one() : S<T>::zero();
  }
}

template <typename T>
__global__ void k_copy_block3(const T* __restrict__ src, int a, int d, int b, T* __restrict__ dst,
                              int A, int B, int off_a, int off_b, T w) {
  const size_t total = (size_t)a * d * b;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int z = (int)(e % b);
    const int y = (int)((e / b) % d);
    const int x = (int)(e / ((size_t)b * d));
    dst[((size_t)(x + off_a) * d + y) * B + (z + off_b)] = w * src[e];
  }
}

constexpr int kVdotBlocks = 304;  // 2 x 152 SMs

template <typename T>
__global__ void k_vdot_partial(size_t n, const T* __restrict__ x, const T* __restrict__ y,
                               double* part) {
  double re = 0.0, im = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const T v = S<T>::cfma(x[e], y[e], S<T>::zero());
    if constexpr (sizeof(T) == sizeof(double)) {
      re += S<T>::real(v);
    } else {
      const cplx c = *reinterpret_cast<const cplx*>(&v);
      re += c.re;
      im += c.im;
    }
  }
  __shared__ double sr[32], si[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  if (threadIdx.x % 32 == 0) {
    sr[threadIdx.x / 32] = re;
    si[threadIdx.x / 32] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    re = im = 0.0;
    for (int w = 0; w < blockDim.x / 32; ++w) {
      re += sr[w];
      im += si[w];
    }
    part[2 * blockIdx.x] = re;
    part[2 * blockIdx.x + 1] = im;
  }
}

__global__ void k_vdot_final(int nb, const double* part, double* out) {
  if (threadIdx.x == 0) {
    double re = 0.0, im = 0.0;
    for (int b = 0; b < nb; ++b) {
      re += part[2 * b];
      im += part[2 * b + 1];
    }
    out[0] = re;
    out[1] = im;
  }
}

template <typename T>
int grid_for(size_t n) {
  return (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 152 * 16));
}

}  // namespace

template <typename T>
int scale_matrix(cudaStream_t st, int M, int N, T beta, T* C, int ldc) {
  const size_t n = (size_t)M * N;
  if (!n) return SM_OK;
  k_scale_matrix<T><<<grid_for<T>(n), 256, 0, st>>>(M, N, beta, C, ldc, S<T>::abs2(beta) == 0.0);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

template <typename T>
int scale_vector(cudaStream_t st, size_t n, double f, T* x) {
  if (!n) return SM_OK;
  k_scale_vector<T><<<grid_for<T>(n), 256, 0, st>>>(n, f, x);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

template <typename T>
int fill_zero(cudaStream_t st, size_t n, T* x) {
  if (!n) return SM_OK;
  SM_CUDA_CHECK(cudaMemsetAsync(x, 0, n * sizeof(T), st));
  return SM_OK;
}

template <typename T>
int mpo_multiply_tensor(cudaStream_t st, const T* O, int a, int i, int j, int b, const T* B,
                        int c, int d, T* C) {
  const size_t n = (size_t)c * a * i * d * b;
  if (!n) return SM_OK;
  k_mpo_multiply<T><<<grid_for<T>(n), 256, 0, st>>>(O, a, i, j, b, B, c, d, C);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

template <typename T>
int mpo_join(cudaStream_t st, const T* B, int a, int i, int j, int b, const T* A, int c, int k,
             int d, T* C) {
  const size_t n = (size_t)a * c * i * k * b * d;
  if (!n) return SM_OK;
  k_mpo_join<T><<<grid_for<T>(n), 256, 0, st>>>(B, a, i, j, b, A, c, k, d, C);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

template <typename T>
int vdot(Ctx& ctx, cudaStream_t st, size_t n, const T* x, const T* y, double* out_dev) {
  double* part;
  SM_CHECK(ctx.scratch("vdot.part", 2 * kVdotBlocks, &part));
  const int nb = (int)std::max<size_t>(1, std::min<size_t>(kVdotBlocks, (n + 255) / 256));
  k_vdot_partial<T><<<nb, 256, 0, st>>>(n, x, y, part);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  k_vdot_final<<<1, 32, 0, st>>>(nb, part, out_dev);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

template <typename T>
int transpose(cudaStream_t st, int m, int n, const T* A, int lda, T* B, int ldb) {
  if (!m || !n) return SM_OK;
  dim3 grid((n + 31) / 32, (m + 31) / 32);
  k_transpose<T><<<grid, dim3(32, 8), 0, st>>>(m, n, A, lda, B, ldb);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

template <typename T>
int set_identity(cudaStream_t st, int k, T* X, int ldx) {
  if (!k) return SM_OK;
  k_identity<T><<<grid_for<T>((size_t)k * k), 256, 0, st>>>(k, X, ldx);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

template <typename T>
int copy_block3(cudaStream_t st, const T* src, int a, int d, int b, T* dst, int A, int B,
                int off_a, int off_b, T w) {
  const size_t n = (size_t)a * d * b;
  if (!n) return SM_OK;
  k_copy_block3<T><<<grid_for<T>(n), 256, 0, st>>>(src, a, d, b, dst, A, B, off_a, off_b, w);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}


#define SM_INST(T)                                                                          \
  template int scale_matrix<T>(cudaStream_t, int, int, T, T*, int);                         \
  template int scale_vector<T>(cudaStream_t, size_t, double, T*);                           \
  template int fill_zero<T>(cudaStream_t, size_t, T*);                                      \
  template int mpo_multiply_tensor<T>(cudaStream_t, const T*, int, int, int, int, const T*, \
                                      int, int, T*);                                        \
  template int mpo_join<T>(cudaStream_t, const T*, int, int, int, int, const T*, int, int,  \
                           int, T*);                                                        \
  template int vdot<T>(Ctx&, cudaStream_t, size_t, const T*, const T*, double*);            \
  template int transpose<T>(cudaStream_t, int, int, const T*, int, T*, int);                \
  template int set_identity<T>(cudaStream_t, int, T*, int);                                 \
  template int copy_block3<T>(cudaStream_t, const T*, int, int, int, T*, int, int, int, int, T);
SM_INST(double)
SM_INST(cplx)

}  // namespace sm
