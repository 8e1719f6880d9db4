// FP64 SVD splits and the truncation rule.
//
// The reference calls LAPACK gesdd (cython/svd.pxi:35-83) and then truncates
// the singular values in place (cython/truncation.pxi:251-334).  Here the SVD
// is a one-sided (Hestenes) Jacobi iteration in FP64, run as ONE cooperative
// persistent kernel per matrix:
//
//  * the k = min(m,n) vectors of the short side (rows of A if m <= n, rows of
//    A^T otherwise) are stored contiguously, k x l with l = max(m,n);
//  * a sweep visits all k(k-1)/2 pairs in k-1 rounds of a round-robin
//    tournament; the k/2 pairs of a round are independent and are spread over
//    the CTAs (one pair per CTA), and rounds are separated by a grid barrier
//    whose spin is bounded (it reports a timeout instead of hanging);
//  * each pair computes <w_p|w_p>, <w_q|w_q>, <w_p|w_q> in FP64 and applies the
//    complex Jacobi rotation that zeroes <w_p|w_q> to both vectors and to the
//    accumulated unitary X (k x k);
//  * the iteration stops after the first sweep without a rotation; a cap on
//    sweeps reports non-convergence (the LinAlgError of the reference).
//
// After convergence W = X A (rows orthogonal): s_i = |w_i|, the long-side
// singular vectors are w_i / s_i and the short-side ones are the rows of X.
// Singular values are sorted on the device (their IEEE bit patterns order like
// the values) and truncated by a single thread with the reference's exact
// comparisons and summation order (no FMA contraction).
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "kernels.cuh"

namespace sm {

namespace {

struct JacobiCtl {
  unsigned int bar_count;
  unsigned int bar_gen;
  unsigned int rot[2];
  int status;
  int sweeps;
  int pad[2];
};

// Grid-wide barrier with a bounded spin.  Returns false (and sets the status
// flag) if the other CTAs did not arrive within the spin limit.
__device__ bool grid_sync(JacobiCtl* ctl) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    if (gridDim.x > 1) {
      volatile unsigned int* vgen = &ctl->bar_gen;
      volatile int* vstatus = &ctl->status;
      const unsigned int gen = *vgen;
      __threadfence();
      const unsigned int arrived = atomicAdd(&ctl->bar_count, 1u);
      if (arrived == gridDim.x - 1) {
        atomicExch(&ctl->bar_count, 0u);
        __threadfence();
        atomicAdd(&ctl->bar_gen, 1u);
      } else {
        long long it = 0;
        while (*vgen == gen) {
          if (++it > kSpinLimit || (*vstatus & DEV_BARRIER_TIMEOUT)) {
            atomicOr(&ctl->status, DEV_BARRIER_TIMEOUT);
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
      __threadfence();
    }
  }
  __syncthreads();
  return ok != 0;
}

template <typename T>
__device__ __forceinline__ T ldcg(const T* p);
template <>
__device__ __forceinline__ double ldcg<double>(const double* p) { return __ldcg(p); }
template <>
__device__ __forceinline__ cplx ldcg<cplx>(const cplx* p) {
  const double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  return {v.x, v.y};
}
template <typename T>
__device__ __forceinline__ void stcg(T* p, T v);
template <>
__device__ __forceinline__ void stcg<double>(double* p, double v) { __stcg(p, v); }
template <>
__device__ __forceinline__ void stcg<cplx>(cplx* p, cplx v) {
  __stcg(reinterpret_cast<double2*>(p), make_double2(v.re, v.im));
}

template <int NT>
__device__ __forceinline__ void block_sum4(double& a, double& b, double& c, double& d,
                                           double (*red)[NT / 32]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
    d += __shfl_xor_sync(0xffffffffu, d, o);
  }
  const int w = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (lane == 0) {
    red[0][w] = a;
    red[1][w] = b;
    red[2][w] = c;
    red[3][w] = d;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a = b = c = d = 0.0;
    for (int i = 0; i < NT / 32; ++i) {
      a += red[0][i];
      b += red[1][i];
      c += red[2][i];
      d += red[3][i];
    }
  }
}

__device__ __forceinline__ void gamma_parts(double g, double& re, double& im) { re = g; im = 0.0; }
__device__ __forceinline__ void gamma_parts(cplx g, double& re, double& im) { re = g.re; im = g.im; }
__device__ __forceinline__ void make_coef(double& sp, double& sq, double s, double er, double ei) {
  sp = s * er;  // real case: e = sign(gamma)
  sq = s * er;
}

template <typename T> struct Rot;
template <> struct Rot<double> {
  double c, sp, sq;
  __device__ void set(double c_, double s, double er, double) { c = c_; sp = s * er; sq = s * er; }
  // p' = c p - sp q ; q' = sq p + c q
  __device__ void apply(double& p, double& q) const {
    const double np = fma(c, p, -sp * q);
    const double nq = fma(sq, p, c * q);
    p = np;
    q = nq;
  }
};
template <> struct Rot<cplx> {
  double c;
  cplx sp, sq;  // sp = s conj(e), sq = s e
  __device__ void set(double c_, double s, double er, double ei) {
    c = c_;
    sp = {s * er, -s * ei};
    sq = {s * er, s * ei};
  }
  __device__ void apply(cplx& p, cplx& q) const {
    const cplx np = {c * p.re - (sp.re * q.re - sp.im * q.im), c * p.im - (sp.re * q.im + sp.im * q.re)};
    const cplx nq = {(sq.re * p.re - sq.im * p.im) + c * q.re, (sq.re * p.im + sq.im * p.re) + c * q.im};
    p = np;
    q = nq;
  }
};

template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_jacobi(T* W, int ldw, T* X, int ldx, int k, int l,
                                               double tol, int max_sweeps, JacobiCtl* ctl) {
  __shared__ double red[4][NT / 32];
  __shared__ double coef[4];
  __shared__ int do_rot;
  __shared__ unsigned int nrot_shared;
  const int kp = k + (k & 1);
  const int rounds = kp - 1, npairs = kp / 2;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    for (int r = 0; r < rounds; ++r) {
      for (int t = blockIdx.x; t < npairs; t += gridDim.x) {
        int p, q;
        if (t == 0) {
          p = kp - 1;
          q = r;
        } else {
          p = (r + t) % (kp - 1);
          q = (r + kp - 1 - t) % (kp - 1);
        }
        if (p >= k || q >= k) continue;  // the dummy player of an odd k
        if (p > q) { const int tmp = p; p = q; q = tmp; }
        T* wp = W + (size_t)p * ldw;
        T* wq = W + (size_t)q * ldw;
        double a = 0.0, b = 0.0, gr = 0.0, gi = 0.0;
        T g = S<T>::zero();
        for (int x = threadIdx.x; x < l; x += NT) {
          const T u = ldcg(wp + x), v = ldcg(wq + x);
          a += S<T>::abs2(u);
          b += S<T>::abs2(v);
          g = S<T>::cfma(u, v, g);
        }
        gamma_parts(g, gr, gi);
        block_sum4<NT>(a, b, gr, gi, red);
        if (threadIdx.x == 0) {
          const double gabs = sqrt(gr * gr + gi * gi);
          int rot = (gabs > 0.0) && (gabs > tol * sqrt(a) * sqrt(b));
          if (rot) {
            const double zeta = (b - a) / (2.0 * gabs);
            double t;
            if (fabs(zeta) > 1e150) t = 0.5 / zeta;
            else t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
            const double c = 1.0 / sqrt(1.0 + t * t);
            coef[0] = c;
            coef[1] = c * t;
            coef[2] = gr / gabs;
            coef[3] = gi / gabs;
            atomicAdd(&ctl->rot[sweep & 1], 1u);
          }
          do_rot = rot;
        }
        __syncthreads();
        if (do_rot) {
          Rot<T> R;
          R.set(coef[0], coef[1], coef[2], coef[3]);
          for (int x = threadIdx.x; x < l; x += NT) {
            T u = ldcg(wp + x), v = ldcg(wq + x);
            R.apply(u, v);
            stcg(wp + x, u);
            stcg(wq + x, v);
          }
          T* xp = X + (size_t)p * ldx;
          T* xq = X + (size_t)q * ldx;
          for (int x = threadIdx.x; x < k; x += NT) {
            T u = ldcg(xp + x), v = ldcg(xq + x);
            R.apply(u, v);
            stcg(xp + x, u);
            stcg(xq + x, v);
          }
        }
        __syncthreads();
      }
      if (!grid_sync(ctl)) return;
      // slot (sweep+1)&1 was read by every CTA before this barrier: recycle it
      if (r == 0 && sweep > 0 && blockIdx.x == 0 && threadIdx.x == 0)
        ctl->rot[(sweep + 1) & 1] = 0u;
    }
    if (threadIdx.x == 0) nrot_shared = ((volatile unsigned int*)ctl->rot)[sweep & 1];
    __syncthreads();
    if (nrot_shared == 0u) {
      if (blockIdx.x == 0 && threadIdx.x == 0) ctl->sweeps = sweep + 1;
      return;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->sweeps = max_sweeps;
    atomicOr(&ctl->status, DEV_NOT_CONVERGED);
  }
}

// s_i = |w_i|, one warp per row
template <typename T>
__global__ void k_row_norms(const T* W, int ldw, int k, int l, double* nrm) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x % 32;
  if (warp >= k) return;
  const T* w = W + (size_t)warp * ldw;
  double a = 0.0;
  for (int x = lane; x < l; x += 32) a += S<T>::abs2(ldcg(w + x));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (lane == 0) nrm[warp] = sqrt(a);
}

// The reference truncation rules, executed by one thread.  Products and sums
// use explicit round-to-nearest intrinsics so that no FMA contraction changes
// the rounding of the discarded-weight sums (truncation.pxi:251-327).
__device__ void truncate_rule(const double* s, int N, const sm_strategy& st, double* errors,
                              int* D_out, double* err_out) {
  const int maxb = st.max_bond_dimension;
  if (st.method == SM_DO_NOT_TRUNCATE) {
    *D_out = N;
    *err_out = 0.0;
    return;
  }
  if (st.method == SM_RELATIVE_NORM_SQUARED_ERROR) {
    double total = 0.0;
    for (int i = 0; i < N; ++i) {
      errors[i] = total;
      const double v = s[N - 1 - i];
      total = __dadd_rn(total, __dmul_rn(v, v));
    }
    errors[N] = total;
    const double max_error = __dmul_rn(total, st.tolerance);
    int i = N - 1;
    for (int j = 0; j < N; ++j) {
      if (errors[j] > max_error) {
        i = j - 1;
        break;
      }
    }
    int final_size = N - i;
    if (final_size > maxb) final_size = maxb;
    *D_out = final_size;
    *err_out = errors[N - final_size];
    return;
  }
  const double max_error =
      st.method == SM_RELATIVE_SINGULAR_VALUE ? __dmul_rn(st.tolerance, s[0]) : st.tolerance;
  int final_size = N < maxb ? N : maxb;
  for (int i = 1; i < final_size; ++i) {
    if (s[i] <= max_error) {
      final_size = i;
      break;
    }
  }
  double err = 0.0;
  for (int i = final_size; i < N; ++i) err = __dadd_rn(err, __dmul_rn(s[i], s[i]));
  *D_out = final_size;
  *err_out = err;
}

__global__ void k_truncate(const double* s, int N, sm_strategy st, double* errors,
                           SplitResult* res) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int D;
    double e;
    truncate_rule(s, N, st, errors, &D, &e);
    res->D = D;
    res->err2 = e;
    res->status = 0;
  }
}

// Sort the k norms descending (stable by index), then truncate.
__global__ void k_sort_truncate(const double* nrm, int k, sm_strategy st, int* perm,
                                double* s_sorted, double* errors, const JacobiCtl* ctl,
                                SplitResult* res) {
  extern __shared__ unsigned long long keys[];
  for (int i = threadIdx.x; i < k; i += blockDim.x)
    keys[i] = (unsigned long long)__double_as_longlong(nrm[i]);
  __syncthreads();
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    const unsigned long long ki = keys[i];
    int rank = 0;
    for (int j = 0; j < k; ++j) {
      const unsigned long long kj = keys[j];
      rank += (kj > ki) || (kj == ki && j < i);
    }
    perm[rank] = i;
    s_sorted[rank] = __longlong_as_double((long long)ki);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int D;
    double e;
    truncate_rule(s_sorted, k, st, errors, &D, &e);
    res->D = D;
    res->err2 = e;
    res->status = ctl ? ctl->status : 0;
    res->sweeps = ctl ? ctl->sweeps : 0;
    // non-finite input shows up as a NaN norm
    for (int i = 0; i < k; ++i)
      if (!(s_sorted[i] == s_sorted[i]) || s_sorted[i] > DBL_MAX) res->status |= DEV_NONFINITE;
  }
}

// Write the factors of the truncated SVD.  Element (i, j) of the left output
// (m x D) and (j, x) of the right output (D x n).
template <typename T>
__global__ void k_emit(int wide, int m, int n, int D, const T* __restrict__ W, int ldw,
                       const T* __restrict__ X, int ldx, const int* __restrict__ perm,
                       const double* __restrict__ s, int left_mode, T* __restrict__ left,
                       int right_mode, T* __restrict__ right) {
  const size_t nl = left_mode ? (size_t)m * D : 0;
  const size_t nr = right_mode ? (size_t)D * n : 0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nl + nr;
       e += (size_t)gridDim.x * blockDim.x) {
    if (e < nl) {
      const int i = (int)(e / D), j = (int)(e % D);
      const int pj = perm[j];
      const double sj = s[j];
      T v;
      if (wide) {
        v = S<T>::conj(X[(size_t)pj * ldx + i]);
        if (left_mode == OUT_US) v = S<T>::scale(v, sj);
      } else {
        v = W[(size_t)pj * ldw + i];
        if (left_mode == OUT_U) v = sj > 0.0 ? S<T>::scale(v, 1.0 / sj) : S<T>::zero();
      }
      left[e] = v;
    } else {
      const size_t f = e - nl;
      const int j = (int)(f / n), x = (int)(f % n);
      const int pj = perm[j];
      const double sj = s[j];
      T v;
      if (wide) {
        v = W[(size_t)pj * ldw + x];
        if (right_mode == OUT_VT) v = sj > 0.0 ? S<T>::scale(v, 1.0 / sj) : S<T>::zero();
      } else {
        v = S<T>::conj(X[(size_t)pj * ldx + x]);
        if (right_mode == OUT_SVT) v = S<T>::scale(v, sj);
      }
      right[f] = v;
    }
  }
}

constexpr int kJacobiThreads = 128;
constexpr int kMaxSweeps = 60;

template <typename T>
int coop_limit(Ctx& ctx) {
  const void* fn = reinterpret_cast<const void*>(&k_jacobi<T, kJacobiThreads>);
  auto it = ctx.coop_blocks.find(fn);
  if (it != ctx.coop_blocks.end()) return it->second;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_jacobi<T, kJacobiThreads>,
                                                    kJacobiThreads, 0) != cudaSuccess)
    per_sm = 1;
  const int lim = std::max(1, per_sm) * std::max(1, ctx.num_sms);
  ctx.coop_blocks[fn] = lim;
  return lim;
}

}  // namespace

int truncate_device(Ctx& ctx, cudaStream_t st, const double* s_dev, int n,
                    const sm_strategy& strat, int* rank, double* err2) {
  double* errors;
  SplitResult* res;
  SM_CHECK(ctx.scratch("trunc.errors", (size_t)n + 1, &errors));
  SM_CHECK(ctx.scratch("trunc.res", 1, &res));
  k_truncate<<<1, 32, 0, st>>>(s_dev, n, strat, errors, res);
  SM_CUDA_CHECK(cudaGetLastError());
  SplitResult* h = reinterpret_cast<SplitResult*>(ctx.pinned);
  SM_CUDA_CHECK(cudaMemcpyAsync(h, res, sizeof(SplitResult), cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  *rank = h->D;
  *err2 = h->err2;
  return SM_OK;
}

template <typename T>
int svd_split(Ctx& ctx, cudaStream_t st, const T* A, int m, int n, const sm_strategy& strat,
              int left_mode, T* left, int right_mode, T* right, double* s_out,
              SplitResult* out) {
  if (m <= 0 || n <= 0) {
    set_error("svd: empty matrix");
    return SM_ERR_VALUE;
  }
  const int k = std::min(m, n), l = std::max(m, n);
  const bool wide = m <= n;
  T *W, *X;
  double *nrm, *s_sorted, *errors;
  int* perm;
  JacobiCtl* ctl;
  SplitResult* res;
  SM_CHECK(ctx.scratch("svd.W", (size_t)k * l, &W));
  SM_CHECK(ctx.scratch("svd.X", (size_t)k * k, &X));
  SM_CHECK(ctx.scratch("svd.nrm", (size_t)k, &nrm));
  SM_CHECK(ctx.scratch("svd.s", (size_t)k, &s_sorted));
  SM_CHECK(ctx.scratch("svd.err", (size_t)k + 1, &errors));
  SM_CHECK(ctx.scratch("svd.perm", (size_t)k, &perm));
  SM_CHECK(ctx.scratch("svd.ctl", 1, &ctl));
  SM_CHECK(ctx.scratch("svd.res", 1, &res));

  if (wide) {
    SM_CUDA_CHECK(cudaMemcpyAsync(W, A, sizeof(T) * (size_t)k * l, cudaMemcpyDeviceToDevice, st));
  } else {
    SM_CHECK(transpose<T>(st, m, n, A, n, W, m));
  }
  SM_CHECK(set_identity<T>(st, k, X, k));
  SM_CUDA_CHECK(cudaMemsetAsync(ctl, 0, sizeof(JacobiCtl), st));
  if (k >= 2) {
    const int npairs = (k + (k & 1)) / 2;
    const int grid = std::min(npairs, coop_limit<T>(ctx));
    int ldw = l, ldx = k, kk = k, ll = l, ms = kMaxSweeps;
    double tol = std::sqrt((double)l) * DBL_EPSILON;
    void* args[] = {&W, &ldw, &X, &ldx, &kk, &ll, &tol, &ms, &ctl};
    SM_CUDA_CHECK(cudaLaunchCooperativeKernel(
        reinterpret_cast<const void*>(&k_jacobi<T, kJacobiThreads>), dim3(grid),
        dim3(kJacobiThreads), args, 0, st));
  }
  k_row_norms<T><<<(k + 7) / 8, 256, 0, st>>>(W, l, k, l, nrm);
  SM_CUDA_CHECK(cudaGetLastError());
  const size_t smem = sizeof(unsigned long long) * (size_t)k;
  if (smem > 200 * 1024) {
    set_error("svd: matrix too large for the on-chip sort");
    return SM_ERR_VALUE;
  }
  if (smem > 48 * 1024)
    SM_CUDA_CHECK(cudaFuncSetAttribute(k_sort_truncate, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
  k_sort_truncate<<<1, 1024, smem, st>>>(nrm, k, strat, perm, s_sorted, errors, ctl, res);
  SM_CUDA_CHECK(cudaGetLastError());
  SplitResult* h = reinterpret_cast<SplitResult*>(ctx.pinned);
  SM_CUDA_CHECK(cudaMemcpyAsync(h, res, sizeof(SplitResult), cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  *out = *h;
  if (h->status & DEV_BARRIER_TIMEOUT) {
    set_error("svd: grid barrier timed out");
    return SM_ERR_TIMEOUT;
  }
  if (h->status & DEV_NONFINITE) {
    set_error("SVD did not converge (non-finite values)");
    return SM_ERR_LINALG;
  }
  if (h->status & DEV_NOT_CONVERGED) {
    set_error("SVD did not converge");
    return SM_ERR_LINALG;
  }
  if (s_out)
    SM_CUDA_CHECK(cudaMemcpyAsync(s_out, s_sorted, sizeof(double) * k, cudaMemcpyDeviceToDevice, st));
  if (ctx.trace) {
    const size_t off = ctx.tr_s.size();
    ctx.tr_s.resize(off + k);
    SM_CUDA_CHECK(cudaMemcpyAsync(ctx.tr_s.data() + off, s_sorted, sizeof(double) * k,
                                  cudaMemcpyDeviceToHost, st));
    SM_CUDA_CHECK(cudaStreamSynchronize(st));
    ctx.tr_rank.push_back(h->D);
    ctx.tr_len.push_back(k);
    ctx.tr_err2.push_back(h->err2);
  }
  const int D = h->D;
  if (left_mode || right_mode) {
    const size_t total = (left_mode ? (size_t)m * D : 0) + (right_mode ? (size_t)D * n : 0);
    const int blocks = (int)std::min<size_t>((total + 255) / 256, 4096);
    k_emit<T><<<std::max(blocks, 1), 256, 0, st>>>(wide, m, n, D, W, l, X, k, perm, s_sorted,
                                                   left_mode, left, right_mode, right);
    SM_CUDA_CHECK(cudaGetLastError());
  }
  return SM_OK;
}

template int svd_split<double>(Ctx&, cudaStream_t, const double*, int, int, const sm_strategy&,
                               int, double*, int, double*, double*, SplitResult*);
template int svd_split<cplx>(Ctx&, cudaStream_t, const cplx*, int, int, const sm_strategy&, int,
                             cplx*, int, cplx*, double*, SplitResult*);

}  // namespace sm
