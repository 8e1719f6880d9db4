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

// Grid-wide barrier with a bounded spin: one arrival counter and a generation
// word (measured on GB300: ~2.3 us for 16-256 CTAs, cheaper than per-CTA
// arrival flags gathered by one CTA).  Returns false (and sets the status
// flag) if the wait exceeded the spin limit.
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
          __nanosleep(32);
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

// One warp per pair.  Each row is [w | x]: the l entries of the vector being
// orthogonalised followed by the k entries of its row of the accumulated
// unitary X, so one rotation updates both in a single pass.  With E > 0 a lane
// keeps its E elements of both rows in registers between the dot product and
// the rotation; E == 0 streams the rows twice from L2 (large sizes).
//
// Rotation parameters avoid FP64 division and square roots (slow on GB300's
// FP64 unit): the convergence test |g|^2 > tol^2 a b needs no root, and the
// angle, c = 1/sqrt(1+t^2), s = c t and the phase g/|g| use the FP64 rsqrt and
// reciprocal intrinsics, so every applied rotation is unitary to FP64
// rounding.  Squared norms are computed exactly in the first round of every
// sweep and updated in closed form after each rotation during the sweep.
template <typename T, int E>
__global__ void __launch_bounds__(256) k_jacobi(T* Wx, int ld, int k, int l, double tol2,
                                                int max_sweeps, double* nrm, const double* nrm0,
                                                JacobiCtl* ctl) {
  __shared__ int sflag;
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const int gw = blockIdx.x * wpb + (threadIdx.x >> 5);
  const int nw = gridDim.x * wpb;
  const int kp = k + (k & 1);
  const int rounds = kp - 1, npairs = kp / 2;
  const int L = l + k;
  volatile int* vflag = reinterpret_cast<volatile int*>(ctl->rot);
  double frob2 = 0.0;  // |A|_F^2 from the squared row norms, fixed order
  for (int i = lane; i < k; i += 32) frob2 += __ldcg(nrm0 + i);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) frob2 += __shfl_xor_sync(0xffffffffu, frob2, o);
  const double tiny = 256.0 * l * DBL_EPSILON * DBL_EPSILON * frob2;
  const double tiny2 = tiny * tiny;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    for (int r = 0; r < rounds; ++r) {
      for (int t = gw; t < npairs; t += nw) {
        int p, q;
        if (t == 0) {
          p = kp - 1;
          q = r;
        } else {
          p = (r + t) % (kp - 1);
          q = (r + kp - 1 - t) % (kp - 1);
        }
        if (p >= k || q >= k) {
          // the dummy player of an odd k: its partner idles this round, but
          // in the first round its exact squared norm must still be refreshed
          if (r == 0) {
            const int row = p < q ? p : q;
            double a = 0.0;
            for (int x = lane; x < l; x += 32) a += S<T>::abs2(ldcg(Wx + (size_t)row * ld + x));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            if (lane == 0) __stcg(nrm + row, a);
          }
          continue;
        }
        if (p > q) { const int tmp = p; p = q; q = tmp; }
        T* rp = Wx + (size_t)p * ld;
        T* rq = Wx + (size_t)q * ld;
        double a = 0.0, b = 0.0;
        T g = S<T>::zero();
        T u[E > 0 ? E : 1], v[E > 0 ? E : 1];
        if constexpr (E > 0) {
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const int x = lane + 32 * e;
            if (x < L) {
              u[e] = ldcg(rp + x);
              v[e] = ldcg(rq + x);
            } else {
              u[e] = S<T>::zero();
              v[e] = S<T>::zero();
            }
            if (x < l) {
              if (r == 0) {
                a += S<T>::abs2(u[e]);
                b += S<T>::abs2(v[e]);
              }
              g = S<T>::cfma(u[e], v[e], g);
            }
          }
        } else {
          for (int x = lane; x < l; x += 32) {
            const T uu = ldcg(rp + x), vv = ldcg(rq + x);
            if (r == 0) {
              a += S<T>::abs2(uu);
              b += S<T>::abs2(vv);
            }
            g = S<T>::cfma(uu, vv, g);
          }
        }
        double gr, gi;
        gamma_parts(g, gr, gi);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          gr += __shfl_xor_sync(0xffffffffu, gr, o);
          gi += __shfl_xor_sync(0xffffffffu, gi, o);
          if (r == 0) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
          }
        }
        if (r != 0) {
          a = __ldcg(nrm + p);
          b = __ldcg(nrm + q);
        }
        const double g2 = gr * gr + gi * gi;
        // relative test |g| > tol sqrt(a b), plus an absolute floor just above
        // the rounding-noise level (256 l eps^2 |A|_F^2): the noise vectors of a
        // numerically rank-deficient matrix are not rotated against each other
        // sweep after sweep, while every vector with a norm above
        // 16 sqrt(l) eps |A| (~1e-13 |A|) is still fully orthogonalised
        const bool rot = g2 > tiny2 && g2 > tol2 * a * b;
        double na = a, nb = b;
        if (rot) {
          const double rsq = rsqrt(g2);  // 1/|g|
          const double gabs = g2 * rsq;
          const double zeta = 0.5 * (b - a) * rsq;
          // t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)), the smaller root
          const double az = fabs(zeta);
          double tt;
          if (az < 1e150) {
            const double w = fma(az, az, 1.0);
            tt = __drcp_rn(az + w * rsqrt(w));
          } else {
            tt = __drcp_rn(2.0 * az);
          }
          tt = copysign(tt, zeta);
          const double c = rsqrt(fma(tt, tt, 1.0));
          const double sn = c * tt;
          Rot<T> R;
          R.set(c, sn, gr * rsq, gi * rsq);
          const double cs2 = 2.0 * c * sn * gabs;
          na = c * c * a + sn * sn * b - cs2;
          nb = sn * sn * a + c * c * b + cs2;
          if constexpr (E > 0) {
#pragma unroll
            for (int e = 0; e < E; ++e) {
              const int x = lane + 32 * e;
              R.apply(u[e], v[e]);
              if (x < L) {
                stcg(rp + x, u[e]);
                stcg(rq + x, v[e]);
              }
            }
          } else {
            for (int x = lane; x < L; x += 32) {
              T uu = ldcg(rp + x), vv = ldcg(rq + x);
              R.apply(uu, vv);
              stcg(rp + x, uu);
              stcg(rq + x, vv);
            }
          }
          if (lane == 0) vflag[sweep & 1] = 1;
        }
        if (lane == 0 && (rot || r == 0)) {
          __stcg(nrm + p, na);
          __stcg(nrm + q, nb);
        }
      }
      if (!grid_sync(ctl)) return;
      // slot (sweep+1)&1 was read by every CTA before this barrier: recycle it
      if (r == 0 && sweep > 0 && blockIdx.x == 0 && threadIdx.x == 0) vflag[(sweep + 1) & 1] = 0;
    }
    if (threadIdx.x == 0) sflag = vflag[sweep & 1];
    __syncthreads();
    if (sflag == 0) {
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
__global__ void k_row_norms(const T* W, int ldw, int k, int l, double* nrm, int squared) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x % 32;
  if (warp >= k) return;
  const T* w = W + (size_t)warp * ldw;
  double a = 0.0;
  for (int x = lane; x < l; x += 32) a += S<T>::abs2(ldcg(w + x));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (lane == 0) nrm[warp] = squared ? a : sqrt(a);
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

constexpr int kMaxSweeps = 60;

template <typename T, int E>
int launch_jacobi(Ctx& ctx, cudaStream_t st, T* Wx, int ld, int k, int l, double tol2,
                  double* nrm, const double* nrm0, JacobiCtl* ctl) {
  const int npairs = (k + (k & 1)) / 2;
  const int sms = std::max(1, ctx.num_sms);
  const int wpb = std::min(8, std::max(1, (npairs + sms - 1) / sms));
  const int threads = 32 * wpb;
  auto fn = k_jacobi<T, E>;
  const void* key = reinterpret_cast<const void*>(fn);
  int per_sm = 0;
  const auto it = ctx.coop_blocks.find(key);
  // occupancy depends on the block size; cache per (kernel, wpb)
  const void* ckey = reinterpret_cast<const char*>(key) + wpb;
  const auto it2 = ctx.coop_blocks.find(ckey);
  (void)it;
  if (it2 != ctx.coop_blocks.end()) per_sm = it2->second;
  else {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess)
      per_sm = 1;
    per_sm = std::max(1, per_sm);
    ctx.coop_blocks[ckey] = per_sm;
  }
  const int grid = std::max(1, std::min((npairs + wpb - 1) / wpb, per_sm * sms));
  int ms = kMaxSweeps;
  void* args[] = {&Wx, &ld, &k, &l, &tol2, &ms, &nrm, &nrm0, &ctl};
  SM_CUDA_CHECK(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(fn), dim3(grid),
                                            dim3(threads), args, 0, st));
                                            note_launch();
  return SM_OK;
}

template <typename T>
int run_jacobi(Ctx& ctx, cudaStream_t st, T* Wx, int ld, int k, int l, double tol2, double* nrm,
               const double* nrm0, JacobiCtl* ctl) {
  const int L = l + k;
  const int need = (L + 31) / 32;
  if constexpr (sizeof(T) == sizeof(double)) {
    if (need <= 2) return launch_jacobi<T, 2>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 4) return launch_jacobi<T, 4>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 8) return launch_jacobi<T, 8>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 12) return launch_jacobi<T, 12>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 16) return launch_jacobi<T, 16>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 24) return launch_jacobi<T, 24>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 32) return launch_jacobi<T, 32>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 40) return launch_jacobi<T, 40>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
  } else {
    if (need <= 2) return launch_jacobi<T, 2>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 4) return launch_jacobi<T, 4>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 8) return launch_jacobi<T, 8>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 12) return launch_jacobi<T, 12>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 16) return launch_jacobi<T, 16>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
    if (need <= 20) return launch_jacobi<T, 20>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
  }
  return launch_jacobi<T, 0>(ctx, st, Wx, ld, k, l, tol2, nrm, nrm0, ctl);
}

template <typename T>
__global__ void k_fill_rows(int k, int l, T* Wx, int ld) {
  // X part of [W | X] = identity
  const size_t total = (size_t)k * k;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / k), j = (int)(e % k);
    Wx[(size_t)i * ld + l + j] = i == j ? S<T>::one() : S<T>::zero();
  }
}

}  // namespace

int truncate_device(Ctx& ctx, cudaStream_t st, const double* s_dev, int n,
                    const sm_strategy& strat, int* rank, double* err2) {
  double* errors;
  SplitResult* res;
  SM_CHECK(ctx.scratch("trunc.errors", (size_t)n + 1, &errors));
  SM_CHECK(ctx.scratch("trunc.res", 1, &res));
  k_truncate<<<1, 32, 0, st>>>(s_dev, n, strat, errors, res);
  note_launch();
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
  const int ld = l + k;  // rows are [w (l) | x (k)]
  T* Wx;
  double *nrm, *s_sorted, *errors;
  int* perm;
  JacobiCtl* ctl;
  SplitResult* res;
  SM_CHECK(ctx.scratch("svd.Wx", (size_t)k * ld, &Wx));
  SM_CHECK(ctx.scratch("svd.nrm", (size_t)k, &nrm));
  double* nrm0;
  SM_CHECK(ctx.scratch("svd.nrm0", (size_t)k, &nrm0));
  SM_CHECK(ctx.scratch("svd.s", (size_t)k, &s_sorted));
  SM_CHECK(ctx.scratch("svd.err", (size_t)k + 1, &errors));
  SM_CHECK(ctx.scratch("svd.perm", (size_t)k, &perm));
  SM_CHECK(ctx.scratch("svd.ctl", 1, &ctl));
  SM_CHECK(ctx.scratch("svd.res", 1, &res));

  if (wide) {
    SM_CUDA_CHECK(cudaMemcpy2DAsync(Wx, sizeof(T) * ld, A, sizeof(T) * n, sizeof(T) * n, m,
                                    cudaMemcpyDeviceToDevice, st));
  } else {
    SM_CHECK(transpose<T>(st, m, n, A, n, Wx, ld));
  }
  {
    const size_t tot = (size_t)k * k;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((tot + 255) / 256, 4096));
    k_fill_rows<T><<<blocks, 256, 0, st>>>(k, l, Wx, ld);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
  }
  SM_CUDA_CHECK(cudaMemsetAsync(ctl, 0, sizeof(JacobiCtl), st));
  if (k >= 2) {
    // squared row norms -> nrm; the Jacobi kernel sums them into |A|_F^2
    k_row_norms<T><<<(k + 7) / 8, 256, 0, st>>>(Wx, ld, k, l, nrm0, 1);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    const double tol = std::sqrt((double)l) * DBL_EPSILON;
    if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
    SM_CHECK(run_jacobi<T>(ctx, st, Wx, ld, k, l, tol * tol, nrm, nrm0, ctl));
    if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
    ctx.stats.jacobi_launches += 1;
    // 4 m n^2 + 8 n^3 with m >= n (x4 for complex arithmetic)
    ctx.stats.jacobi_flops += (4.0 * l * (double)k * k + 8.0 * (double)k * k * k) *
                              (sizeof(T) == sizeof(double) ? 1.0 : 4.0);
  }
  k_row_norms<T><<<(k + 7) / 8, 256, 0, st>>>(Wx, ld, k, l, nrm, 0);
  note_launch();
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
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  SplitResult* h = reinterpret_cast<SplitResult*>(ctx.pinned);
  SM_CUDA_CHECK(cudaMemcpyAsync(h, res, sizeof(SplitResult), cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  *out = *h;
  ctx.stats.splits += 1;
  ctx.stats.jacobi_sweeps += h->sweeps;
  if (ctx.timing && k >= 2) {
    float ms = 0.f;
    SM_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
    ctx.stats.jacobi_ms += ms;
  }
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
    k_emit<T><<<std::max(blocks, 1), 256, 0, st>>>(wide, m, n, D, Wx, ld, Wx + l, ld, perm,
                                                   s_sorted, left_mode, left, right_mode, right);
                                                   note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
  }
  return SM_OK;
}

template int svd_split<double>(Ctx&, cudaStream_t, const double*, int, int, const sm_strategy&,
                               int, double*, int, double*, double*, SplitResult*);
template int svd_split<cplx>(Ctx&, cudaStream_t, const cplx*, int, int, const sm_strategy&, int,
                             cplx*, int, cplx*, double*, SplitResult*);

}  // namespace sm
