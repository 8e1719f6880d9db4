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
#include <atomic>
#include <cfloat>
#include <climits>
#include <cmath>

#include "kernels.cuh"

namespace sm {

namespace {

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

// One CTA (NT threads, NT/32 warps) per pair, so that every SM sub-partition's
// FP64 unit works on a pair (GB300 FP64 is latency-bound with one warp per
// pair).  Each row is [w | x]: the l entries of the vector being
// orthogonalised followed by the k entries of its row of the accumulated
// unitary X, so one rotation updates both in a single pass.  With E > 0 a
// thread keeps its E elements of both rows in registers between the dot
// products and the rotation; E == 0 streams the rows twice from L2.
//
// Rotation parameters: the convergence test |g|^2 > tol^2 a b needs no root;
// zeta = (b - a) / 2|g| uses one FP64 rsqrt; t = tan(theta) is evaluated in
// FP32 (an inexact angle only leaves a slightly larger residual for the next
// sweep) except for |zeta| >= 1e18 where t = 1/2zeta in FP64; c = 1/sqrt(1+t^2),
// s = c t and the complex phase g/|g| use FP64 rsqrt, so every applied rotation
// is unitary to FP64 rounding.  Squared norms are computed exactly in the first
// round of every sweep and updated in closed form after each rotation.
//
// Pairs whose overlap is below an absolute floor (16 l eps^2 |A|_F^2, just
// above the rounding-noise level) count as orthogonal when `use_floor` is set:
// the noise vectors of a numerically rank-deficient matrix are then not
// rotated against each other sweep after sweep.  The caller sets it only when
// the truncation rule is certain to discard every such vector.
template <typename T, int NT, int E>
__global__ void __launch_bounds__(NT) k_jacobi(T* Wx, int ld, int k, int l, int L, double tol2,
                                               int use_floor, double defl_rel, double defl_abs,
                                               int max_sweeps, double* nrm, const double* nrm0,
                                               int* act, JacobiCtl* ctl) {
  constexpr int NW = NT / 32;
  __shared__ double part[2][NW][4];
  __shared__ int sflag, snact;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  volatile int* vflag = reinterpret_cast<volatile int*>(ctl->rot);
  double frob2 = 0.0;  // |A|_F^2 from the squared row norms, fixed order
  for (int i = lane; i < k; i += 32) frob2 += __ldcg(nrm0 + i);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) frob2 += __shfl_xor_sync(0xffffffffu, frob2, o);
  double tiny2 = 0.0;
  if (use_floor) {
    const double tiny = 16.0 * l * DBL_EPSILON * DBL_EPSILON * frob2;
    tiny2 = tiny * tiny;
  }
  // rows whose squared norm falls to thr or below are deflated: the
  // truncation rule certainly discards them, so they leave the round-robin
  const double thr = defl_abs > 0.0 ? fmin(defl_rel * frob2, defl_abs) : defl_rel * frob2;
  int it = 0;  // pair iterations of this CTA (selects the smem buffer)
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    // exact squared norms at the start of every sweep
    for (int i = blockIdx.x; i < k; i += gridDim.x) {
      double a = 0.0;
      for (int x = tid; x < l; x += NT) a += S<T>::abs2(ldcg(Wx + (size_t)i * ld + x));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0) part[0][warp][0] = a;
      __syncthreads();
      if (tid == 0) {
        double s = 0.0;
        for (int w = 0; w < NW; ++w) s += part[0][w][0];
        __stcg(nrm + i, s);
      }
      __syncthreads();
    }
    if (!grid_sync(ctl)) return;
    // every CTA read the previous sweep's rotation flag before this barrier
    if (sweep > 0 && blockIdx.x == 0 && tid == 0) vflag[(sweep + 1) & 1] = 0;
    // active rows, in ascending order, compacted by CTA 0
    if (blockIdx.x == 0) {
      __shared__ int wcount[NW];
      int base = 0;
      for (int i0 = 0; i0 < k; i0 += NT) {
        const int i = i0 + tid;
        const bool on = i < k && __ldcg(nrm + i) > thr;
        const unsigned int bal = __ballot_sync(0xffffffffu, on);
        if (lane == 0) wcount[warp] = __popc(bal);
        __syncthreads();
        int off = base;
        for (int w = 0; w < warp; ++w) off += wcount[w];
        if (on) act[off + __popc(bal & ((1u << lane) - 1u))] = i;
        int tot = 0;
        for (int w = 0; w < NW; ++w) tot += wcount[w];
        base += tot;
        __syncthreads();
      }
      if (tid == 0) ((volatile int*)&ctl->nact)[0] = base;
    }
    if (!grid_sync(ctl)) return;
    if (tid == 0) snact = ((volatile int*)&ctl->nact)[0];
    __syncthreads();
    const int ka = snact;
    const int kp = ka + (ka & 1);
    const int rounds = ka >= 2 ? kp - 1 : 0, npairs = kp / 2;
    for (int r = 0; r < rounds; ++r) {
      for (int t = blockIdx.x; t < npairs; t += gridDim.x, ++it) {
        int p, q;
        if (t == 0) {
          p = kp - 1;
          q = r;
        } else {
          p = (r + t) % (kp - 1);
          q = (r + kp - 1 - t) % (kp - 1);
        }
        double (*pt)[4] = part[it & 1];
        if (p >= ka || q >= ka) continue;  // the dummy player of an odd count
        p = __ldcg(act + p);
        q = __ldcg(act + q);
        if (p > q) { const int tmp = p; p = q; q = tmp; }
        T* rp = Wx + (size_t)p * ld;
        T* rq = Wx + (size_t)q * ld;
        double a = 0.0, b = 0.0;
        T g0 = S<T>::zero(), g1 = S<T>::zero();
        T u[E > 0 ? E : 1], v[E > 0 ? E : 1];
        if constexpr (E > 0) {
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const int x = tid + NT * e;
            if (x < L) {
              u[e] = ldcg(rp + x);
              v[e] = ldcg(rq + x);
            } else {
              u[e] = S<T>::zero();
              v[e] = S<T>::zero();
            }
          }
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const int x = tid + NT * e;
            if (x < l) {
              if (e & 1) g1 = S<T>::cfma(u[e], v[e], g1);
              else g0 = S<T>::cfma(u[e], v[e], g0);
            }
          }
        } else {
          for (int x = tid; x < l; x += NT) {
            const T uu = ldcg(rp + x), vv = ldcg(rq + x);
            g0 = S<T>::cfma(uu, vv, g0);
          }
        }
        constexpr bool kCplx = sizeof(T) != sizeof(double);
        double gr, gi, hr, hi;
        gamma_parts(g0, gr, gi);
        gamma_parts(g1, hr, hi);
        gr += hr;
        if constexpr (kCplx) gi += hi;
        // every reduced value costs one FP64 add per level (each FP64 warp
        // instruction occupies a sub-partition's FP64 pipe for ~64 cycles on
        // GB300), so only the values this round needs are reduced
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          gr += __shfl_xor_sync(0xffffffffu, gr, o);
          if constexpr (kCplx) gi += __shfl_xor_sync(0xffffffffu, gi, o);
        }
        if (lane == 0) {
          pt[warp][0] = gr;
          pt[warp][1] = gi;
        }
        __syncthreads();
        gr = pt[0][0];
        if constexpr (kCplx) gi = pt[0][1];
#pragma unroll
        for (int w = 1; w < NW; ++w) {  // same order in every thread
          gr += pt[w][0];
          if constexpr (kCplx) gi += pt[w][1];
        }
        if constexpr (!kCplx) gi = 0.0;
        // squared norms: exact at the start of the sweep, updated in closed
        // form after each rotation
        a = __ldcg(nrm + p);
        b = __ldcg(nrm + q);
        const double g2 = kCplx ? fma(gr, gr, gi * gi) : gr * gr;
        const bool rot = g2 > tiny2 && g2 > tol2 * a * b;
        double na = a, nb = b;
        if (rot) {
          // Angle in FP32 on values scaled by a power of two so that a + b
          // lands in [1, 2): zeta = (b - a) / 2|g|, t = sign(zeta) /
          // (|zeta| + sqrt(1 + zeta^2)).  The (c, s) pair (and the complex
          // phase) are then brought to unit norm in FP64 with a two-term
          // correction f = 1 - d/2 + 3d^2/8, d = c^2 + s^2 - 1 ~ 1e-7, which
          // leaves c^2 + s^2 - 1 = O(d^3): each rotation is unitary to FP64
          // rounding whatever the accuracy of the angle.
          // An FP32 angle annihilates the overlap only to ~1e-7 of itself.
          // Far from convergence that is harmless (the next sweep finishes
          // the job), but once the pair's cosine |g|/sqrt(ab) is small the
          // residual no longer shrinks quadratically, and inside a cluster
          // of (nearly) equal singular values the iteration stalls at the
          // FP32 level.  So the FP32 angle is only taken while the cosine is
          // at least 1e-4; the last sweeps' few rotations use FP64.
          const int ex = (__double2hiint(a + b) >> 20) & 0x7ff;
          const double sc = __hiloint2double((2046 - ex) << 20, 0);     // 2^(1023 - ex)
          const double sc_inv = __hiloint2double(ex << 20, 0);           // 2^(ex - 1023)
          const float as = (float)(a * sc), bs = (float)(b * sc);
          const float grs = (float)(gr * sc), gis = kCplx ? (float)(gi * sc) : 0.0f;
          const float gabs_f = kCplx ? sqrtf(fmaf(grs, grs, gis * gis)) : fabsf(grs);
          double tt, c, sn;
          float zf = 0.0f;
          const bool fp32_ok = ex > 0 && ex < 2046 && gabs_f > 1e-30f && g2 >= 1e-8 * a * b;
          if (fp32_ok) zf = 0.5f * (bs - as) / gabs_f;
          if (fp32_ok && fabsf(zf) < 1e18f) {
            const float az = fabsf(zf);
            const float tf = copysignf(1.0f / (az + sqrtf(fmaf(az, az, 1.0f))), zf);
            const float cf = rsqrtf(fmaf(tf, tf, 1.0f));
            const double c64 = (double)cf, s64 = (double)(cf * tf);
            const double d = fma(c64, c64, fma(s64, s64, -1.0));
            const double f = fma(d, fma(0.375, d, -0.5), 1.0);
            c = c64 * f;
            sn = s64 * f;
            tt = (double)tf;
          } else {
            // extremely graded pair (|g| below 1e-30 (a + b) or |zeta| >= 1e18):
            // the whole angle in FP64, rare
            const double zeta = 0.5 * (b - a) / sqrt(g2);
            const double az = fabs(zeta);
            tt = az < 1e150 ? 1.0 / (az + sqrt(fma(az, az, 1.0))) : 0.5 / az;
            tt = copysign(tt, zeta);
            c = 1.0 / sqrt(fma(tt, tt, 1.0));
            sn = c * tt;
          }
          double er, ei;
          if constexpr (kCplx) {
            if (fp32_ok) {
              const float inv = 1.0f / gabs_f;
              const double e_r = (double)(grs * inv), e_i = (double)(gis * inv);
              const double de = fma(e_r, e_r, fma(e_i, e_i, -1.0));
              const double fe = fma(de, fma(0.375, de, -0.5), 1.0);
              er = e_r * fe;
              ei = e_i * fe;
            } else {
              const double inv = 1.0 / sqrt(g2);
              er = gr * inv;
              ei = gi * inv;
            }
          } else {
            er = gr >= 0.0 ? 1.0 : -1.0;  // the phase of a real overlap is its sign
            ei = 0.0;
          }
          // closed-form norm update (approximate; exact norms return at the
          // first round of the next sweep)
          const double gabs = fp32_ok ? (double)gabs_f * sc_inv : sqrt(g2);
          na = fma(-tt, gabs, a);
          nb = fma(tt, gabs, b);
          Rot<T> R;
          R.set(c, sn, er, ei);
          if constexpr (E > 0) {
#pragma unroll
            for (int e = 0; e < E; ++e) {
              const int x = tid + NT * e;
              R.apply(u[e], v[e]);
              if (x < L) {
                stcg(rp + x, u[e]);
                stcg(rq + x, v[e]);
              }
            }
          } else {
            for (int x = tid; x < L; x += NT) {
              T uu = ldcg(rp + x), vv = ldcg(rq + x);
              R.apply(uu, vv);
              stcg(rp + x, uu);
              stcg(rq + x, vv);
            }
          }
          if (tid == 0) vflag[sweep & 1] = 1;
        }
        if (tid == 0 && rot) {
          __stcg(nrm + p, na);
          __stcg(nrm + q, nb);
        }
      }
      if (!grid_sync(ctl)) return;
    }
    if (tid == 0) sflag = vflag[sweep & 1];
    __syncthreads();
    if (sflag == 0) {
      if (blockIdx.x == 0 && tid == 0) ctl->sweeps = sweep + 1;
      return;
    }
  }
  if (blockIdx.x == 0 && tid == 0) {
    ctl->sweeps = max_sweeps;
    atomicOr(&ctl->status, DEV_NOT_CONVERGED);
  }
}

// s_i = |w_i|, one warp per row
// The FP64 splits square entries (row norms, overlaps, Householder norms) and
// square those again (the Jacobi's g^2 vs tol^2 a b test), which under- or
// overflows for matrices whose entries are far from 1 (the canonical form of a
// long random chain carries a scale of 1e-120 and below).  So, as LAPACK
// rescales its input, the split runs on the matrix times 2^-e, e the exponent
// of its largest entry: exact, so singular values and vectors scale back
// exactly.  k_max_exp takes e with an atomic max over the blocks (the word is
// set to 0x80808080, below every exponent, beforehand); scale_exp reads it
// back (0 for an all-zero or non-finite matrix, which the split reports).
__device__ __forceinline__ int scale_exp(const int* wexp) {
  const int e = *wexp;
  return (e < -1100 || e > 1100) ? 0 : e;
}

template <typename T>
__global__ void k_row_norms(const T* W, int ldw, int k, int l, double* nrm, int squared,
                            const int* wexp = nullptr) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x % 32;
  if (warp >= k) return;
  const T* w = W + (size_t)warp * ldw;
  double a = 0.0;
  for (int x = lane; x < l; x += 32) a += S<T>::abs2(ldcg(w + x));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  // rows scaled by 2^-e (see k_max_exp): the norm of the unscaled row
  if (lane == 0) nrm[warp] = squared ? a : (wexp ? ldexp(sqrt(a), scale_exp(wexp)) : sqrt(a));
}

template <typename T>
__global__ void k_max_exp(const T* __restrict__ X, int rows, int cols, int ldx, int* e_out) {
  int best = INT_MIN;
  const size_t total = (size_t)rows * cols;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const T v = X[(i / cols) * ldx + (i % cols)];
    double m;
    if constexpr (sizeof(T) == sizeof(double)) m = fabs((double)S<T>::real(v));
    else m = fmax(fabs(v.re), fabs(v.im));
    if (m > 0.0 && isfinite(m)) best = max(best, ilogb(m));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best != INT_MIN) atomicMax(e_out, best);
}

template <typename T>
__global__ void k_scale_exp(T* __restrict__ X, int rows, int cols, int ldx,
                            const int* __restrict__ wexp) {
  const int e = -scale_exp(wexp);
  if (e == 0) return;
  const size_t total = (size_t)rows * cols;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    T& v = X[(i / cols) * ldx + (i % cols)];
    if constexpr (sizeof(T) == sizeof(double)) v = ldexp((double)S<T>::real(v), e);
    else v = T{ldexp(v.re, e), ldexp(v.im, e)};
  }
}

// Scale the rows x cols block of X (leading dimension ldx) by 2^-e, e the
// exponent of its largest entry, kept in *wexp for the way back.
template <typename T>
int prescale(cudaStream_t st, T* X, int rows, int cols, int ldx, int* wexp) {
  const size_t total = (size_t)rows * cols;
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>((total + 255) / 256, 1024));
  SM_CUDA_CHECK(cudaMemsetAsync(wexp, 0x80, sizeof(int), st));
  k_max_exp<T><<<blocks, 256, 0, st>>>(X, rows, cols, ldx, wexp);
  k_scale_exp<T><<<blocks, 256, 0, st>>>(X, rows, cols, ldx, wexp);
  note_launch(2);
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
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

// Rank sort of the k non-negative keys (descending, stable by index) by k
// threads; writes perm, s_sorted (global) and ss (shared, may alias).
__device__ void rank_sort(const unsigned long long* keys, int k, int* perm, double* s_sorted,
                          double* ss) {
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    const unsigned long long ki = keys[i];
    int rank = 0;
    for (int j = 0; j < k; ++j) {
      const unsigned long long kj = keys[j];
      rank += (kj > ki) || (kj == ki && j < i);
    }
    perm[rank] = i;
    const double v = __longlong_as_double((long long)ki);
    s_sorted[rank] = v;
    ss[rank] = v;
  }
}

// Sort the k norms descending (stable by index), then truncate with the
// reference rule.  With `staged` the sorted values and the error table live in
// shared memory while the one-thread truncation rule runs over them (dynamic
// shared memory 24 k + 8 bytes instead of 8 k).
__global__ void k_sort_truncate(const double* nrm, int k, sm_strategy st, int* perm,
                                double* s_sorted, double* errors, const JacobiCtl* ctl,
                                SplitResult* res, int staged) {
  extern __shared__ unsigned long long keys[];
  double* ss = staged ? reinterpret_cast<double*>(keys + k) : s_sorted;
  double* er = staged ? ss + k : errors;
  for (int i = threadIdx.x; i < k; i += blockDim.x)
    keys[i] = (unsigned long long)__double_as_longlong(nrm[i]);
  __syncthreads();
  rank_sort(keys, k, perm, s_sorted, ss);
  __syncthreads();
  if (threadIdx.x == 0) {
    int D;
    double e;
    truncate_rule(ss, k, st, er, &D, &e);
    res->D = D;
    res->err2 = e;
    res->status = ctl ? ctl->status : 0;
    res->sweeps = ctl ? ctl->sweeps : 0;
    // non-finite input shows up as a NaN norm
    for (int i = 0; i < k; ++i)
      if (!(ss[i] == ss[i]) || ss[i] > DBL_MAX) res->status |= DEV_NONFINITE;
  }
  if (staged) {
    __syncthreads();
    for (int i = threadIdx.x; i <= k; i += blockDim.x) errors[i] = er[i];
  }
}

// Launches k_sort_truncate (one CTA of 1024 threads), staging in shared
// memory when 24 k + 8 bytes fit.
static int sort_truncate(cudaStream_t st, const double* nrm, int k, const sm_strategy& strat,
                         int* perm, double* s_sorted, double* errors, const JacobiCtl* ctl,
                         SplitResult* res) {
  constexpr size_t kLimit = 200 * 1024;
  const size_t keys = sizeof(unsigned long long) * (size_t)k;
  const size_t full = keys + sizeof(double) * (2 * (size_t)k + 1);
  const bool staged = full <= kLimit;
  const size_t smem = staged ? full : keys;
  if (smem > kLimit) {
    set_error("svd: matrix too large for the on-chip sort");
    return SM_ERR_VALUE;
  }
  if (smem > 48 * 1024) SM_CHECK(raise_smem_limit(k_sort_truncate, smem));
  k_sort_truncate<<<1, 1024, smem, st>>>(nrm, k, strat, perm, s_sorted, errors, ctl, res,
                                         staged ? 1 : 0);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

// Write the factors of the truncated SVD.  Element (i, j) of the left output
// (m x D) and (j, x) of the right output (D x n).
template <typename T>
__global__ void k_emit(int wide, int m, int n, int D, const T* __restrict__ W, int ldw,
                       const T* __restrict__ X, int ldx, const int* __restrict__ perm,
                       const double* __restrict__ s, int left_mode, T* __restrict__ left,
                       int right_mode, T* __restrict__ right, const int* wexp = nullptr) {
  // W's rows carry the prescale 2^-e (X's do not): normalising a W row takes
  // the singular value times 2^-e
  const int we = wexp ? -scale_exp(wexp) : 0;
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
        if (left_mode == OUT_U) v = sj > 0.0 ? S<T>::scale(v, 1.0 / ldexp(sj, we)) : S<T>::zero();
        else if (we) v = S<T>::scale(v, ldexp(1.0, -we));  // U s: undo the prescale
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
        if (right_mode == OUT_VT) v = sj > 0.0 ? S<T>::scale(v, 1.0 / ldexp(sj, we)) : S<T>::zero();
        else if (we) v = S<T>::scale(v, ldexp(1.0, -we));  // s V: undo the prescale
      } else {
        v = S<T>::conj(X[(size_t)pj * ldx + x]);
        if (right_mode == OUT_SVT) v = S<T>::scale(v, sj);
      }
      right[f] = v;
    }
  }
}

constexpr int kMaxSweeps = 60;

constexpr int kJacobiNT = 128;

// Deflation thresholds on a row's squared norm, relative to |A|_F^2 (rel) or
// absolute (abs), below which the strategy certainly discards the row's
// singular value: the relative-norm rule drops a tail of total weight up to
// tol |A|_F^2, so rows of at most 1e-6 tol |A|_F^2 / k each are dropped even
// all together; the singular-value rules drop s <= tol s_max (or <= tol), and
// |A|_F^2 <= k s_max^2.  No deflation without truncation or at tol = 0.
static void deflation(const sm_strategy& s, int k, double* rel, double* abs_) {
  // A deflated row keeps a singular value of at most sqrt(rel k) s_max that
  // the iteration no longer refines, so rel <= 1e-24 / k also bounds its
  // error by 1e-12 s_max.
  *rel = 0.0;
  *abs_ = 0.0;
  if (s.tolerance <= 0.0) return;
  if (s.method == SM_RELATIVE_NORM_SQUARED_ERROR) *rel = std::min(1e-24, 1e-6 * s.tolerance) / k;
  else if (s.method == SM_RELATIVE_SINGULAR_VALUE)
    *rel = std::min(1e-24, 1e-4 * s.tolerance * s.tolerance) / k;
  else if (s.method == SM_ABSOLUTE_SINGULAR_VALUE)
    *rel = 1e-24 / k;  // no absolute threshold: the iteration runs on prescaled values
}

template <typename T, int E>
int launch_jacobi(Ctx& ctx, cudaStream_t st, T* Wx, int ld, int k, int l, int L, double tol2,
                  int use_floor, double defl_rel, double defl_abs, double* nrm, const double* nrm0,
                  int* act, JacobiCtl* ctl) {
  const int npairs = (k + (k & 1)) / 2;
  const int sms = std::max(1, ctx.num_sms);
  auto fn = k_jacobi<T, kJacobiNT, E>;
  const void* key = reinterpret_cast<const void*>(fn);
  int per_sm = 0;
  const auto it = ctx.coop_blocks.find(key);
  if (it != ctx.coop_blocks.end()) per_sm = it->second;
  else {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kJacobiNT, 0) != cudaSuccess)
      per_sm = 1;
    per_sm = std::max(1, per_sm);
    ctx.coop_blocks[key] = per_sm;
  }
  // a context whose work shares the device with other streams runs the
  // iteration as one CTA: its grid barrier then never waits for CTAs that
  // other streams' kernels keep from being resident
  const int grid = ctx.concurrent ? 1 : std::max(1, std::min(npairs, per_sm * sms));
  int ms = kMaxSweeps;
  void* args[] = {&Wx, &ld, &k, &l, &L, &tol2, &use_floor, &defl_rel, &defl_abs, &ms, &nrm,
                  &nrm0, &act, &ctl};
  SM_CHECK(coop_launch(reinterpret_cast<const void*>(fn), dim3(grid), dim3(kJacobiNT), args, st));
  note_launch();
  return SM_OK;
}

// Rows of length L: l entries of the vector, then (L - l) accumulated-unitary
// entries (L = l + k when the short-side factor is accumulated, L = l when not).
template <typename T>
int run_jacobi(Ctx& ctx, cudaStream_t st, T* Wx, int ld, int k, int l, int L, double tol2,
               int use_floor, double defl_rel, double defl_abs, double* nrm, const double* nrm0,
               int* act, JacobiCtl* ctl) {
  const int need = (L + kJacobiNT - 1) / kJacobiNT;
#define SM_J(EV)                                                                              \
  return launch_jacobi<T, EV>(ctx, st, Wx, ld, k, l, L, tol2, use_floor, defl_rel, defl_abs, nrm, \
                              nrm0, act, ctl)
  if constexpr (sizeof(T) == sizeof(double)) {
    if (need <= 1) SM_J(1);
    if (need <= 2) SM_J(2);
    if (need <= 4) SM_J(4);
    if (need <= 6) SM_J(6);
    if (need <= 8) SM_J(8);
    if (need <= 10) SM_J(10);
    if (need <= 12) SM_J(12);
    if (need <= 16) SM_J(16);
  } else {
    if (need <= 1) SM_J(1);
    if (need <= 2) SM_J(2);
    if (need <= 4) SM_J(4);
    if (need <= 6) SM_J(6);
    if (need <= 8) SM_J(8);
  }
  SM_J(0);
#undef SM_J
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

// ---------------------------------------------------------------------------
// Rank-revealing Householder QR preconditioner (FP64, no pivoting).
//
// The one-sided Jacobi iteration on the rows of W (k x l) is replaced by the
// same iteration on the rows of R from W = Q R: both have the same singular
// values and right singular vectors, but the rows of R converge in fewer
// sweeps, and for a numerically rank-deficient W (a two-site tensor of rank
// ~chi inside a 2chi x 2chi matrix) the trailing rows of R are already at
// rounding level, so the Jacobi deflation drops them before the first sweep.
// The factorisation stops early once the trailing block holds at most `thr`
// of |W|_F^2, the weight the truncation rule certainly discards.
//
// Storage: Wt = W^T (l x k, row-major) so that every column of W is a
// contiguous row; one warp owns a column.  Step j applies the reflector
// H_j = I - tau v v^H (published in the previous step, double-buffered by
// step parity) to every column c > j; the warp owning column j + 1 then forms
// the next reflector.  One bounded grid barrier per step.
// ---------------------------------------------------------------------------
struct QrCtl {
  JacobiCtl bar;  // barrier words and status, shared layout with the Jacobi kernel
  int steps;      // reflections performed (the rank estimate)
  int pad;
  double tau[2];  // tau of the published reflector, by step parity
};

__device__ bool qr_grid_sync(QrCtl* ctl) { return grid_sync(&ctl->bar); }

// Reflector for x = Wt[c][j:k]: v = x + nu e1, nu = (x0/|x0|) |x|,
// tau = 1 / (|x| (|x| + |x0|)); writes v (v0 = x0 + nu) to vdst[j:k] and sets
// Wt[c][j] = -nu, the diagonal of R.  Executed by one warp.
template <typename T>
__device__ void qr_reflector(T* row, int j, int k, T* vdst, double* tau_out) {
  const int lane = threadIdx.x & 31;
  double nx2 = 0.0;
  for (int i = j + lane; i < k; i += 32) nx2 += S<T>::abs2(ldcg(row + i));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nx2 += __shfl_xor_sync(0xffffffffu, nx2, o);
  const T x0 = ldcg(row + j);
  const double nx = sqrt(nx2);
  const double a0 = sqrt(S<T>::abs2(x0));
  T nu;
  if (a0 > 0.0) nu = S<T>::scale(x0, nx / a0);
  else nu = S<T>::scale(S<T>::one(), nx);
  const double tau = nx > 0.0 ? 1.0 / (nx * (nx + a0)) : 0.0;
  for (int i = j + lane; i < k; i += 32) {
    T v = ldcg(row + i);
    if (i == j) v = v + nu;
    stcg(vdst + i, v);
  }
  __syncwarp();
  if (lane == 0) {
    stcg(row + j, S<T>::scale(nu, -1.0));
    *tau_out = tau;
  }
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_house_qr(T* Wt, int k, int l, double thr_rel,
                                                 T* vbuf, double* part, QrCtl* ctl) {
  constexpr int NW = NT / 32;
  __shared__ double wpart[NW];
  __shared__ int stop_flag;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gw = blockIdx.x * NW + warp, nw = gridDim.x * NW;
  const int nmax = k < l ? k : l;
  // |W|_F^2
  {
    double a = 0.0;
    for (int c = gw; c < l; c += nw)
      for (int i = lane; i < k; i += 32) a += S<T>::abs2(ldcg(Wt + (size_t)c * k + i));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) wpart[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < NW; ++w) t += wpart[w];
      __stcg(part + blockIdx.x, t);
    }
    // reflector 0 from column 0
    if (gw == 0) qr_reflector<T>(Wt, 0, k, vbuf, &ctl->tau[0]);
  }
  if (!qr_grid_sync(ctl)) return;
  // per-CTA partials summed by every warp in the same order (lane-strided,
  // then a fixed shuffle tree): a serial FP64 sum over 100+ CTAs costs
  // microseconds on GB300's FP64 unit
  double frob2 = 0.0;
  for (int b = lane; b < (int)gridDim.x; b += 32) frob2 += __ldcg(part + b);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) frob2 += __shfl_xor_sync(0xffffffffu, frob2, o);
  const double thr = thr_rel * frob2;
  int steps = nmax;
  for (int j = 0; j < nmax; ++j) {
    const T* v = vbuf + (size_t)(j & 1) * k;
    const double tau = ((volatile double*)ctl->tau)[j & 1];
    double trail = 0.0;
    for (int c = gw; c < l; c += nw) {
      if (c <= j) continue;
      T* row = Wt + (size_t)c * k;
      T w = S<T>::zero();
      for (int i = j + lane; i < k; i += 32) w = S<T>::cfma(ldcg(v + i), ldcg(row + i), w);
      double wr, wi;
      gamma_parts(w, wr, wi);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        wr += __shfl_xor_sync(0xffffffffu, wr, o);
        wi += __shfl_xor_sync(0xffffffffu, wi, o);
      }
      T tw;
      if constexpr (sizeof(T) == sizeof(double)) tw = tau * wr;
      else tw = cplx{tau * wr, tau * wi};
      for (int i = j + lane; i < k; i += 32) {
        // y -= tau (v^H y) v
        T y = ldcg(row + i);
        const T vi = ldcg(v + i);
        y = y - tw * vi;
        stcg(row + i, y);
        if (i > j) trail += S<T>::abs2(y);
      }
      if (c == j + 1 && j + 1 < nmax) {
        // this column's entries below row j were counted in the trailing
        // block above, before the next reflection moves them into R
        __syncwarp();
        qr_reflector<T>(row, j + 1, k, vbuf + (size_t)((j + 1) & 1) * k, &ctl->tau[(j + 1) & 1]);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) trail += __shfl_xor_sync(0xffffffffu, trail, o);
    if (lane == 0) wpart[warp] = trail;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < NW; ++w) t += wpart[w];
      __stcg(part + blockIdx.x, t);
    }
    if (!qr_grid_sync(ctl)) return;
    if (warp == 0) {
      double tot = 0.0;
      for (int b = lane; b < (int)gridDim.x; b += 32) tot += __ldcg(part + b);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
      if (lane == 0) stop_flag = tot <= thr;
    }
    __syncthreads();
    if (stop_flag) {
      steps = j + 1;
      break;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->steps = steps;
}

// Wx[i][c] = R[i][c] from Wt after `steps` reflections: row i < steps is the
// upper-triangular row of R; rows i >= steps are the trailing block rows.
template <typename T>
__global__ void k_qr_extract(const T* __restrict__ Wt, int k, int l, int kk, const QrCtl* ctl,
                             T* __restrict__ Wx, JacobiCtl* jctl) {
  const int steps = ctl->steps;
  // a QR barrier timeout is reported through the Jacobi status word
  if (blockIdx.x == 0 && threadIdx.x == 0 && ctl->bar.status)
    atomicOr(&jctl->status, ctl->bar.status);
  const size_t total = (size_t)kk * l;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / l), c = (int)(e % l);
    const int first = i < steps ? i : steps;
    Wx[e] = c >= first ? Wt[(size_t)c * k + i] : S<T>::zero();
  }
}

// Split where only one factor must be an isometry: U for (OUT_U, OUT_SVT)
// (left_orth_2site, right canonical update) and V for (OUT_US, OUT_VT).
// The Jacobi iteration then orthogonalises the vectors of that side -- the
// columns of A (rows of A^T) for U, the rows of A for V -- without
// accumulating a unitary: after convergence those vectors are s_i times the
// singular vectors, so the isometry is the normalised rows and the other
// factor is one FP64 GEMM, S V = U^H A or U S = A V^H.  Used when the
// orthogonalised side is also the short side (k = min(m, n)), which keeps
// the singular-value count and the truncation input identical to the full
// SVD's.
template <typename T>
int svd_split_xfree(Ctx& ctx, cudaStream_t st, const T* A, int m, int n, const sm_strategy& strat,
                    bool want_u, T* left, T* right, double* s_out, SplitResult* out) {
  // W (kw x l): its rows are orthogonalised -- W = A^T for U, W = A for V
  const int kw = want_u ? n : m;
  const int l = want_u ? m : n;
  const int k = std::min(kw, l);  // rows of R, = min(m, n) singular values
  const int ld = l;
  T *Wt, *Wx, *vbuf;
  double *nrm, *nrm0, *s_sorted, *errors, *qpart;
  int *perm, *act;
  JacobiCtl* ctl;
  QrCtl* qctl;
  SplitResult* res;
  SM_CHECK(ctx.scratch("svd.Wt", (size_t)l * kw, &Wt));
  SM_CHECK(ctx.scratch("svd.Wx", (size_t)k * ld, &Wx));
  SM_CHECK(ctx.scratch("svd.v", (size_t)2 * kw, &vbuf));
  SM_CHECK(ctx.scratch("svd.nrm", (size_t)k, &nrm));
  SM_CHECK(ctx.scratch("svd.nrm0", (size_t)k, &nrm0));
  SM_CHECK(ctx.scratch("svd.s", (size_t)k, &s_sorted));
  SM_CHECK(ctx.scratch("svd.err", (size_t)k + 1, &errors));
  SM_CHECK(ctx.scratch("svd.perm", (size_t)k, &perm));
  SM_CHECK(ctx.scratch("svd.act", (size_t)k, &act));
  SM_CHECK(ctx.scratch("svd.ctl", 1, &ctl));
  SM_CHECK(ctx.scratch("svd.qctl", 1, &qctl));
  SM_CHECK(ctx.scratch("svd.res", 1, &res));
  int* wexp;
  SM_CHECK(ctx.scratch("svd.wexp", 1, &wexp));
  // Wt = W^T (l x kw): A itself for U, A^T for V; then scaled to O(1) entries
  if (want_u) {
    SM_CUDA_CHECK(cudaMemcpyAsync(Wt, A, sizeof(T) * (size_t)m * n, cudaMemcpyDeviceToDevice, st));
  } else {
    SM_CHECK(transpose<T>(st, m, n, A, n, Wt, m));
  }
  SM_CHECK(prescale<T>(st, Wt, l, kw, kw, wexp));
  double drel, dabs;
  deflation(strat, k, &drel, &dabs);
  // rank-revealing QR preconditioner: W = Q R, R has k rows
  {
    constexpr int QNT = 128;
    auto fn = k_house_qr<T, QNT>;
    const void* key = reinterpret_cast<const void*>(fn);
    int per_sm = 0;
    const auto it = ctx.coop_blocks.find(key);
    if (it != ctx.coop_blocks.end()) per_sm = it->second;
    else {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, QNT, 0) != cudaSuccess) per_sm = 1;
      per_sm = std::max(1, per_sm);
      ctx.coop_blocks[key] = per_sm;
    }
    const int grid =
        ctx.concurrent
            ? 1  // one CTA: no grid barrier to wait on (see run_jacobi)
            : std::max(1, std::min((l + QNT / 32 - 1) / (QNT / 32), per_sm * std::max(1, ctx.num_sms)));
    SM_CHECK(ctx.scratch("svd.qpart", (size_t)grid, &qpart));
    SM_CUDA_CHECK(cudaMemsetAsync(qctl, 0, sizeof(QrCtl), st));
    int kk = kw, ll = l;
    void* args[] = {&Wt, &kk, &ll, &drel, &vbuf, &qpart, &qctl};
    SM_CHECK(coop_launch(reinterpret_cast<const void*>(fn), dim3(grid), dim3(QNT), args, st));
    note_launch();
    const size_t tot = (size_t)k * l;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((tot + 255) / 256, 4096));
    SM_CUDA_CHECK(cudaMemsetAsync(ctl, 0, sizeof(JacobiCtl), st));
    k_qr_extract<T><<<blocks, 256, 0, st>>>(Wt, kw, l, k, qctl, Wx, ctl);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
  }
  const double eps = DBL_EPSILON;
  bool use_floor = false;
  if (strat.method == SM_RELATIVE_NORM_SQUARED_ERROR)
    use_floor = strat.tolerance >= 64.0 * k * (double)l * eps * eps;
  else if (strat.method == SM_RELATIVE_SINGULAR_VALUE)
    use_floor = strat.tolerance >= 16.0 * std::sqrt((double)k * l) * eps;
  if (k >= 2) {
    k_row_norms<T><<<(k + 7) / 8, 256, 0, st>>>(Wx, ld, k, l, nrm0, 1);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    const double tol = std::sqrt((double)l) * DBL_EPSILON;
    if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
    SM_CHECK(run_jacobi<T>(ctx, st, Wx, ld, k, l, l, tol * tol, use_floor ? 1 : 0, drel, dabs, nrm,
                           nrm0, act, ctl));
    if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
    ctx.stats.jacobi_launches += 1;
    ctx.stats.jacobi_flops += (4.0 * std::max(m, n) * (double)k * k + 8.0 * (double)k * k * k) *
                              (sizeof(T) == sizeof(double) ? 1.0 : 4.0);
  }
  k_row_norms<T><<<(k + 7) / 8, 256, 0, st>>>(Wx, ld, k, l, nrm, 0, wexp);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  SM_CHECK(sort_truncate(st, nrm, k, strat, perm, s_sorted, errors, ctl, res));
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
  ctx.last_s = s_sorted;
  ctx.last_len = k;
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
  const T one = S<T>::one(), zero = S<T>::zero();
  // The closing GEMM reads A: when an output buffer overlaps A (the canonical
  // updates write the new site over the old one), stage both outputs.
  const char* a0 = reinterpret_cast<const char*>(A);
  const char* a1 = a0 + sizeof(T) * (size_t)m * n;
  auto overlaps = [&](const T* p, size_t count) {
    const char* p0 = reinterpret_cast<const char*>(p);
    return p0 < a1 && p0 + sizeof(T) * count > a0;
  };
  const size_t n_iso = want_u ? (size_t)m * D : (size_t)D * n;
  const size_t n_oth = want_u ? (size_t)D * n : (size_t)m * D;
  T* iso = want_u ? left : right;
  T* oth = want_u ? right : left;
  const bool stage = overlaps(iso, n_iso) || overlaps(oth, n_oth);
  T *iso_w = iso, *oth_w = oth;
  if (stage) {
    SM_CHECK(ctx.scratch("svd.iso", n_iso, &iso_w));
    SM_CHECK(ctx.scratch("svd.oth", n_oth, &oth_w));
  }
  const int blocks = (int)std::min<size_t>((n_iso + 255) / 256, 4096);
  if (want_u) {
    // U (m x D) = normalised rows of W^T; then S V (D x n) = U^H A
    k_emit<T><<<std::max(blocks, 1), 256, 0, st>>>(0, m, n, D, Wx, ld, Wx, ld, perm, s_sorted, OUT_U,
                                                   iso_w, 0, oth_w, wexp);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_C, SM_OP_N, D, n, m, one, iso_w, D, A, n, zero, oth_w, n));
  } else {
    // V (D x n) = normalised rows of W; then U S (m x D) = A V^H
    k_emit<T><<<std::max(blocks, 1), 256, 0, st>>>(1, m, n, D, Wx, ld, Wx, ld, perm, s_sorted, 0,
                                                   oth_w, OUT_VT, iso_w, wexp);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_N, SM_OP_C, m, D, n, one, A, n, iso_w, n, zero, oth_w, D));
  }
  if (stage) {
    SM_CUDA_CHECK(cudaMemcpyAsync(iso, iso_w, sizeof(T) * n_iso, cudaMemcpyDeviceToDevice, st));
    SM_CUDA_CHECK(cudaMemcpyAsync(oth, oth_w, sizeof(T) * n_oth, cudaMemcpyDeviceToDevice, st));
  }
  return SM_OK;
}

// ---------------------------------------------------------------------------
// Mixed-precision split (SM_PRECISION_MIXED): the cluster kernel of
// svd_mixed.cu gives the right singular vectors of W to FP32 accuracy; FP64
// GEMMs then refine them with the exact matrix:
//   1. the rows, normalised, are approximate eigenvectors of W^H W within the
//      row space the FP32 QR kept (it drops at most 1% of the weight the
//      tolerance allows).  A power step (rows of V W^H W) is NOT used: rows
//      whose sigma is below FP64 resolution relative to sigma_max would turn
//      into rounding-level copies of the dominant directions.
//   2. refinement of the approximate eigenvectors of W^H W (Ogita & Aishima,
//      "Iterative refinement for symmetric eigenvalue decomposition", Japan J.
//      Indust. Appl. Math. 35 (2018)): with G = V W^H W V^H and M = V V^H,
//      lambda_i = G_ii / M_ii, R = I - M,
//        E_ij = (G_ij + lambda_j R_ij) / (lambda_j - lambda_i)   (|E_ij| <= 1/4)
//        E_ij = R_ij / 2                                         (otherwise)
//      and V <- (I + E)^H V.  Each step squares the error for separated pairs;
//      nearly degenerate pairs are only re-orthonormalised, which leaves the
//      subspace they span unchanged.
//   3. sigma_i = |W v_i^H| from the final C = W V^H.  For the relative-norm
//      rule D is the smallest rank whose exact discarded weight
//      |A|_F^2 - sum_{kept} sigma_i^2 is within tolerance (this stays exact
//      where FP32 cannot resolve the individual small sigma_i); the singular
//      value rules apply the reference rule to these FP64 values.  The
//      factors are V's rows and C's columns, so the output never has to be
//      formed from A again.
// The caller falls back to the FP64 split (svd_split_xfree) when the cluster
// iteration did not converge, when the coupling left between a resolved kept
// and a dropped direction after the refinement could move the truncated
// matrix by more than 1e-6 |A|_F (a cut gap below the FP32 backward error), when a singular-value rule cuts below the FP32
// resolution (1e-4 s_max), or when the exact discarded weight breaks the
// strategy's tolerance while fewer than max_bond_dimension values are kept.
// ---------------------------------------------------------------------------
namespace {

constexpr int kMixedRefine = 2;    // refinement steps
constexpr double kMixedBlind = 1e-4;  // smallest kept s / s_max the FP32 stage resolves
constexpr double kMixedCutAmp = 1e-6;  // largest kept/dropped coupling (angle s_i / |A|)
constexpr double kMixedMinTol = 1e-14;   // smallest relative-norm tolerance taken in mixed
constexpr double kMixedRowFloor = 1e-12;  // FP32 rows lighter than this times |A|_F are dropped
constexpr double kMixedOrthMax = 0.25;    // largest |V V^H - I| entry a Newton-Schulz step takes
constexpr double kMixedNsOne = 3e-7;      // deviation after which one step reaches 1.4e-13
constexpr int kMixedNsMax = 5;            // Newton-Schulz steps at most
constexpr double kCapUseful = 0.8;        // largest predicted-rank cap applied, of min(m, n)

template <typename T>
__global__ void k_gather_rows(const T* __restrict__ rows, int l, const int* __restrict__ perm,
                              const double* __restrict__ s, int cnt, T* __restrict__ dst) {
  const size_t tot = (size_t)cnt * l;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / l), x = (int)(e % l);
    const double si = s[i];
    dst[e] = si > 0.0 ? S<T>::scale(rows[(size_t)perm[i] * l + x], 1.0 / si) : S<T>::zero();
  }
}

// X[i] /= nrm[i] (zero rows stay zero)
template <typename T>
__global__ void k_scale_rows(T* __restrict__ X, int k, int l, const double* __restrict__ nrm) {
  const size_t tot = (size_t)k * l;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot;
       e += (size_t)gridDim.x * blockDim.x) {
    const double r = nrm[e / l];
    X[e] = r > 0.0 ? S<T>::scale(X[e], 1.0 / r) : S<T>::zero();
  }
}

__device__ __forceinline__ double re_of(double x) { return x; }
__device__ __forceinline__ double re_of(cplx x) { return x.re; }

// F = (I + E)^H from G and M (k x k, Hermitian), E as described above.
// Pairs of rows that are both below FP32 resolution (lambda < blind2 *
// lambda_0; row 0 has the largest norm) are only re-orthonormalised
// (E = R / 2): their FP32 directions are rounding noise and a first-order
// rotation between them is meaningless; they are still decoupled from the
// resolved rows.
template <typename T>
__global__ void k_refine_matrix(const T* __restrict__ G, const T* __restrict__ M, int k,
                                double blind2, T* __restrict__ F) {
  const double m00 = re_of(M[0]);
  const double lmax = m00 > 0.0 ? re_of(G[0]) / m00 : 0.0;
  const size_t tot = (size_t)k * k;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / k), j = (int)(e % k);
    // F_ij = delta_ij + conj(E_ji)
    const double mii = re_of(M[(size_t)i * k + i]), mjj = re_of(M[(size_t)j * k + j]);
    const double li = mii > 0.0 ? re_of(G[(size_t)i * k + i]) / mii : 0.0;
    const double lj = mjj > 0.0 ? re_of(G[(size_t)j * k + j]) / mjj : 0.0;
    T Eji;
    if (i == j) {
      Eji = S<T>::from_real(0.5 * (1.0 - mii));
    } else if (li < blind2 * lmax && lj < blind2 * lmax) {
      Eji = S<T>::scale(S<T>::neg(M[(size_t)j * k + i]), 0.5);
    } else {
      const T r = S<T>::neg(M[(size_t)j * k + i]);  // R_ji = -M_ji
      const T num = G[(size_t)j * k + i] + S<T>::scale(r, li);
      const double gap = li - lj;
      if (gap != 0.0 && 16.0 * S<T>::abs2(num) <= gap * gap) Eji = S<T>::scale(num, 1.0 / gap);
      else Eji = S<T>::scale(r, 0.5);
    }
    T f = S<T>::conj(Eji);
    if (i == j) f = f + S<T>::one();
    F[e] = f;
  }
}

// F = 1.5 I - 0.5 M: one Newton-Schulz step X <- F X towards orthonormal rows;
// dev = max |M - I| over the grid (atomic max on the bits of the non-negative
// double; dev must be zero beforehand).
template <typename T>
__global__ void __launch_bounds__(256) k_ns_matrix(const T* __restrict__ M, int k,
                                                   T* __restrict__ F, double* dev) {
  __shared__ double red[8];
  const size_t tot = (size_t)k * k;
  double worst = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot;
       e += (size_t)gridDim.x * blockDim.x) {
    T f = S<T>::scale(M[e], -0.5);
    T d = M[e];
    if (e / k == e % k) {
      f = f + S<T>::from_real(1.5);
      d = d - S<T>::one();
    }
    F[e] = f;
    const double a = sqrt(S<T>::abs2(d));
    worst = a == a ? fmax(worst, a) : 1e300;
  }
  for (int o = 16; o > 0; o >>= 1) worst = fmax(worst, __shfl_xor_sync(0xffffffffu, worst, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = worst;
  __syncthreads();
  if (threadIdx.x == 0) {
    double w = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) w = fmax(w, red[i]);
    if (w > 0.0)
      atomicMax(reinterpret_cast<unsigned long long*>(dev),
                (unsigned long long)__double_as_longlong(w));
  }
}

// Block-wide (blockDim.x = 1024 >= n) inclusive prefix sums P[i] = sum_{j<=i}
// s[j]^2 in a fixed order (warp shuffles, then the warp totals): deterministic.
__device__ void block_prefix_sq(const double* s, int n, double* P, double* wsum) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  double v = t < n ? s[t] * s[t] : 0.0;
  for (int o = 1; o < 32; o <<= 1) {
    const double u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) wsum[w] = v;
  __syncthreads();
  if (w == 0) {
    double x = wsum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const double u = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += u;
    }
    wsum[lane] = x;  // inclusive scan of the warp totals
  }
  __syncthreads();
  if (t < n) P[t] = v + (w ? wsum[w - 1] : 0.0);
  __syncthreads();
}

// Rank and bookkeeping of a mixed split from its n sorted values ss (shared)
// and their prefix sums P (shared), all 1024 threads.  Relative-norm-squared
// rule with exact weights (exact_rule): D = the smallest rank whose discarded
// weight |A|^2 - P[D-1] is at most tol |A|^2 (|A|^2 = info[0], summed in FP64
// from A itself); the singular-value rules: the first i >= 1 with s_i at or
// below tol s_0 (relative) or tol (absolute); D is clamped to [1,
// max_bond_dimension] (cython/truncation.pxi:251-327 states the same
// contracts through the sorted values).  Writes res (D, err2 = |A|^2 -
// P[D-1], status from ctl plus non-finite values), info[2] = s_0, info[3] =
// s_{D-1} and info[7] = |A|^2 - P[n-1] (the weight outside the rows' span);
// returns D to every thread.
__device__ int mixed_rank_block(const double* ss, const double* P, int n, const sm_strategy& st,
                                int exact_rule, const JacobiCtl* ctl, SplitResult* res,
                                double* info, int* shD, int* shBad) {
  const int t = threadIdx.x;
  const int maxb = st.max_bond_dimension;
  const double total = info[0];
  if (t == 0) {
    *shD = 0x7fffffff;
    *shBad = 0;
  }
  __syncthreads();
  if (t < n) {
    bool cand = false;
    int D = 0;
    if (st.method == SM_DO_NOT_TRUNCATE) {
    } else if (exact_rule) {
      cand = total - P[t] <= st.tolerance * total;
      D = t + 1;
    } else {
      const double max_error =
          st.method == SM_RELATIVE_SINGULAR_VALUE ? st.tolerance * ss[0] : st.tolerance;
      cand = t >= 1 && ss[t] <= max_error;
      D = t;
    }
    if (cand) atomicMin(shD, D);
    if (!(ss[t] == ss[t]) || ss[t] > DBL_MAX) atomicOr(shBad, 1);
  }
  __syncthreads();
  int D = *shD == 0x7fffffff ? n : *shD;
  D = max(1, min(D, maxb));
  if (t == 0) {
    res->D = D;
    res->err2 = fmax(0.0, total - (D <= n ? P[D - 1] : P[n - 1]));
    res->status = (ctl ? ctl->status : 0) | (*shBad ? DEV_NONFINITE : 0);
    res->sweeps = ctl ? ctl->sweeps : 0;
    info[2] = ss[0];
    info[3] = ss[min(D, n) - 1];
    info[7] = fmax(0.0, total - P[n - 1]);
  }
  return D;
}

// First step of a mixed split, one CTA of 1024 threads (n <= 1024): the FP32
// rows' norms sorted descending (perm, s_sorted) and mixed_rank_block on them
// (the host uses info[2], info[3] and the status); ctl->nkeep = the number of
// rows of norm at least row_floor |A|_F (the lighter rows, each below 1e-24
// of |A|^2 and far below FP32 resolution, are left out of the refinement);
// info[8] = 0 for the orthonormality measure of k_ns_matrix.  Dynamic shared
// memory: 24 n bytes.
__global__ void __launch_bounds__(1024) k_mixed_sort(const double* __restrict__ nrm, int n,
                                                     sm_strategy st, int exact_rule,
                                                     JacobiCtl* ctl, double row_floor, int* perm,
                                                     double* s_sorted, SplitResult* res,
                                                     double* info) {
  extern __shared__ unsigned long long keys[];
  double* ss = reinterpret_cast<double*>(keys + n);
  double* P = ss + n;
  __shared__ double wsum[32];
  __shared__ int shD, shBad;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    keys[i] = (unsigned long long)__double_as_longlong(nrm[i]);
  __syncthreads();
  rank_sort(keys, n, perm, s_sorted, ss);
  __syncthreads();
  block_prefix_sq(ss, n, P, wsum);
  mixed_rank_block(ss, P, n, st, exact_rule, ctl, res, info, &shD, &shBad);
  const double floor = row_floor * sqrt(fmax(info[0], 0.0));
  const int t = threadIdx.x;
  if (t == 0) {
    info[8] = 0.0;
    if (!(ss[0] >= floor)) ctl->nkeep = 0;
  }
  if (t < n && ss[t] >= floor && (t + 1 == n || !(ss[t + 1] >= floor))) ctl->nkeep = t + 1;
}

// Final step of a mixed split, one CTA of 1024 threads, on G = C^H C of the
// refined rows (C = W V^H, kw x cnt):
//  * s_j = |C[:, j]| = sqrt(G_jj), sorted descending (perm);
//  * mixed_rank_block: the rank (exact weights for the relative-norm rule:
//    s_j^2 are Rayleigh quotients of orthonormal rows), err2, status, info[2],
//    info[3], info[7];
//  * info[4] = 0 for the coupling check that k_mixed_coupling runs next.
// Dynamic shared memory: 24 cnt bytes.
template <typename T>
__global__ void __launch_bounds__(1024) k_mixed_final(const T* __restrict__ G, int cnt,
                                                      sm_strategy st, int exact_rule, double blind,
                                                      const JacobiCtl* ctl, int* perm,
                                                      double* s_sorted, double* errors,
                                                      SplitResult* res, double* info) {
  extern __shared__ unsigned long long keys[];
  double* ss = reinterpret_cast<double*>(keys + cnt);
  double* P = ss + cnt;
  __shared__ double red[32];
  __shared__ int shD, shBad;
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
    const double g = fmax(0.0, S<T>::real(G[(size_t)i * cnt + i]));
    keys[i] = (unsigned long long)__double_as_longlong(sqrt(g));
  }
  __syncthreads();
  rank_sort(keys, cnt, perm, s_sorted, ss);
  __syncthreads();
  block_prefix_sq(ss, cnt, P, red);
  mixed_rank_block(ss, P, cnt, st, exact_rule, ctl, res, info, &shD, &shBad);
  (void)errors;
  (void)blind;
  if (threadIdx.x == 0) info[4] = 0.0;
}

// Coupling check of a mixed split (after k_mixed_final), over the whole grid:
// info[4] = the largest state change left by the coupling between a kept row
// a and a dropped row b, angle |G_ab| / (lambda_a - lambda_b) (lambda = s^2)
// times s_a / |A|_F; its square bounds the fidelity error the split can add.
// Pairs whose both values lie below the FP32 resolution (s < blind s_0) are
// skipped: which of two unresolved directions is kept does not matter once
// the kept weight is exact.  The maximum goes into info[4] by an atomic max on
// the bits of the non-negative double (order-independent).
template <typename T>
__global__ void __launch_bounds__(256) k_mixed_coupling(const T* __restrict__ G, int cnt,
                                                        const int* __restrict__ perm,
                                                        const double* __restrict__ ss,
                                                        const SplitResult* __restrict__ res,
                                                        double blind, double* info) {
  __shared__ double red[8];
  const int D = min(res->D, cnt);
  const double sb = blind * ss[0];
  const double rnorm = info[0] > 0.0 ? 1.0 / sqrt(info[0]) : 0.0;
  double worst = 0.0;
  const long pairs = (long)D * (cnt - D);
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < pairs;
       e += (long)gridDim.x * blockDim.x) {
    const int a = (int)(e / (cnt - D)), b = D + (int)(e % (cnt - D));
    if (ss[a] < sb && ss[b] < sb) continue;
    const double gap = ss[a] * ss[a] - ss[b] * ss[b];
    const double g = sqrt(S<T>::abs2(G[(size_t)perm[a] * cnt + perm[b]]));
    const double th = gap > 0.0 ? g / gap : (g > 0.0 ? 1e300 : 0.0);
    worst = fmax(worst, th * ss[a] * rnorm);
  }
  for (int o = 16; o > 0; o >>= 1) worst = fmax(worst, __shfl_xor_sync(0xffffffffu, worst, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = worst;
  __syncthreads();
  if (threadIdx.x == 0) {
    double w = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) w = fmax(w, red[i]);
    if (w > 0.0)
      atomicMax(reinterpret_cast<unsigned long long*>(info + 4),
                (unsigned long long)__double_as_longlong(w));
  }
}

// Factors from the refined rows V (cnt x l) and C = W V^H (kw x cnt).
template <typename T>
__global__ void k_emit_mixed(int want_u, int m, int n, int D, const T* __restrict__ V, int l,
                             const T* __restrict__ C, int cnt, const int* __restrict__ perm,
                             T* __restrict__ iso, T* __restrict__ oth) {
  const size_t niso = want_u ? (size_t)m * D : (size_t)D * n;
  const size_t noth = want_u ? (size_t)D * n : (size_t)m * D;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < niso + noth;
       e += (size_t)gridDim.x * blockDim.x) {
    if (e < niso) {
      if (want_u) {  // U[i][j] = V[perm j][i]
        const int i = (int)(e / D), j = (int)(e % D);
        iso[e] = V[(size_t)perm[j] * l + i];
      } else {  // Vh[j][x] = V[perm j][x]
        const int j = (int)(e / n), x = (int)(e % n);
        iso[e] = V[(size_t)perm[j] * l + x];
      }
    } else {
      const size_t f = e - niso;
      if (want_u) {  // SV[j][x] = C[x][perm j]
        const int j = (int)(f / n), x = (int)(f % n);
        oth[f] = C[(size_t)x * cnt + perm[j]];
      } else {  // US[i][j] = C[i][perm j]
        const int i = (int)(f / D), j = (int)(f % D);
        oth[f] = C[(size_t)i * cnt + perm[j]];
      }
    }
  }
}

inline int grid_for(size_t tot) { return (int)std::max<size_t>(1, std::min<size_t>((tot + 255) / 256, 4096)); }

// Largest discarded weight the strategy allows with D of k values kept
// (the exact check that sends a mixed split back to the FP64 path).
double allowed_discard(const sm_strategy& st, double norm2, double s0, int k, int D) {
  const int drop = std::max(0, k - D);
  switch (st.method) {
    case SM_RELATIVE_NORM_SQUARED_ERROR: return st.tolerance * norm2;
    case SM_RELATIVE_SINGULAR_VALUE: return drop * (st.tolerance * s0) * (st.tolerance * s0);
    case SM_ABSOLUTE_SINGULAR_VALUE: return drop * st.tolerance * st.tolerance;
    default: return 0.0;
  }
}

}  // namespace

// rf_k > 0 (real operands): instead of factoring W, the cluster factors
// BH = W^T Q (l x rf_k) of a randomized range finder (rangefinder.cu) sized by
// the predicted rank; its rows (length rf_k) map back to W's right singular
// vectors by one product with BH^T, and everything after (refinement against
// the exact W, exact discarded weight, redo when the subspace missed weight the
// rank needs) is shared with the QR path, the range finder playing the capped
// QR's part (qr_cap = rf_k).
template <typename T>
int svd_split_mixed(Ctx& ctx, cudaStream_t st, const T* A, int m, int n, const sm_strategy& strat,
                    bool want_u, T* left, T* right, SplitResult* out, bool* done, int qr_cap,
                    bool* missed_out, int rf_k = 0, const int* cap_dev = nullptr) {
  *done = false;
  *missed_out = false;
  const int kw = want_u ? n : m;
  const int l = want_u ? m : n;
  const int k = std::min(kw, l);
  if (k < kMixedMinRank || strat.method == SM_DO_NOT_TRUNCATE || strat.tolerance <= 0.0)
    return SM_OK;
  if constexpr (sizeof(T) != sizeof(double)) rf_k = 0;
  if (rf_k > 0 && (rf_k >= k || rf_k > range_finder_max_k() || !split_cluster_fits<T>(l, rf_k)))
    rf_k = 0;
  // the matrix the cluster factors: W (kw x l), or BH (l x rf_k)
  const int ckw = rf_k > 0 ? l : kw, cl = rf_k > 0 ? rf_k : l;
  if (rf_k > 0) qr_cap = rf_k;
  if (rf_k == 0 && !split_cluster_fits<T>(kw, l)) return SM_OK;
  // the exact-weight rank rule resolves discarded weights down to the FP64
  // rounding of |A|^2 - kept (~ k eps |A|^2): tighter relative tolerances
  // take the FP64 path (counted as a fallback)
  if (strat.method == SM_RELATIVE_NORM_SQUARED_ERROR && strat.tolerance < kMixedMinTol) {
    ctx.stats.mixed_splits += 1;
    ctx.stats.mixed_fallbacks += 1;
    return SM_OK;
  }
  const int kcap = std::min(ckw, cl) + 32;  // the Jacobi writes 32 blocks of ceil(rows / 32)
  T *rows, *V0, *V1, *Cb, *Gb, *Mb, *Fb;
  double *nrm, *s_sorted, *errors, *info, *cn;
  int* perm;
  JacobiCtl* ctl;
  SplitResult* res;
  SM_CHECK(ctx.scratch("mx.rows", (size_t)kcap * cl, &rows));
  SM_CHECK(ctx.scratch("mx.nrm", (size_t)kcap, &nrm));
  SM_CHECK(ctx.scratch("mx.s", (size_t)kcap, &s_sorted));
  SM_CHECK(ctx.scratch("mx.err", (size_t)kcap + 1, &errors));
  SM_CHECK(ctx.scratch("mx.perm", (size_t)kcap, &perm));
  SM_CHECK(ctx.scratch("mx.info", 16, &info));
  SM_CHECK(ctx.scratch("mx.ctl", 1, &ctl));
  float* vbuf;
  SM_CHECK(ctx.scratch("mx.vbuf", split_cluster_vbuf_floats(ckw), &vbuf));
  SM_CHECK(ctx.scratch("mx.res", 1, &res));
  // RRQR stop: drop at most 1% of what the tolerance allows (never more than
  // 1e-10 of |A|^2, which the power step then suppresses further)
  double thr_rel = 0.0, thr_abs = 0.0;
  if (strat.method == SM_RELATIVE_NORM_SQUARED_ERROR) thr_rel = std::min(1e-10, 1e-2 * strat.tolerance);
  else if (strat.method == SM_RELATIVE_SINGULAR_VALUE)
    thr_rel = std::min(1e-10, 1e-2 * strat.tolerance * strat.tolerance);
  else thr_abs = 1e-2 * strat.tolerance * strat.tolerance;
  // The FP32 trailing-weight estimate is rounding noise below ~1e-7 |W|^2, so
  // a QR that stops on it can leave weight that the exact FP64 check finds
  // over the tolerance (the tolerance-limited splits of the n=30 chi=256
  // workload at tol 1e-12 did).  The redo of such a split (qr_cap = min(m, n))
  // therefore runs the full QR.
  if (qr_cap >= std::min(m, n)) thr_rel = thr_abs = 0.0;
  SM_CUDA_CHECK(cudaMemsetAsync(ctl, 0, sizeof(JacobiCtl), st));
  // a predicted rank caps the rank-revealing QR (qr_cap rows of R), or sizes
  // the range finder
  if (qr_cap > 0) ctx.stats.mixed_capped += 1;
  T* BH = nullptr;
  if constexpr (sizeof(T) == sizeof(double)) {
    if (rf_k > 0) {
      int* rf_status;
      double* a2;
      SM_CHECK(ctx.scratch("rf.BH", (size_t)l * rf_k, &BH));
      SM_CHECK(ctx.scratch("rf.status", 1, &rf_status));
      SM_CHECK(ctx.scratch("rf.a2", 2, &a2));
      ctx.stats.rf_splits += 1;
      SM_CHECK(range_finder_bh(ctx, st, A, m, n, want_u, rf_k, ctx.rf_power, BH, rf_status));
      if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
      // BH (l x rf_k) is the cluster's W; A's own |A|^2 replaces |BH|^2 below
      // no column pivoting here: W^T Q's columns come in the sketch's order, and
      // pivoting them cost the range finder a redo per split (measured)
      SM_CHECK(split_cluster_f32<T>(st, BH, l, rf_k, false, thr_rel, thr_abs, 40, rows, nrm,
                                    kcap, ctl, info, 0, vbuf, false));
      if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
      SM_CHECK(vdot<T>(ctx, st, (size_t)m * n, A, A, a2));
      SM_CUDA_CHECK(cudaMemcpyAsync(info, a2, sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
  }
  if (rf_k == 0) {
    if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
    SM_CHECK(split_cluster_f32<T>(st, A, m, n, want_u, thr_rel, thr_abs, 40, rows, nrm, kcap, ctl,
                                  info, qr_cap, vbuf, true, cap_dev));
    if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
  }
  struct Head {
    JacobiCtl c;
    double info[7];
  };
  // FP32 singular values: sorted, and the rank the rule gives on them; for the
  // singular-value rules a cut below the FP32 resolution sends the split to
  // the FP64 path right away
  const bool exact_rule = strat.method == SM_RELATIVE_NORM_SQUARED_ERROR;
  k_mixed_sort<<<1, 1024, 3 * sizeof(double) * (size_t)kcap, st>>>(
      nrm, kcap, strat, exact_rule ? 1 : 0, ctl, kMixedRowFloor, perm, s_sorted, res, info);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  Head* h = reinterpret_cast<Head*>(ctx.pinned);
  SM_CUDA_CHECK(cudaMemcpyAsync(&h->c, ctl, sizeof(JacobiCtl), cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaMemcpyAsync(h->info, info, 7 * sizeof(double), cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  const double norm2 = h->info[0];  // the pinned block is reused below
  const JacobiCtl hc = h->c;
  if (cap_dev) {  // the cap the predictor set on the device, now known here
    qr_cap = hc.cap;
    if (qr_cap > 0) ctx.stats.mixed_capped += 1;
    ctx.stats.rank_predicted_sum += hc.pred;
    ctx.stats.rank_predictions += 1;
  }
  ctx.stats.mixed_splits += 1;
  ctx.stats.cluster_qr_ms += h->info[5];
  ctx.stats.cluster_jacobi_ms += h->info[6];
  if (ctx.timing) {
    float ms = 0.f;
    SM_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
    ctx.stats.cluster_ms += ms;
  }
  ctx.stats.jacobi_sweeps += hc.sweeps;
  {  // algorithmic FP32 work of the launch (QR reflectors, then Jacobi pairs x sweeps)
    const int keff = hc.nact;
    double fl = 0.0;
    for (int j = 0; j < keff; ++j) fl += 4.0 * (ckw - j) * std::max(0, cl - j - 1);
    const double rows = 32.0 * ((keff + 31) / 32);  // the Jacobi's 32 blocks, zero rows included
    fl += 12.0 * cl * (rows * (rows - 1) / 2) * hc.sweeps;
    const double cf = sizeof(T) == sizeof(double) ? 1.0 : 4.0;
    ctx.stats.cluster_flops += cf * fl;
    // the split's algorithmic SVD work, 4 m n^2 + 8 n^3 (m >= n), and its
    // algorithmic bytes: the matrix read once, the converged rows written
    const double mm = std::max(m, n), nn = std::min(m, n);
    ctx.stats.cluster_alg_flops += cf * (4.0 * mm * nn * nn + 8.0 * nn * nn * nn);
    ctx.stats.cluster_bytes += (double)sizeof(T) * ((double)ckw * cl + (double)keff * cl);
  }
  if (hc.status != 0 || (!exact_rule && h->info[3] < kMixedBlind * h->info[2])) {
    ctx.stats.mixed_fallbacks += 1;
    ctx.stats.mixed_fallback_fp32 += 1;
    if (hc.status != 0) ctx.stats.mixed_fallback_unconverged += 1;
    return SM_OK;
  }
  const int cnt = std::max(1, std::min(std::min(hc.nact, hc.nkeep), std::min(ckw, cl)));
  ctx.stats.mixed_rows += cnt;
  SM_CHECK(ctx.scratch("mx.V0", (size_t)cnt * l, &V0));
  SM_CHECK(ctx.scratch("mx.V1", (size_t)cnt * l, &V1));
  SM_CHECK(ctx.scratch("mx.C", (size_t)kw * cnt, &Cb));
  SM_CHECK(ctx.scratch("mx.G", (size_t)cnt * cnt, &Gb));
  SM_CHECK(ctx.scratch("mx.M", (size_t)cnt * cnt, &Mb));
  SM_CHECK(ctx.scratch("mx.F", (size_t)cnt * cnt, &Fb));
  SM_CHECK(ctx.scratch("mx.cn", (size_t)cnt, &cn));
  const T one = S<T>::one(), zero = S<T>::zero();
  if (rf_k == 0) {
    // rows by decreasing norm (sorted above), normalised
    k_gather_rows<T><<<grid_for((size_t)cnt * l), 256, 0, st>>>(rows, l, perm, s_sorted, cnt, V0);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
  } else {
    // the rows of U_B^T (sorted, normalised), then W's right singular vectors
    // U_B^T B = U_B^T BH^T (rows of norm sigma), normalised below
    k_gather_rows<T><<<grid_for((size_t)cnt * rf_k), 256, 0, st>>>(rows, rf_k, perm, s_sorted, cnt,
                                                                    V1);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_N, SM_OP_C, cnt, l, rf_k, one, V1, rf_k, BH, rf_k, zero, V0,
                         l));
  }
  // C = W V^H (kw x cnt)
  auto w_vh = [&](const T* V, T* C) -> int {
    if (want_u) return gemm_ctx<T>(ctx, st, SM_OP_T, SM_OP_C, n, cnt, m, one, A, n, V, m, zero, C, cnt);
    return gemm_ctx<T>(ctx, st, SM_OP_N, SM_OP_C, m, cnt, n, one, A, n, V, n, zero, C, cnt);
  };
  auto normalise = [&](T* X) -> int {
    k_row_norms<T><<<(cnt + 7) / 8, 256, 0, st>>>(X, l, cnt, l, cn, 0);
    note_launch();
    k_scale_rows<T><<<grid_for((size_t)cnt * l), 256, 0, st>>>(X, cnt, l, cn);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    return SM_OK;
  };
  if (rf_k > 0) SM_CHECK(normalise(V0));
  // 2. refinement (V0 holds the normalised FP32 rows)
  T* V = V0;
  T* Vn = V1;
  // the range finder's rows come from the small side (U_B^T Q, length rf_k):
  // mapping them to W's row space multiplies their FP32 error by the condition
  // of the kept spectrum (1e-7 (s_max / s_i)^2 on a row of singular value s_i,
  // against 1e-7 s_max / s_i for rows that the Jacobi forms in W's row space),
  // which two more quadratically convergent steps take back to FP64 level
  const int refine_steps = rf_k > 0 ? kMixedRefine + 2 : kMixedRefine;
  for (int it = 0; it < refine_steps; ++it) {
    SM_CHECK(w_vh(V, Cb));
    SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_C, SM_OP_N, cnt, cnt, kw, one, Cb, cnt, Cb, cnt, zero, Gb, cnt));
    SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_N, SM_OP_C, cnt, cnt, l, one, V, l, V, l, zero, Mb, cnt));
    k_refine_matrix<T><<<grid_for((size_t)cnt * cnt), 256, 0, st>>>(Gb, Mb, cnt,
                                                                    kMixedBlind * kMixedBlind, Fb);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_N, SM_OP_N, cnt, l, cnt, one, Fb, cnt, V, l, zero, Vn, l));
    std::swap(V, Vn);
  }
  // Newton-Schulz steps V <- (1.5 I - 0.5 V V^H) V take the largest
  // deviation e of V V^H from I to about 1.5 e^2.  Two refinement steps leave
  // e below kMixedNsOne for resolved rows (one step then reaches FP64 level);
  // rows below FP32 resolution that a tolerance-limited cut keeps leave up to
  // ~1e-5 and take a second step; the range finder's rows beyond the rank
  // (noise of the sketch) a few more.  A deviation beyond kMixedOrthMax, or one
  // that a step did not reduce, means rows that the FP32 stage left nearly
  // parallel: the split goes to FP64.
  // a capped QR (the predicted rank, or the range finder's k) that missed
  // weight the rank needs is redone by the caller with the full QR
  const bool capped = qr_cap > 0 && qr_cap < k;
  SM_CHECK(normalise(V));
  double e_ns = 0.0;
  bool ns_done = false;
  double* hdev = reinterpret_cast<double*>(ctx.pinned) + 512;
  for (int ns = 0; ns < kMixedNsMax; ++ns) {
    SM_CUDA_CHECK(cudaMemsetAsync(info + 8, 0, sizeof(double), st));
    SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_N, SM_OP_C, cnt, cnt, l, one, V, l, V, l, zero, Mb, cnt));
    k_ns_matrix<T><<<grid_for((size_t)cnt * cnt), 256, 0, st>>>(Mb, cnt, Fb, info + 8);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    SM_CUDA_CHECK(cudaMemcpyAsync(hdev, info + 8, sizeof(double), cudaMemcpyDeviceToHost, st));
    SM_CUDA_CHECK(cudaStreamSynchronize(st));
    const double e_prev = ns ? e_ns : kMixedOrthMax;
    e_ns = *hdev;
    if (!(e_ns <= e_prev)) break;
    SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_N, SM_OP_N, cnt, l, cnt, one, Fb, cnt, V, l, zero, Vn, l));
    std::swap(V, Vn);
    SM_CHECK(normalise(V));
    ctx.stats.mixed_ns_steps += 1;
    if (e_ns <= kMixedNsOne) {
      ns_done = true;
      break;
    }
  }
  if (!ns_done && capped) {  // rows of a missed subspace: no use finishing this attempt
    ctx.stats.mixed_cap_redone += 1;
    *missed_out = true;
    return SM_OK;
  }
  // 3. singular values, truncation, exact discarded weight
  SM_CHECK(w_vh(V, Cb));
  SM_CHECK(gemm_ctx<T>(ctx, st, SM_OP_C, SM_OP_N, cnt, cnt, kw, one, Cb, cnt, Cb, cnt, zero, Gb, cnt));
  const size_t fin_smem = sizeof(double) * 3 * (size_t)cnt;
  if (fin_smem > 48 * 1024) SM_CHECK(raise_smem_limit(k_mixed_final<T>, fin_smem));
  k_mixed_final<T><<<1, 1024, fin_smem, st>>>(Gb, cnt, strat, exact_rule ? 1 : 0, kMixedBlind, ctl,
                                              perm, s_sorted, errors, res, info);
  {
    const long maxpairs = (long)(cnt / 2) * (cnt - cnt / 2);  // D (cnt - D) at its largest
    const int cb = (int)std::max(1L, std::min((maxpairs + 255) / 256, 4L * ctx.num_sms));
    k_mixed_coupling<T><<<cb, 256, 0, st>>>(Gb, cnt, perm, s_sorted, res, kMixedBlind, info);
  }
  note_launch(2);
  SM_CUDA_CHECK(cudaGetLastError());
  SplitResult* hr = reinterpret_cast<SplitResult*>(ctx.pinned);
  SM_CUDA_CHECK(cudaMemcpyAsync(hr, res, sizeof(SplitResult), cudaMemcpyDeviceToHost, st));
  double* hs = reinterpret_cast<double*>(hr + 1);
  SM_CUDA_CHECK(cudaMemcpyAsync(hs, info + 2, 6 * sizeof(double), cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  const double s0 = hs[0];
  const SplitResult r = *hr;
  const int D = r.D;
  // FP32 resolves a singular vector only down to ~1e-4 s_max (the refinement
  // needs the FP32 error below 1/4 of the relative gap): a cut below that, or a
  // discarded weight beyond the tolerance with fewer than max_bond values
  // kept, sends the split to the FP64 path.
  const double s_last = hs[1];
  const double cut_angle = hs[2];
  const bool blind = !exact_rule && s_last < kMixedBlind * s0;
  // a capped QR that left weight the rank may need: more than 1% of what the
  // tolerance allows (and more than 1e-12 of |A|^2) outside the rows' span,
  // computed exactly after the refinement
  const bool missed = capped && hs[5] > std::max(1e-12, 1e-2 * strat.tolerance) * norm2;
  const bool coupled = !(cut_angle <= kMixedCutAmp);
  const bool over_tol = r.err2 > allowed_discard(strat, norm2, s0, k, D) * (1.0 + 1e-12);
  const bool over = D < strat.max_bond_dimension && D < k && over_tol;
  // The Newton-Schulz steps must have converged, and a split that keeps every
  // value leaves nothing to discard: either failing means the FP32 stage lost
  // directions, and the split goes to FP64.
  const bool lost = !ns_done || (D >= k && over_tol);
  if (capped && !blind && (missed || over || coupled || lost)) {
    // the cap left weight the rank needs (then the rows span the wrong space
    // and every later check may fail with it): the caller retries with the
    // full QR; a split without a cap goes to FP64 instead
    ctx.stats.mixed_cap_redone += 1;
    *missed_out = true;
    return SM_OK;
  }
  if (blind || coupled || over || lost) {
    ctx.stats.mixed_fallbacks += 1;
    if (coupled) ctx.stats.mixed_fallback_cut += 1;
    else ctx.stats.mixed_fallback_fp32 += 1;
    if (over && !coupled && !blind) ctx.stats.mixed_fallback_over += 1;
    return SM_OK;
  }
  T* iso = want_u ? left : right;
  T* oth = want_u ? right : left;
  const size_t tot = (size_t)D * (m + n);
  k_emit_mixed<T><<<grid_for(tot), 256, 0, st>>>(want_u ? 1 : 0, m, n, D, V, l, Cb, cnt, perm, iso,
                                                 oth);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  *out = r;
  out->status = 0;
  ctx.stats.splits += 1;
  ctx.last_s = s_sorted;
  ctx.last_len = cnt;
  if (ctx.trace) {
    const size_t off = ctx.tr_s.size();
    ctx.tr_s.resize(off + cnt);
    SM_CUDA_CHECK(cudaMemcpyAsync(ctx.tr_s.data() + off, s_sorted, sizeof(double) * cnt,
                                  cudaMemcpyDeviceToHost, st));
    SM_CUDA_CHECK(cudaStreamSynchronize(st));
    ctx.tr_rank.push_back(D);
    ctx.tr_len.push_back(cnt);
    ctx.tr_err2.push_back(r.err2);
  }
  *done = true;
  return SM_OK;
}

template <typename T>
static int svd_split_run(Ctx& ctx, cudaStream_t st, const T* A, int m, int n,
                         const sm_strategy& strat, int left_mode, T* left, int right_mode, T* right,
                         double* s_out, SplitResult* out) {
  if (m <= 0 || n <= 0) {
    set_error("svd: empty matrix");
    return SM_ERR_VALUE;
  }
  const bool xu = left_mode == OUT_U && right_mode == OUT_SVT;
  const bool xv = left_mode == OUT_US && right_mode == OUT_VT;
  if ((xu || xv) && ctx.precision != SM_PRECISION_FP64 && !s_out) {
    int cap = 0, rf_k = 0;
    const int* cap_dev = nullptr;
    const bool hint = ctx.range_finder && ctx.rf_rank_hint > 0;
    const bool learned = ctx.precision == SM_PRECISION_MIXED_LEARNED &&
                         std::min(m, n) >= kMixedMinRank &&
                         strat.method == SM_RELATIVE_NORM_SQUARED_ERROR &&
                         strat.tolerance >= kMixedMinTol;
    if (learned && !ctx.range_finder && ctx.model.loaded) {
      // the cap stays on the device: features, network and cap without a host
      // round trip; the cluster kernel reads it (the host learns it with the
      // kernel's other results)
      int* d_cap;
      SM_CHECK(ctx.scratch("rank.cap", 2, &d_cap));
      SM_CHECK(rank_predict_dev(ctx, st, std::min(m, n), strat, kCapUseful, d_cap));
      cap_dev = d_cap;
    } else if (learned && (ctx.model.loaded || hint)) {
      int r = ctx.rf_rank_hint;
      if (!hint) SM_CHECK(rank_predict(ctx, st, std::min(m, n), strat, &r));
      cap = std::min(std::min(m, n), (int)std::ceil(ctx.cap_margin * r) + ctx.cap_extra);
      // a cap near the split size saves few QR steps and risks a redo of the
      // whole split: only caps below kCapUseful of min(m, n) are applied
      if (cap > kCapUseful * std::min(m, n)) cap = 0;
      // the range finder at the predicted rank + oversampling (used when that
      // is below min(m, n); otherwise the split keeps the QR path)
      if (ctx.range_finder) rf_k = std::min(std::min(m, n), r + ctx.rf_oversample);
      ctx.stats.rank_predicted_sum += r;
      ctx.stats.rank_predictions += 1;
    }
    bool done = false, missed = false;
    SM_CHECK(svd_split_mixed<T>(ctx, st, A, m, n, strat, xu, left, right, out, &done, cap,
                                &missed, rf_k, cap_dev));
    if (done) return SM_OK;
    if (missed)  // predicted rank too small: the full QR
      SM_CHECK(svd_split_mixed<T>(ctx, st, A, m, n, strat, xu, left, right, out, &done,
                                  std::min(m, n), &missed));
    if (done) return SM_OK;
  }
  if (xu) return svd_split_xfree<T>(ctx, st, A, m, n, strat, true, left, right, s_out, out);
  if (xv) return svd_split_xfree<T>(ctx, st, A, m, n, strat, false, left, right, s_out, out);
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
  int* wexp;
  SM_CHECK(ctx.scratch("svd.wexp", 1, &wexp));

  if (wide) {
    SM_CUDA_CHECK(cudaMemcpy2DAsync(Wx, sizeof(T) * ld, A, sizeof(T) * n, sizeof(T) * n, m,
                                    cudaMemcpyDeviceToDevice, st));
  } else {
    SM_CHECK(transpose<T>(st, m, n, A, n, Wx, ld));
  }
  SM_CHECK(prescale<T>(st, Wx, k, l, ld, wexp));
  {
    const size_t tot = (size_t)k * k;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((tot + 255) / 256, 4096));
    k_fill_rows<T><<<blocks, 256, 0, st>>>(k, l, Wx, ld);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
  }
  SM_CUDA_CHECK(cudaMemsetAsync(ctl, 0, sizeof(JacobiCtl), st));
  // The absolute floor leaves vectors with sigma^2 below ~16 l eps^2 |A|_F^2
  // unorthogonalised among themselves; enable it only when the truncation
  // rule certainly drops all of them (their summed weight is at most
  // 16 k l eps^2 |A|_F^2).
  const double eps = DBL_EPSILON;
  bool use_floor = false;
  if (strat.method == SM_RELATIVE_NORM_SQUARED_ERROR)
    use_floor = strat.tolerance >= 64.0 * k * (double)l * eps * eps;
  else if (strat.method == SM_RELATIVE_SINGULAR_VALUE)
    use_floor = strat.tolerance >= 16.0 * std::sqrt((double)k * l) * eps;
  if (k >= 2) {
    // squared row norms -> nrm; the Jacobi kernel sums them into |A|_F^2
    k_row_norms<T><<<(k + 7) / 8, 256, 0, st>>>(Wx, ld, k, l, nrm0, 1);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    const double tol = std::sqrt((double)l) * DBL_EPSILON;
    if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev0, st));
    double drel, dabs;
    deflation(strat, k, &drel, &dabs);
    int* act;
    SM_CHECK(ctx.scratch("svd.act", (size_t)k, &act));
    SM_CHECK(run_jacobi<T>(ctx, st, Wx, ld, k, l, l + k, tol * tol, use_floor ? 1 : 0, drel, dabs,
                           nrm, nrm0, act, ctl));
    if (ctx.timing) SM_CUDA_CHECK(cudaEventRecord(ctx.ev1, st));
    ctx.stats.jacobi_launches += 1;
    // 4 m n^2 + 8 n^3 with m >= n (x4 for complex arithmetic)
    ctx.stats.jacobi_flops += (4.0 * l * (double)k * k + 8.0 * (double)k * k * k) *
                              (sizeof(T) == sizeof(double) ? 1.0 : 4.0);
  }
  k_row_norms<T><<<(k + 7) / 8, 256, 0, st>>>(Wx, ld, k, l, nrm, 0, wexp);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  SM_CHECK(sort_truncate(st, nrm, k, strat, perm, s_sorted, errors, ctl, res));
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
  ctx.last_s = s_sorted;
  ctx.last_len = k;
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
                                                   s_sorted, left_mode, left, right_mode, right,
                                                   wexp);
                                                   note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
  }
  return SM_OK;
}

// Every split: features of the split (when recording or predicting), the
// split itself, then the record (features, kept rank) and the previous-split
// state the next split's features use.
template <typename T>
int svd_split(Ctx& ctx, cudaStream_t st, const T* A, int m, int n, const sm_strategy& strat,
              int left_mode, T* left, int right_mode, T* right, double* s_out,
              SplitResult* out) {
  const bool feat = ctx.record || ctx.precision == SM_PRECISION_MIXED_LEARNED;
  float f[SM_RANK_FEATURES];
  if (feat) rank_features(ctx, std::min(m, n), strat, f);
  ctx.last_s = nullptr;
  ctx.last_len = 0;
  SM_CHECK(svd_split_run<T>(ctx, st, A, m, n, strat, left_mode, left, right_mode, right, s_out,
                            out));
  if (feat) {
    if (ctx.record) {
      ctx.rec_x.insert(ctx.rec_x.end(), f, f + SM_RANK_FEATURES);
      ctx.rec_y.push_back(out->D);
    }
    ctx.prev_rank = out->D;
    const int c = std::min(32, ctx.last_len);
    // the next split's features: on the device for the device-side predictor
    // (no host round trip), on the host when recording or predicting there
    ctx.prev_len_dev = 0;
    if (c > 0 && ctx.last_s) {
      SM_CHECK(ctx.scratch("rank.prev_s", 32, &ctx.prev_s_dev));
      SM_CUDA_CHECK(cudaMemcpyAsync(ctx.prev_s_dev, ctx.last_s, sizeof(double) * c,
                                    cudaMemcpyDeviceToDevice, st));
      ctx.prev_len_dev = c;
    }
    ctx.prev_s.assign(c, 0.0);
    if (c > 0 && ctx.last_s && (ctx.record || ctx.range_finder || !ctx.model.loaded)) {
      SM_CUDA_CHECK(cudaMemcpyAsync(ctx.prev_s.data(), ctx.last_s, sizeof(double) * c,
                                    cudaMemcpyDeviceToHost, st));
      SM_CUDA_CHECK(cudaStreamSynchronize(st));
    }
  }
  return SM_OK;
}

template int svd_split<double>(Ctx&, cudaStream_t, const double*, int, int, const sm_strategy&,
                               int, double*, int, double*, double*, SplitResult*);
template int svd_split<cplx>(Ctx&, cudaStream_t, const cplx*, int, int, const sm_strategy&, int,
                             cplx*, int, cplx*, double*, SplitResult*);


// ---------------------------------------------------------------------------
// Allocation-free two-site split.
//
// Some callers cannot allocate device memory while they run: code embedded in
// a host application that owns all device memory through its own pool, code
// running where a cudaMalloc would synchronise the device or fail (inside a
// latency-critical loop, under a memory cap), or plugins that are only handed
// buffers.  For them sm_left_orth_2site_noalloc performs the same split as
// sm_left_orth_2site with every intermediate array carved out of the static
// device array below instead of the context's growable scratch.  The caller
// still passes the input and the two output buffers.
//
// Limits: both matrix dimensions a*d1 and d2*b at most kNoAllocMaxDim (256);
// the array then holds the [W | X] rows (at most 256 x 512 complex128
// elements, 2 MiB) plus the per-row vectors.  Every GPU that loads the library
// holds this array until the process exits.  All calls share it and it keeps
// the previous call's contents (everything that must start at zero is cleared
// by each call); calls whose work overlaps on the GPU (different streams,
// different host threads) race on it and must be serialised by the caller.
// ---------------------------------------------------------------------------
constexpr int kNoAllocMaxDim = 256;
constexpr size_t kNoAllocRowsBytes =
    (size_t)kNoAllocMaxDim * (2 * kNoAllocMaxDim) * sizeof(cplx);  // [W | X], 2 MiB
constexpr size_t kNoAllocVecBytes = 16 * 1024;                     // norms, order, control
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocRowsBytes + kNoAllocVecBytes];

// Host copies of the array's device address, one per device.  Several host
// threads may make their first call at once: each looks the address up and
// stores the same value, so a relaxed atomic is enough.  The address is kept
// for the life of the process; a cudaDeviceReset (which unloads this module
// from the device) is not supported between calls.
static std::atomic<unsigned char*> g_noalloc_ptr[64];

// One-time set-up per device (with that device current): the array's name is
// only a host-side stand-in, the kernels need its device address.
static int noalloc_scratch(unsigned char** out) {
  int dev = 0;
  SM_CUDA_CHECK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("noalloc: device ordinal out of range");
    return SM_ERR_VALUE;
  }
  unsigned char* p = g_noalloc_ptr[dev].load(std::memory_order_relaxed);
  if (!p) {
    void* q = nullptr;
    SM_CUDA_CHECK(cudaGetSymbolAddress(&q, g_noalloc_scratch));
    p = reinterpret_cast<unsigned char*>(q);
    g_noalloc_ptr[dev].store(p, std::memory_order_relaxed);
  }
  *out = p;
  return SM_OK;
}

// Cooperative Jacobi launch without any cache (the context-based launcher
// keeps occupancy results in a map; this one queries the runtime each time).
// `one_cta` runs the Jacobi as a single CTA (no inter-CTA barrier).
template <typename T, int E>
int launch_jacobi_noalloc(cudaStream_t st, T* Wx, int ld, int k, int l, double tol2, int use_floor,
                          double defl_rel, double defl_abs, double* nrm, const double* nrm0,
                          int* act, JacobiCtl* ctl, bool one_cta) {
  const int npairs = (k + (k & 1)) / 2;
  int dev = 0, sms = 1, per_sm = 1;
  SM_CUDA_CHECK(cudaGetDevice(&dev));
  SM_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  auto fn = k_jacobi<T, kJacobiNT, E>;
  SM_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kJacobiNT, 0));
  const int grid =
      one_cta ? 1 : std::max(1, std::min(npairs, std::max(1, per_sm) * std::max(1, sms)));
  int ms = kMaxSweeps;
  int L = l + k;
  void* args[] = {&Wx, &ld, &k, &l, &L, &tol2, &use_floor, &defl_rel, &defl_abs, &ms, &nrm,
                  &nrm0, &act, &ctl};
  SM_CHECK(coop_launch(reinterpret_cast<const void*>(fn), dim3(grid), dim3(kJacobiNT), args, st));
  note_launch();
  return SM_OK;
}

template <typename T>
int run_jacobi_noalloc(cudaStream_t st, T* Wx, int ld, int k, int l, double tol2, int use_floor,
                       double defl_rel, double defl_abs, double* nrm, const double* nrm0, int* act,
                       JacobiCtl* ctl, bool one_cta) {
  // k <= 256 and l <= 256 here, so a thread holds at most 4 elements per row
  const int need = (l + k + kJacobiNT - 1) / kJacobiNT;
  if (need <= 1)
    return launch_jacobi_noalloc<T, 1>(st, Wx, ld, k, l, tol2, use_floor, defl_rel, defl_abs, nrm,
                                       nrm0, act, ctl, one_cta);
  if (need <= 2)
    return launch_jacobi_noalloc<T, 2>(st, Wx, ld, k, l, tol2, use_floor, defl_rel, defl_abs, nrm,
                                       nrm0, act, ctl, one_cta);
  return launch_jacobi_noalloc<T, 4>(st, Wx, ld, k, l, tol2, use_floor, defl_rel, defl_abs, nrm,
                                     nrm0, act, ctl, one_cta);
}

// One attempt at the split, from the input onwards.  `one_cta` runs the
// Jacobi as a single CTA.
template <typename T>
int noalloc_attempt(cudaStream_t st, const T* A, int m, int n, const sm_strategy& strat, T* left,
                    T* right, int* D_out, double* err_out, bool one_cta) {
  unsigned char* base;
  SM_CHECK(noalloc_scratch(&base));
  const int k = std::min(m, n), l = std::max(m, n);
  const bool wide = m <= n;
  const int ld = l + k;
  T* Wx = reinterpret_cast<T*>(base);
  unsigned char* v = base + kNoAllocRowsBytes;
  double* nrm = reinterpret_cast<double*>(v);
  double* nrm0 = nrm + kNoAllocMaxDim;
  double* s_sorted = nrm0 + kNoAllocMaxDim;
  double* errors = s_sorted + kNoAllocMaxDim;  // k + 1 entries
  int* perm = reinterpret_cast<int*>(errors + kNoAllocMaxDim + 1);
  JacobiCtl* ctl = reinterpret_cast<JacobiCtl*>(
      reinterpret_cast<unsigned char*>(perm) + ((kNoAllocMaxDim * sizeof(int) + 255) & ~size_t(255)));
  SplitResult* res = reinterpret_cast<SplitResult*>(reinterpret_cast<unsigned char*>(ctl) + 256);
  int* act = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(res) + 256);
  int* wexp = act + kNoAllocMaxDim;

  if (wide) {
    SM_CUDA_CHECK(cudaMemcpy2DAsync(Wx, sizeof(T) * ld, A, sizeof(T) * n, sizeof(T) * n, m,
                                    cudaMemcpyDeviceToDevice, st));
  } else {
    SM_CHECK(transpose<T>(st, m, n, A, n, Wx, ld));
  }
  SM_CHECK(prescale<T>(st, Wx, k, l, ld, wexp));
  {
    const size_t tot = (size_t)k * k;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((tot + 255) / 256, 4096));
    k_fill_rows<T><<<blocks, 256, 0, st>>>(k, l, Wx, ld);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
  }
  SM_CUDA_CHECK(cudaMemsetAsync(ctl, 0, sizeof(JacobiCtl), st));
  const double eps = DBL_EPSILON;
  bool use_floor = false;
  if (strat.method == SM_RELATIVE_NORM_SQUARED_ERROR)
    use_floor = strat.tolerance >= 64.0 * k * (double)l * eps * eps;
  else if (strat.method == SM_RELATIVE_SINGULAR_VALUE)
    use_floor = strat.tolerance >= 16.0 * std::sqrt((double)k * l) * eps;
  if (k >= 2) {
    k_row_norms<T><<<(k + 7) / 8, 256, 0, st>>>(Wx, ld, k, l, nrm0, 1);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
    const double tol = std::sqrt((double)l) * DBL_EPSILON;
    double drel, dabs;
    deflation(strat, k, &drel, &dabs);
    SM_CHECK(run_jacobi_noalloc<T>(st, Wx, ld, k, l, tol * tol, use_floor ? 1 : 0, drel, dabs, nrm,
                                   nrm0, act, ctl, one_cta));
  }
  k_row_norms<T><<<(k + 7) / 8, 256, 0, st>>>(Wx, ld, k, l, nrm, 0, wexp);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  SM_CHECK(sort_truncate(st, nrm, k, strat, perm, s_sorted, errors, ctl, res));
  SplitResult h;
  SM_CUDA_CHECK(cudaMemcpyAsync(&h, res, sizeof(SplitResult), cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  if (h.status & DEV_BARRIER_TIMEOUT) {
    set_error("svd: grid barrier timed out");
    return SM_ERR_TIMEOUT;
  }
  if (h.status & (DEV_NONFINITE | DEV_NOT_CONVERGED)) {
    set_error("SVD did not converge");
    return SM_ERR_LINALG;
  }
  const int D = h.D;
  const size_t total = (size_t)m * D + (size_t)D * n;
  const int blocks = (int)std::min<size_t>((total + 255) / 256, 4096);
  k_emit<T><<<std::max(blocks, 1), 256, 0, st>>>(wide, m, n, D, Wx, ld, Wx + l, ld, perm, s_sorted,
                                                 OUT_U, left, OUT_SVT, right, wexp);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  *D_out = D;
  *err_out = std::sqrt(h.err2);
  return SM_OK;
}

template <typename T>
int left_orth_2site_noalloc(cudaStream_t st, const T* A, long long m, long long n,
                            const sm_strategy& strat, T* left, T* right, int* D_out,
                            double* err_out) {
  if (m <= 0 || n <= 0) {
    set_error("noalloc split: empty matrix");
    return SM_ERR_VALUE;
  }
  if (m > kNoAllocMaxDim || n > kNoAllocMaxDim) {
    set_error("noalloc split: matrix " + std::to_string(m) + " x " + std::to_string(n) +
              " exceeds the static scratch limit of " + std::to_string(kNoAllocMaxDim) +
              " per dimension");
    return SM_ERR_VALUE;
  }
  // The multi-CTA Jacobi needs all its CTAs resident at once; when kernels of
  // other streams hold the SMs its bounded grid barrier gives up with a
  // timeout.  The split is then redone from the input with a one-CTA Jacobi.
  int rc = noalloc_attempt<T>(st, A, (int)m, (int)n, strat, left, right, D_out, err_out, false);
  if (rc == SM_ERR_TIMEOUT)
    rc = noalloc_attempt<T>(st, A, (int)m, (int)n, strat, left, right, D_out, err_out, true);
  return rc;
}

}  // namespace sm

extern "C" int sm_left_orth_2site_noalloc(int dtype, const void* AA, int a, int d1, int d2, int b,
                                          const sm_strategy* st, void* U, void* SV, int* D,
                                          double* err, void* stream) {
  using namespace sm;
  if (!st || !AA || !U || !SV || !D || !err) {
    set_error("sm_left_orth_2site_noalloc: null argument");
    return SM_ERR_VALUE;
  }
  if (st->tolerance < 0 || st->tolerance >= 1.0 || st->max_bond_dimension <= 0 || st->method < 0 ||
      st->method > 3) {
    set_error("Invalid Strategy passed to sm_left_orth_2site_noalloc");
    return SM_ERR_STRATEGY;
  }
  if (a <= 0 || d1 <= 0 || d2 <= 0 || b <= 0) {
    set_error("sm_left_orth_2site_noalloc: non-positive dimension");
    return SM_ERR_VALUE;
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  // the products in 64 bits, so that no overflow gets past the size limit
  const long long m = (long long)a * d1, n = (long long)d2 * b;
  if (dtype == SM_FLOAT64)
    return left_orth_2site_noalloc<double>(s, (const double*)AA, m, n, *st, (double*)U,
                                           (double*)SV, D, err);
  if (dtype == SM_COMPLEX128)
    return left_orth_2site_noalloc<cplx>(s, (const cplx*)AA, m, n, *st, (cplx*)U, (cplx*)SV, D,
                                         err);
  set_error("dtype must be SM_FLOAT64 or SM_COMPLEX128");
  return SM_ERR_VALUE;
}
