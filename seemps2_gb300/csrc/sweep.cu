// Device-resident simplification driver (host C++ issuing sm_103a kernels).
//
// Mirrors, step for step, the reference's Python sweep so that the truncation
// decisions are taken on the same matrices in the same order:
//   simplify / simplify_mps_sum      state/simplification.py:32-280
//   AntilinearForm                   state/antilinear.py:13-146
//   CanonicalMPS / _canonicalize     state/canonical_mps.py:76-108, cython/schmidt.pxi:18-120
//   _left_orth_2site/_right_orth_2site cython/schmidt.pxi:123-174
//   MPSSum.join / delete_zero_components state/mpssum.py:130-228
// All tensors stay in device memory; only kept ranks and the sweep's scalar
// error estimate come back to the host (they decide shapes and the stop rule).
// Two refinements over the reference that do not change any result: the
// environment update after a split reuses the L*A (or B*R) product already
// formed for the two-site tensor (the reference recomputes the same product),
// and the site buffers are allocated once per context and reused.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "kernels.cuh"

namespace sm {

namespace {

template <typename T>
T from_pair(const double* w);
template <>
double from_pair<double>(const double* w) { return w[0]; }
template <>
cplx from_pair<cplx>(const double* w) { return {w[0], w[1]}; }

inline double abs_pair(const double* w) { return std::sqrt(w[0] * w[0] + w[1] * w[1]); }

template <typename T>
struct Sweeper {
  Ctx& ctx;
  cudaStream_t st;
  sm_strategy s;
  int L;
  std::vector<int> d;
  // kets: one per term of the sum
  int nt = 0;
  std::vector<std::vector<const T*>> ket;
  std::vector<std::vector<int>> kb;
  std::vector<T> w;
  std::vector<double> wabs, term_err;
  // bra (the approximation being optimised)
  std::vector<int> bb, cap;
  std::vector<T*> bra;
  // environments per term
  std::vector<std::vector<T*>> Lenv, Renv;
  std::vector<T*> LA, BR;
  T *AA = nullptr, *tmp = nullptr, *tmp2 = nullptr;
  double* dsc = nullptr;  // device scalars
  int splits = 0;

  // each call starts the split features afresh (no previous split)
  Sweeper(Ctx& c, cudaStream_t stream, const sm_strategy& strat) : ctx(c), st(stream), s(strat) {
    ctx.prev_s.clear();
    ctx.prev_len_dev = 0;
    ctx.prev_rank = 0;
    ctx.split_site = -1;
    ctx.split_n = 0;
  }

  size_t site_elems(int i) const { return (size_t)bb[i] * d[i] * bb[i + 1]; }

  // Sweep contractions in FP32 arithmetic: the mixed forms' setting, taken
  // only when every two-site split of the sweep fits the FP32 cluster kernel.
  // A split beyond it runs the FP64 Jacobi, which cannot deflate the FP32
  // rounding noise of its input (singular values at 1e-7 of the largest
  // instead of 1e-16): at n=40, chi=512 that made the FP64 splits 2.7x slower.
  bool c32 = false;
  void choose_contractions() {
    c32 = ctx.precision != SM_PRECISION_FP64 && ctx.contract32;
    for (int i = 0; c32 && i + 1 < L; ++i) {
      const int M = cap[i] * d[i], N = d[i + 1] * cap[i + 2];
      if (std::min(M, N) < kMixedMinRank) continue;  // FP64 path either way
      c32 = split_cluster_size_ok<T>(N, M) && split_cluster_size_ok<T>(M, N);
    }
  }

  int buf(const std::string& name, size_t n, T** p) { return ctx.scratch(name, std::max<size_t>(n, 1), p); }

  // ---- helpers -------------------------------------------------------------
  int gemm_(int opA, int opB, int M, int N, int K, T alpha, const T* A, int lda, const T* B,
            int ldb, T beta, T* C, int ldc) {
    if (c32) return gemm_ctx_f32<T>(ctx, st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
    return gemm_ctx<T>(ctx, st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  }
  // FP64 contractions whatever the context's setting (norms and overlaps)
  int gemm64_(int opA, int opB, int M, int N, int K, T alpha, const T* A, int lda, const T* B,
              int ldb, T beta, T* C, int ldc) {
    return gemm_ctx<T>(ctx, st, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  }
  static T one() { return S<T>::one(); }
  static T zero() { return S<T>::zero(); }

  // sqrt(err^2) of a right canonical update at site i (schmidt.pxi:18-42)
  int canon_right(int i, double* err) {
    const int a = bb[i], di = d[i], b = bb[i + 1];
    SplitResult r;
    ctx.split_site = i;
    ctx.split_n = L;
    SM_CHECK(svd_split<T>(ctx, st, bra[i], a * di, b, s, OUT_U, bra[i], OUT_SVT, tmp, nullptr, &r));
    ++splits;
    const int D = r.D;
    // bra[i+1] <- (s V) @ bra[i+1]
    const int dn = d[i + 1], bn = bb[i + 2];
    SM_CHECK(gemm_(SM_OP_N, SM_OP_N, D, dn * bn, b, one(), tmp, b, bra[i + 1], dn * bn, zero(),
                   tmp2, dn * bn));
    SM_CUDA_CHECK(cudaMemcpyAsync(bra[i + 1], tmp2, sizeof(T) * (size_t)D * dn * bn,
                                  cudaMemcpyDeviceToDevice, st));
    bb[i + 1] = D;
    *err = std::sqrt(r.err2);
    return SM_OK;
  }

  // sqrt(err^2) of a left canonical update at site i (schmidt.pxi:59-82)
  int canon_left(int i, double* err) {
    const int a = bb[i], di = d[i], b = bb[i + 1];
    SplitResult r;
    ctx.split_site = i;
    ctx.split_n = L;
    SM_CHECK(svd_split<T>(ctx, st, bra[i], a, di * b, s, OUT_US, tmp, OUT_VT, bra[i], nullptr, &r));
    ++splits;
    const int D = r.D;
    // bra[i-1] <- bra[i-1] @ (U s)
    const int ap = bb[i - 1], dp = d[i - 1];
    SM_CHECK(gemm_(SM_OP_N, SM_OP_N, ap * dp, D, a, one(), bra[i - 1], a, tmp, D, zero(), tmp2, D));
    SM_CUDA_CHECK(cudaMemcpyAsync(bra[i - 1], tmp2, sizeof(T) * (size_t)ap * dp * D,
                                  cudaMemcpyDeviceToDevice, st));
    bb[i] = D;
    *err = std::sqrt(r.err2);
    return SM_OK;
  }

  int canonicalize(int center, double* err) {
    double e = 0.0, x;
    for (int i = 0; i < center; ++i) {
      SM_CHECK(canon_right(i, &x));
      e += x;
    }
    for (int i = L - 1; i > center; --i) {
      SM_CHECK(canon_left(i, &x));
      e += x;
    }
    *err = e;
    return SM_OK;
  }

  int recanonicalize(int oldc, int newc, double* err) {
    double e = 0.0, x;
    while (oldc > newc) {
      SM_CHECK(canon_left(oldc, &x));
      e += x;
      --oldc;
    }
    while (oldc < newc) {
      SM_CHECK(canon_right(oldc, &x));
      e += x;
      ++oldc;
    }
    *err = e;
    return SM_OK;
  }

  int normalize_site(int c) {
    double* h = reinterpret_cast<double*>(ctx.pinned) + 64;
    SM_CHECK(vdot<T>(ctx, st, site_elems(c), bra[c], bra[c], dsc));
    SM_CUDA_CHECK(cudaMemcpyAsync(h, dsc, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    SM_CUDA_CHECK(cudaStreamSynchronize(st));
    const double nrm = std::sqrt(h[0]);
    if (nrm) SM_CHECK(scale_vector<T>(st, site_elems(c), 1.0 / nrm, bra[c]));
    return SM_OK;
  }

  // <bra|ket> of two arbitrary MPS through left environments (environments.pxi:87-118)
  int scprod(const std::vector<const T*>& A, const std::vector<int>& ab,
             const std::vector<const T*>& B, const std::vector<int>& bbnd, double* out) {
    T *rho, *rho2, *t;
    size_t mx = 1, mt = 1;
    for (int i = 0; i <= L; ++i) mx = std::max(mx, (size_t)ab[i] * bbnd[i]);
    for (int i = 0; i < L; ++i) mt = std::max(mt, (size_t)ab[i] * d[i] * bbnd[i + 1]);
    SM_CHECK(buf("sc.rho", mx, &rho));
    SM_CHECK(buf("sc.rho2", mx, &rho2));
    SM_CHECK(buf("sc.t", mt, &t));
    SM_CHECK(set_identity<T>(st, 1, rho, 1));
    for (int i = 0; i < L; ++i) {
      // t = rho (ab[i] x bb[i]) @ B[i] (bb[i] x d*bb[i+1])
      SM_CHECK(gemm64_(SM_OP_N, SM_OP_N, ab[i], d[i] * bbnd[i + 1], bbnd[i], one(), rho, bbnd[i], B[i],
                     d[i] * bbnd[i + 1], zero(), t, d[i] * bbnd[i + 1]));
      // rho' = A[i]^H (ab[i+1] x ab[i]*d) @ t (ab[i]*d x bb[i+1])
      SM_CHECK(gemm64_(SM_OP_C, SM_OP_N, ab[i + 1], bbnd[i + 1], ab[i] * d[i], one(), A[i], ab[i + 1], t,
                     bbnd[i + 1], zero(), rho2, bbnd[i + 1]));
      std::swap(rho, rho2);
    }
    double* h = reinterpret_cast<double*>(ctx.pinned) + 64;
    SM_CUDA_CHECK(cudaMemcpyAsync(h, rho, sizeof(T), cudaMemcpyDeviceToHost, st));
    SM_CUDA_CHECK(cudaStreamSynchronize(st));
    out[0] = h[0];
    out[1] = sizeof(T) == sizeof(double) ? 0.0 : h[1];
    return SM_OK;
  }

  // left environment update: out = B^H (rho A) with B = bra[i], A = ket_t[i]
  int env_left_from(int t, int i, T* LAt) {
    // LAt already holds rho @ A as (bb[i]*d x kb[i+1])
    return gemm_(SM_OP_C, SM_OP_N, bb[i + 1], kb[t][i + 1], bb[i] * d[i], one(), bra[i], bb[i + 1],
                 LAt, kb[t][i + 1], zero(), Lenv[t][i + 1], kb[t][i + 1]);
  }
  // right environment update R[i-1] = (A R[i]) B^H with B = bra[i], A = ket_t[i]
  int env_right_from(int t, int i, T* BRt) {
    // BRt already holds A @ rho as (kb[i] x d*bb[i+1]); out = BRt @ bra[i]^H
    return gemm_(SM_OP_N, SM_OP_C, kb[t][i], bb[i], d[i] * bb[i + 1], one(), BRt, d[i] * bb[i + 1],
                 bra[i], d[i] * bb[i + 1], zero(), Renv[t][i - 1], bb[i]);
  }
  int form_LA(int t, int i, T* out) {  // L_t[i] @ ket_t[i]
    return gemm_(SM_OP_N, SM_OP_N, bb[i], d[i] * kb[t][i + 1], kb[t][i], one(), Lenv[t][i], kb[t][i],
                 ket[t][i], d[i] * kb[t][i + 1], zero(), out, d[i] * kb[t][i + 1]);
  }
  int form_BR(int t, int j, T* out) {  // ket_t[j] @ R_t[j]
    return gemm_(SM_OP_N, SM_OP_N, kb[t][j] * d[j], bb[j + 1], kb[t][j + 1], one(), ket[t][j],
                 kb[t][j + 1], Renv[t][j], bb[j + 1], zero(), out, bb[j + 1]);
  }

  int init_environments(int center) {
    for (int t = 0; t < nt; ++t) {
      SM_CHECK(set_identity<T>(st, 1, Renv[t][L - 1], 1));
      for (int i = L - 1; i > center; --i) {
        SM_CHECK(form_BR(t, i, BR[t]));
        SM_CHECK(env_right_from(t, i, BR[t]));  // R[i-1]
      }
      SM_CHECK(set_identity<T>(st, 1, Lenv[t][0], 1));
      for (int i = 0; i < center; ++i) {
        SM_CHECK(form_LA(t, i, LA[t]));
        SM_CHECK(env_left_from(t, i, LA[t]));
      }
    }
    return SM_OK;
  }

  // AA = sum_t w_t (L_t[i] A_t[i]) (A_t[j] R_t[j]),  j = i+1
  int two_site(int i) {
    const int j = i + 1;
    const int M = bb[i] * d[i], N = d[j] * bb[j + 1];
    for (int t = 0; t < nt; ++t) {
      SM_CHECK(form_LA(t, i, LA[t]));
      SM_CHECK(form_BR(t, j, BR[t]));
      SM_CHECK(gemm_(SM_OP_N, SM_OP_N, M, N, kb[t][j], w[t], LA[t], kb[t][j], BR[t],
                     N, t == 0 ? zero() : one(), AA, N));
    }
    return SM_OK;
  }

  int step_right(int n) {
    SM_CHECK(two_site(n));
    SplitResult r;
    ctx.split_site = n;
    ctx.split_n = L;
    SM_CHECK(svd_split<T>(ctx, st, AA, bb[n] * d[n], d[n + 1] * bb[n + 2], s, OUT_U, bra[n], OUT_SVT,
                          bra[n + 1], nullptr, &r));
    ++splits;
    bb[n + 1] = r.D;
    for (int t = 0; t < nt; ++t) SM_CHECK(env_left_from(t, n, LA[t]));
    return SM_OK;
  }

  int step_left(int n) {
    SM_CHECK(two_site(n));
    SplitResult r;
    ctx.split_site = n;
    ctx.split_n = L;
    SM_CHECK(svd_split<T>(ctx, st, AA, bb[n] * d[n], d[n + 1] * bb[n + 2], s, OUT_US, bra[n], OUT_VT,
                          bra[n + 1], nullptr, &r));
    ++splits;
    bb[n + 1] = r.D;
    for (int t = 0; t < nt; ++t) SM_CHECK(env_right_from(t, n + 1, BR[t]));
    return SM_OK;
  }

  // vdot(bra[c], bra[c]) and vdot(bra[c], sum_t w_t L_t[c] ket_t[c] R_t[c])
  int estimate(int c, double* nm, double* sc) {
    const size_t n = site_elems(c);
    for (int t = 0; t < nt; ++t) {
      SM_CHECK(form_BR(t, c, BR[t]));  // ket[c] @ R[c] : (kb[c] x d*bb[c+1])
      SM_CHECK(gemm_(SM_OP_N, SM_OP_N, bb[c], d[c] * bb[c + 1], kb[t][c], w[t],
                     Lenv[t][c], kb[t][c], BR[t], d[c] * bb[c + 1], t == 0 ? zero() : one(), tmp,
                     d[c] * bb[c + 1]));
    }
    SM_CHECK(vdot<T>(ctx, st, n, bra[c], bra[c], dsc));
    SM_CHECK(vdot<T>(ctx, st, n, bra[c], tmp, dsc + 2));
    double* h = reinterpret_cast<double*>(ctx.pinned) + 64;
    SM_CUDA_CHECK(cudaMemcpyAsync(h, dsc, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
    SM_CUDA_CHECK(cudaStreamSynchronize(st));
    *nm = h[0];
    *sc = h[2];
    return SM_OK;
  }
};

}  // namespace

template <typename T>
int simplify_impl(Ctx& ctx, cudaStream_t st, int L, const int* phys, int nterms,
                  const double* weights, const double* term_errors, const int* ket_bonds,
                  const void* const* ket_sites, const sm_strategy& s, int direction,
                  void* const* out_sites, const int64_t* out_cap, int* out_bonds,
                  sm_simplify_report* rep, const double* gram, const int* guess_bonds,
                  const void* const* guess_sites) {
  Sweeper<T> S_(ctx, st, s);
  auto& w = S_;
  w.L = L;
  w.d.assign(phys, phys + L);
  // ---- terms (delete_zero_components for sums, state/mpssum.py:204-228) ----
  std::vector<int> keep;
  double norm_state_sqr = 0.0;
  {
    std::vector<std::vector<const T*>> kets(nterms);
    std::vector<std::vector<int>> kbs(nterms);
    for (int t = 0; t < nterms; ++t) {
      kets[t].assign(reinterpret_cast<const T* const*>(ket_sites) + (size_t)t * L,
                     reinterpret_cast<const T* const*>(ket_sites) + (size_t)(t + 1) * L);
      kbs[t].assign(ket_bonds + (size_t)t * (L + 1), ket_bonds + (size_t)(t + 1) * (L + 1));
    }
    // a plain MPS is the one-term sum with weight 1: |w|^2 |<s|s>| is then
    // exactly the reference's abs(scprod(state, state).real).  A caller that
    // knows the terms' products (the MPO apply, from the factors) passes them
    // as `gram` (<s_i|s_j>, row-major complex pairs) instead.
    auto product = [&](int i, int j, double* v) -> int {
      if (gram) {
        v[0] = gram[2 * ((size_t)i * nterms + j)];
        v[1] = gram[2 * ((size_t)i * nterms + j) + 1];
        return SM_OK;
      }
      return w.scprod(kets[i], kbs[i], kets[j], kbs[j], v);
    };
    double c = 0.0;
    for (int i = 0; i < nterms; ++i) {
      const double* wi = weights + 2 * i;
      double sc[2];
      SM_CHECK(product(i, i, sc));
      const double ni = (wi[0] * wi[0] + wi[1] * wi[1]) * std::fabs(sc[0]);
      if (ni) {
        for (int j : keep) {
          const double* wj = weights + 2 * j;
          double p[2];
          SM_CHECK(product(i, j, p));
          // (conj(wi) wj <s_i|s_j>).real
          const double ar = wi[0] * wj[0] + wi[1] * wj[1];
          const double ai = wi[0] * wj[1] - wi[1] * wj[0];
          c += 2.0 * (ar * p[0] - ai * p[1]);
        }
        keep.push_back(i);
        c += ni;
      }
    }
    norm_state_sqr = std::fabs(c);
    for (int t : keep) {
      w.ket.push_back(kets[t]);
      w.kb.push_back(kbs[t]);
      w.w.push_back(from_pair<T>(weights + 2 * t));
      w.wabs.push_back(abs_pair(weights + 2 * t));
      w.term_err.push_back(term_errors ? term_errors[t] : 0.0);
    }
    w.nt = (int)keep.size();
  }
  rep->norm_state_sqr = norm_state_sqr;
  rep->zero_state = 0;
  rep->sweeps = 0;
  rep->splits = 0;
  rep->last_err = 0.0;
  auto emit_zero = [&]() -> int {
    for (int i = 0; i <= L; ++i) out_bonds[i] = 1;
    for (int i = 0; i < L; ++i) {
      if (out_cap[i] < phys[i]) {
        set_error("simplify: output capacity too small");
        return SM_ERR_VALUE;
      }
      SM_CHECK(fill_zero<T>(st, (size_t)phys[i], reinterpret_cast<T*>(out_sites[i])));
    }
    rep->zero_state = 1;
    rep->center = 0;
    rep->error = 0.0;
    return SM_OK;
  };
  const bool variational = s.simplify != SM_CANONICAL_FORM && s.simplify != SM_DO_NOT_SIMPLIFY;
  if (w.nt == 0) return emit_zero();  // every term of the sum is zero

  // ---- the guess: the joined kets (state/mpssum.py:130-167), or the caller's
  // guess (simplification.py:93-98: CanonicalMPS(guess, center=start)) -------
  std::vector<int> K(L + 1, 0);
  K[0] = K[L] = 1;
  for (int i = 1; i < L; ++i) {
    int acc = 0;
    for (int t = 0; t < w.nt; ++t) acc += w.kb[t][i];
    K[i] = acc;
  }
  const bool has_guess = guess_bonds != nullptr && guess_sites != nullptr && variational;
  // buffer sizes: the guess's bonds may exceed the joined kets' bonds
  std::vector<int> KX = K;
  if (has_guess) {
    if (guess_bonds[0] != 1 || guess_bonds[L] != 1) {
      set_error("simplify: the guess's open boundary bonds must be 1");
      return SM_ERR_VALUE;
    }
    for (int i = 0; i <= L; ++i) {
      if (guess_bonds[i] <= 0) {
        set_error("simplify: non-positive bond in the guess");
        return SM_ERR_VALUE;
      }
      KX[i] = std::max(K[i], guess_bonds[i]);
    }
  }
  const bool unit_single = w.nt == 1 && S<T>::abs2(w.w[0] - S<T>::one()) == 0.0;
  w.bb = has_guess ? std::vector<int>(guess_bonds, guess_bonds + L + 1) : K;
  w.bra.resize(L);
  for (int i = 0; i < L; ++i) {
    SM_CHECK(w.buf("sw.bra." + std::to_string(i), (size_t)KX[i] * w.d[i] * KX[i + 1], &w.bra[i]));
    if (has_guess) {
      SM_CUDA_CHECK(cudaMemcpyAsync(w.bra[i], guess_sites[i],
                                    sizeof(T) * (size_t)guess_bonds[i] * w.d[i] * guess_bonds[i + 1],
                                    cudaMemcpyDeviceToDevice, st));
    } else if (unit_single) {
      SM_CUDA_CHECK(cudaMemcpyAsync(w.bra[i], w.ket[0][i], sizeof(T) * (size_t)K[i] * w.d[i] * K[i + 1],
                                    cudaMemcpyDeviceToDevice, st));
    } else {
      SM_CHECK(fill_zero<T>(st, (size_t)K[i] * w.d[i] * K[i + 1], w.bra[i]));
      int oa = 0, ob = 0;
      for (int t = 0; t < w.nt; ++t) {
        const int a = w.kb[t][i], b = w.kb[t][i + 1];
        const T wt = i == 0 ? w.w[t] : S<T>::one();
        if (i == 0) {
          SM_CHECK(copy_block3<T>(st, w.ket[t][i], a, w.d[i], b, w.bra[i], K[i], K[i + 1], 0, ob, wt));
        } else if (i == L - 1) {
          SM_CHECK(copy_block3<T>(st, w.ket[t][i], a, w.d[i], b, w.bra[i], K[i], K[i + 1], oa, 0, wt));
        } else {
          SM_CHECK(copy_block3<T>(st, w.ket[t][i], a, w.d[i], b, w.bra[i], K[i], K[i + 1], oa, ob, wt));
        }
        oa += a;
        ob += b;
      }
    }
  }
  // bond caps for the sweep buffers: every split keeps at most min(max bond, K)
  // (and the guess's own bonds, which the canonical form can only reduce)
  w.cap.assign(L + 1, 1);
  for (int i = 0; i <= L; ++i)
    w.cap[i] = std::max({1, std::min(K[i], s.max_bond_dimension), has_guess ? guess_bonds[i] : 1});
  w.cap[0] = K[0];
  w.cap[L] = K[L];
  // scratch for the sweep
  size_t mx_tmp = 1, mx_AA = 1;
  for (int i = 0; i < L; ++i) {
    mx_tmp = std::max(mx_tmp, (size_t)KX[i] * w.d[i] * KX[i + 1]);
    mx_tmp = std::max(mx_tmp, (size_t)KX[i] * KX[i]);
    mx_tmp = std::max(mx_tmp, (size_t)KX[i + 1] * KX[i + 1]);
    if (i + 1 < L)
      mx_AA = std::max(mx_AA, (size_t)w.cap[i] * w.d[i] * w.d[i + 1] * w.cap[i + 2]);
  }
  SM_CHECK(w.buf("sw.tmp", mx_tmp, &w.tmp));
  SM_CHECK(w.buf("sw.tmp2", mx_tmp, &w.tmp2));
  SM_CHECK(w.buf("sw.AA", mx_AA, &w.AA));
  SM_CHECK(ctx.scratch("sw.dsc", 8, &w.dsc));

  const int start = direction > 0 ? 0 : L - 1;
  double canon_err = 0.0;
  if (!variational) {
    // CANONICAL_FORM: two passes; DO_NOT_SIMPLIFY: one (simplification.py:66-91)
    const int c0 = s.simplify == SM_CANONICAL_FORM ? start : L - 1 - start;
    SM_CHECK(w.canonicalize(c0, &canon_err));
    if (s.normalize) SM_CHECK(w.normalize_site(c0));
    int c = c0;
    if (s.simplify == SM_CANONICAL_FORM) {
      double e2;
      const int c1 = L - 1 - start;
      SM_CHECK(w.recanonicalize(c0, c1, &e2));
      canon_err += e2;
      c = c1;
    }
    rep->center = c;
    rep->error = canon_err;  // the input's own error is not carried (MPS.__init__ error=0)
  } else {
    SM_CHECK(w.canonicalize(start, &canon_err));  // CanonicalMPS(..., normalize=False)
    if (!norm_state_sqr) return emit_zero();
    // environments (antilinear.py:38-57), one form per term
    w.Lenv.assign(w.nt, std::vector<T*>(L, nullptr));
    w.Renv.assign(w.nt, std::vector<T*>(L, nullptr));
    w.LA.resize(w.nt);
    w.BR.resize(w.nt);
    for (int t = 0; t < w.nt; ++t) {
      size_t mla = 1, mbr = 1;
      for (int i = 0; i < L; ++i) {
        const std::string k = std::to_string(t) + "." + std::to_string(i);
        SM_CHECK(w.buf("sw.L." + k, (size_t)w.cap[i] * w.kb[t][i], &w.Lenv[t][i]));
        SM_CHECK(w.buf("sw.R." + k, (size_t)w.kb[t][i + 1] * w.cap[i + 1], &w.Renv[t][i]));
        mla = std::max(mla, (size_t)w.cap[i] * w.d[i] * w.kb[t][i + 1]);
        mbr = std::max(mbr, (size_t)w.kb[t][i] * w.d[i] * w.cap[i + 1]);
      }
      SM_CHECK(w.buf("sw.LA." + std::to_string(t), mla, &w.LA[t]));
      SM_CHECK(w.buf("sw.BR." + std::to_string(t), mbr, &w.BR[t]));
    }
    w.choose_contractions();
    SM_CHECK(w.init_environments(start));
    double err = 2.0, nm = 0.0;
    int c = start;
    int dir = direction;
    const int nsweeps = std::max(1, s.max_sweeps);
    for (int sweep = 0; sweep < nsweeps; ++sweep) {
      if (dir > 0) {
        for (int n = 0; n < L - 1; ++n) SM_CHECK(w.step_right(n));
        c = L - 1;
      } else {
        for (int n = L - 2; n >= 0; --n) SM_CHECK(w.step_left(n));
        c = 0;
      }
      double sc;
      SM_CHECK(w.estimate(c, &nm, &sc));
      const double old_err = err;
      err = 2.0 * std::fabs(1.0 - sc / std::sqrt(nm * norm_state_sqr));
      if (sweep < 64) rep->sweep_err[sweep] = err;
      rep->sweeps = sweep + 1;
      if (err < s.simplification_tolerance || err > old_err) break;
      dir = -dir;
    }
    if (w.c32) {
      // the error bound's last term needs the overlap to FP64 accuracy: rebuild
      // the environments of the final centre with FP64 contractions
      w.c32 = false;
      const int rc = w.init_environments(c);
      double sc = 0.0;
      const int rc2 = rc == SM_OK ? w.estimate(c, &nm, &sc) : rc;
      SM_CHECK(rc2);
      err = 2.0 * std::fabs(1.0 - sc / std::sqrt(nm * norm_state_sqr));
      if (rep->sweeps >= 1 && rep->sweeps <= 64) rep->sweep_err[rep->sweeps - 1] = err;
    }
    // a tensor-core pipeline wait that timed out (none expected) fails the call
    if (ctx.precision != SM_PRECISION_FP64) SM_CHECK(tc_status_check(ctx, st));
    double state_error = 0.0;
    for (int t = 0; t < w.nt; ++t) state_error += w.wabs[t] * w.term_err[t];
    double bound = state_error + std::sqrt(err);
    if (s.normalize && nm) {
      const double f = std::sqrt(nm);
      SM_CHECK(scale_vector<T>(st, w.site_elems(c), 1.0 / f, w.bra[c]));
      bound /= f;
    }
    rep->error = bound;
    rep->center = c;
    rep->norm_mps_sqr = nm;
    rep->last_err = err;
  }
  // ---- copy out ----
  for (int i = 0; i <= L; ++i) out_bonds[i] = w.bb[i];
  for (int i = 0; i < L; ++i) {
    const size_t n = w.site_elems(i);
    if ((size_t)out_cap[i] < n) {
      set_error("simplify: output capacity too small at site " + std::to_string(i));
      return SM_ERR_VALUE;
    }
    SM_CUDA_CHECK(cudaMemcpyAsync(out_sites[i], w.bra[i], sizeof(T) * n, cudaMemcpyDeviceToDevice, st));
  }
  rep->splits = w.splits;
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  return SM_OK;
}

// In-place canonicalisation of caller buffers (cython/schmidt.pxi:109-120).
template <typename T>
int canonicalize_impl(Ctx& ctx, cudaStream_t st, int L, const int* phys, int* bonds,
                      void* const* sites, const int64_t* cap, int center, const sm_strategy& s,
                      double* err) {
  Sweeper<T> w(ctx, st, s);
  w.L = L;
  w.d.assign(phys, phys + L);
  w.bb.assign(bonds, bonds + L + 1);
  w.bra.resize(L);
  size_t mx = 1;
  for (int i = 0; i < L; ++i) {
    w.bra[i] = reinterpret_cast<T*>(sites[i]);
    if ((size_t)cap[i] < w.site_elems(i)) {
      set_error("canonicalize: site buffer smaller than its tensor");
      return SM_ERR_VALUE;
    }
    mx = std::max(mx, w.site_elems(i));
  }
  SM_CHECK(w.buf("cn.tmp", mx, &w.tmp));
  SM_CHECK(w.buf("cn.tmp2", mx, &w.tmp2));
  SM_CHECK(w.canonicalize(center, err));
  for (int i = 0; i <= L; ++i) bonds[i] = w.bb[i];
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  return SM_OK;
}

// In-place move of the orthogonality centre (cython/schmidt.pxi:96-106).
template <typename T>
int recanonicalize_impl(Ctx& ctx, cudaStream_t st, int L, const int* phys, int* bonds,
                        void* const* sites, const int64_t* cap, int oldc, int newc,
                        const sm_strategy& s, double* err) {
  Sweeper<T> w(ctx, st, s);
  w.L = L;
  w.d.assign(phys, phys + L);
  w.bb.assign(bonds, bonds + L + 1);
  w.bra.resize(L);
  size_t mx = 1;
  for (int i = 0; i < L; ++i) {
    w.bra[i] = reinterpret_cast<T*>(sites[i]);
    if ((size_t)cap[i] < w.site_elems(i)) {
      set_error("recanonicalize: site buffer smaller than its tensor");
      return SM_ERR_VALUE;
    }
    mx = std::max(mx, w.site_elems(i));
  }
  SM_CHECK(w.buf("cn.tmp", mx, &w.tmp));
  SM_CHECK(w.buf("cn.tmp2", mx, &w.tmp2));
  SM_CHECK(w.recanonicalize(oldc, newc, err));
  for (int i = 0; i <= L; ++i) bonds[i] = w.bb[i];
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  return SM_OK;
}

template <typename T>
int scprod_impl(Ctx& ctx, cudaStream_t st, int L, const int* phys, const int* ab,
                const void* const* A, const int* bbnd, const void* const* B, double* out) {
  sm_strategy s{};
  Sweeper<T> w(ctx, st, s);
  w.L = L;
  w.d.assign(phys, phys + L);
  std::vector<const T*> a(reinterpret_cast<const T* const*>(A), reinterpret_cast<const T* const*>(A) + L);
  std::vector<const T*> b(reinterpret_cast<const T* const*>(B), reinterpret_cast<const T* const*>(B) + L);
  std::vector<int> av(ab, ab + L + 1), bv(bbnd, bbnd + L + 1);
  return w.scprod(a, av, b, bv, out);
}

#define SM_INST2(T)                                                                             \
  template int simplify_impl<T>(Ctx&, cudaStream_t, int, const int*, int, const double*,       \
                                const double*, const int*, const void* const*,                 \
                                const sm_strategy&, int, void* const*, const int64_t*, int*,   \
                                sm_simplify_report*, const double*, const int*,                \
                                const void* const*);                                           \
  template int canonicalize_impl<T>(Ctx&, cudaStream_t, int, const int*, int*, void* const*,   \
                                    const int64_t*, int, const sm_strategy&, double*);         \
  template int recanonicalize_impl<T>(Ctx&, cudaStream_t, int, const int*, int*, void* const*, \
                                      const int64_t*, int, int, const sm_strategy&, double*);  \
  template int scprod_impl<T>(Ctx&, cudaStream_t, int, const int*, const int*,                 \
                              const void* const*, const int*, const void* const*, double*);
SM_INST2(double)
SM_INST2(cplx)

}  // namespace sm
