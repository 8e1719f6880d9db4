/*
 * seemps_gb300.h — C ABI of the GB300 (sm_103a) MPO·MPS + simplify path.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as void*, may be NULL for the legacy stream) and returns an int
 * status (SM_OK on success).  No entry point takes or returns a PyTorch type.
 * Tensors are C-ordered (row-major):
 *   MPS site  A[a, i, b]        (reference state/mps.py:23-38)
 *   MPO site  O[a, i, j, b]     (reference operators/mpo.py:51-54)
 * dtype SM_FLOAT64 is double; SM_COMPLEX128 is interleaved (re, im) doubles,
 * the byte layout of numpy/torch complex128.
 *
 * Status codes map onto the exceptions the reference raises:
 *   SM_ERR_VALUE     -> ValueError     (bad shapes, e.g. cython/environments.pxi:11-17)
 *   SM_ERR_STRATEGY  -> AssertionError (invalid Strategy, cython/truncation.pxi:103-131)
 *   SM_ERR_LINALG    -> LinAlgError    (SVD did not converge, cython/svd.pxi:80-83)
 *   SM_ERR_CUDA, SM_ERR_TIMEOUT, SM_ERR_NOMEM -> RuntimeError
 * sm_last_error() returns the message of the last failure on this thread.
 */
#ifndef SEEMPS_GB300_H
#define SEEMPS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SM_ABI_VERSION 1

enum {
  SM_OK = 0,
  SM_ERR_VALUE = 1,
  SM_ERR_CUDA = 2,
  SM_ERR_LINALG = 3,
  SM_ERR_TIMEOUT = 4,
  SM_ERR_STRATEGY = 5,
  SM_ERR_NOMEM = 6,
};

enum { SM_FLOAT64 = 0, SM_COMPLEX128 = 1 };
enum { SM_OP_N = 0, SM_OP_T = 1, SM_OP_C = 2 }; /* GemmOrder: cython/gemm.pxi:17-20 */

/* Truncation / Simplification codes: cython/truncation.pxi:4-16 */
enum {
  SM_DO_NOT_TRUNCATE = 0,
  SM_RELATIVE_SINGULAR_VALUE = 1,
  SM_RELATIVE_NORM_SQUARED_ERROR = 2,
  SM_ABSOLUTE_SINGULAR_VALUE = 3,
};
enum {
  SM_DO_NOT_SIMPLIFY = 0,
  SM_CANONICAL_FORM = 1,
  SM_VARIATIONAL = 2,
  SM_VARIATIONAL_EXACT_GUESS = 3,
};

/* Plain-data mirror of the reference cdef class Strategy (cython/truncation.pxi:66-100). */
typedef struct sm_strategy {
  int32_t method;
  int32_t max_bond_dimension;
  double tolerance;
  double simplification_tolerance;
  int32_t normalize;
  int32_t simplify;
  int32_t max_sweeps;
  int32_t reserved;
} sm_strategy;

/* Outcome of a simplify / apply call (state/simplification.py:104-142). */
typedef struct sm_simplify_report {
  double error;           /* total error bound written into the result (mps._error) */
  double norm_state_sqr;  /* |state|^2 used by the stop rule */
  double norm_mps_sqr;    /* |result|^2 before optional normalisation */
  double last_err;        /* final sweep estimate err = 2|1 - Re<mps|state>/..| */
  int32_t sweeps;         /* sweeps actually run */
  int32_t center;         /* orthogonality centre of the result */
  int32_t splits;         /* number of SVD splits performed (canonical + two-site) */
  int32_t zero_state;     /* 1 when |state|^2 == 0 and the zero state was returned */
  double sweep_err[64];   /* per-sweep err estimates (first 64) */
} sm_simplify_report;

/* ---- library / context ------------------------------------------------- */
int sm_abi_version(void);
const char* sm_last_error(void);
/* A context owns scratch device memory and pinned host words; one per thread. */
int sm_ctx_create(void** ctx, int device);
int sm_ctx_destroy(void* ctx);

/* Arithmetic of the splits run through this context (no reference
 * counterpart: the reference always computes in FP64).
 *   SM_PRECISION_FP64  (default) every split is the FP64 Jacobi SVD; ranks and
 *                      singular values follow the reference's gesdd.
 *   SM_PRECISION_MIXED the one-isometry splits of canonical updates and
 *                      simplify sweeps (k >= 24) run an FP32 rank-revealing QR
 *                      + Jacobi inside one 16-CTA cluster, refined by FP64 GEMMs
 *                      against the exact matrix; the discarded weight is exact
 *                      in FP64 and the split falls back to SM_PRECISION_FP64
 *                      when it exceeds the strategy's tolerance with fewer
 *                      than max_bond_dimension values kept.  Ranks may differ
 *                      from the reference's at the tolerance boundary. */
enum { SM_PRECISION_FP64 = 0, SM_PRECISION_MIXED = 1, SM_PRECISION_MIXED_LEARNED = 2 };
/* SM_PRECISION_MIXED_LEARNED: as SM_PRECISION_MIXED, but the rank predictor set
 * with sm_rank_model_set predicts each split's kept rank r and the FP32
 * rank-revealing QR stops after ceil(1.15 r) + 10 steps at most; a split whose
 * capped QR left weight behind (more than 1% of what the tolerance allows
 * outside the rows' span, computed exactly after the refinement) is redone
 * without the cap, and the exact discarded-weight check still sends tolerance
 * violations to the FP64 Jacobi SVD. */
int sm_ctx_set_precision(void* ctx, int precision);
/* SM_PRECISION_MIXED_LEARNED's cap on the FP32 QR: ceil(margin * r) + extra
 * rows for a predicted rank r (default 1.15 and 10; margin >= 1, extra >= 0). */
int sm_ctx_set_rank_cap(void* ctx, double margin, int extra);
/* Arithmetic of the sweep contractions (environments, two-site tensors,
 * canonical absorptions) in the mixed forms: 64 (default, FP64) or 32 (FP32
 * arithmetic on FP64 data, ~1e-7 relative error per contraction).  Ignored in
 * SM_PRECISION_FP64. */
int sm_ctx_set_contraction_bits(void* ctx, int bits);

/* ---- rank predictor (no reference counterpart) ------------------------------
 * An MLP with GELU hidden layers; parameters are one FP32 device array, layer
 * by layer W_k (dims[k+1] x dims[k], row-major) then b_k (dims[k+1]).  The
 * forward / backward / MSE / Adam entry points train it on the GPU; features
 * of every split can be recorded (sm_rank_features_record) together with the
 * kept rank; sm_rank_model_set installs a trained model (dims[0] =
 * SM_RANK_FEATURES, one output = log2 of the kept rank) for
 * SM_PRECISION_MIXED_LEARNED.  Features of a split: log10(s_i / s_0) of the 32
 * largest singular values of the previous split (-20 padding), site / n,
 * log10(tolerance), log2(1 + previous kept rank), log2(min(m, n)),
 * log2(bond cap). */
#define SM_RANK_FEATURES 37
int64_t sm_mlp_param_count(int n_layers, const int* dims);
int64_t sm_mlp_cache_count(int n_layers, const int* dims, int batch);
int sm_mlp_forward(void* ctx, int n_layers, const int* dims, const float* params, const float* X,
                   int batch, float* Y, float* cache, void* stream);
int sm_mlp_backward(void* ctx, int n_layers, const int* dims, const float* params, const float* X,
                    int batch, const float* cache, const float* dY, float* grads, void* stream);
int sm_mse_loss(void* ctx, const float* yhat, const float* y, int batch, float* dyhat, float* loss,
                void* stream);
int sm_adam_step(void* ctx, float* p, const float* g, float* m, float* v, int64_t n, float lr,
                 float beta1, float beta2, float eps, int step, void* stream);
int sm_rank_model_set(void* ctx, int n_layers, const int* dims, const float* params);
int sm_rank_features_record(void* ctx, int on);
int sm_rank_features_read(void* ctx, float* X, int* D, int cap, int* count);
int sm_rank_predict(void* ctx, const float* X, int batch, float* out, void* stream);

/* Kernel-level entry of the mixed split's FP32 stage (no reference
 * counterpart; for unit tests of that stage): rank-revealing QR + one-sided
 * Jacobi of W = (want_u ? A^T : A), A m x n on the device, inside one 16-CTA
 * cluster.  Writes kcap >= min(m,n) + 32 rows of length l (= m if want_u else
 * n) to `rows` (FP64 / complex128, in no particular order, mutually orthogonal
 * to FP32 accuracy, spanning W's row space; zero past *keff) and their norms
 * (= singular values of W) to `nrm`.  *keff = rows the QR kept; *sweeps =
 * Jacobi sweeps.  SM_ERR_VALUE when the sizes exceed the cluster's capacity,
 * SM_ERR_LINALG when the iteration did not converge. */
int sm_split_rows_f32(void* ctx, int dtype, const void* A, int m, int n, int want_u,
                      double thr_rel, double thr_abs, void* rows, double* nrm, int kcap,
                      int* keff, int* sweeps, void* stream);

/* ---- kernel table (replaces seemps.cython, cython/__init__.py:25-54) ----- */

/* destructively_truncate_vector (cython/truncation.pxi:329-334): s_dev holds n
 * descending singular values on the device; returns the kept size and the
 * squared discarded weight with the reference's exact comparisons. */
int sm_truncate(void* ctx, const double* s_dev, int n, const sm_strategy* st,
                int* rank, double* err2, void* stream);

/* _gemm (cython/gemm.pxi:21-122) in row-major form: C[M,N] = op(A) op(B). */
int sm_gemm(void* ctx, int dtype, int opA, int opB, int M, int N, int K,
            const void* A, int lda, const void* B, int ldb, void* C, int ldc,
            void* stream);

/* sm_gemm with scalars: C = alpha op(A) op(B) + beta C (alpha, beta as (re, im)
 * pairs; beta = 0 does not read C).  FP64 SIMT kernel. */
int sm_gemm_ex(void* ctx, int dtype, int opA, int opB, int M, int N, int K,
               const double* alpha, const void* A, int lda, const void* B, int ldb,
               const double* beta, void* C, int ldc, void* stream);

/* The same product at FP64 accuracy on the BF16 tensor cores (no reference
 * counterpart): real operands with M, N >= 32, K >= 32 and at least 2 Mi
 * multiply-adds are scaled by powers of two per row of op(A) / column of
 * op(B), cut into 8 slices of 7-bit integers (exact in BF16) and multiplied
 * slice by slice with tcgen05 (Ozaki, Ogita, Oishi and Rump, Numer. Algorithms
 * 59, 2012), exact FP32 accumulation over chunks of 256 and FP64 across
 * chunks; the error is that of an FP64 GEMM.  Complex operands are held as
 * split real planes (re, im, re + im) and multiplied with three real products
 * of this kind (T1 = Ar Br, T2 = Ai Bi, T3 = (Ar+Ai)(Br+Bi); C = T1 - T2 +
 * i (T3 - T1 - T2)).  Shapes below the tensor-core threshold run the FP64 SIMT
 * kernel.  The mixed precision forms route their
 * FP64 products here (sm_ctx_set_fp64_products). */
int sm_gemm_f64tc(void* ctx, int dtype, int opA, int opB, int M, int N, int K,
                  const void* A, int lda, const void* B, int ldb, void* C, int ldc,
                  void* stream);
/* Marks a context whose calls run concurrently with other streams' work on the
 * same device (several host threads, each with its own context and stream):
 * the FP64 SVD's grid-barrier kernels (Householder QR, Jacobi) then run as one
 * CTA, since a multi-CTA grid barrier can wait indefinitely for CTAs that other
 * streams' kernels keep from being resident (its bounded spin then reports
 * SM_ERR_TIMEOUT).  seemps2_gb300.batch sets it on its worker contexts. */
int sm_ctx_set_concurrent(void* ctx, int on);

/* Learned form (SM_PRECISION_MIXED_LEARNED) with on != 0: the predicted kept
 * rank r (or rank_hint in its place when > 0, no model needed) sizes a
 * randomized range finder (Halko, Martinsson and Tropp, SIAM Rev. 53, 2011):
 * k = r + oversample columns of W Omega, power_iters subspace iterations
 * (3xTF32 products, shifted CholeskyQR between them), B^T = W^T Q.  The FP32
 * cluster factorisation then works on B^T (rows of length k) instead of W;
 * the FP64 refinement against the exact W, the exact discarded weight and the
 * redo with the full QR when the subspace missed weight are those of the QR
 * cap.  Real operands; on = 0 (default) caps the QR instead.  No reference
 * counterpart. */
int sm_ctx_set_range_finder(void* ctx, int on, int oversample, int power_iters, int rank_hint);
/* The range finder alone: BH (l x k, row-major) = W^T Q for W = A^T (want_u)
 * or A (real A, m x n, l = the length of W's rows), Q an orthonormal basis of
 * the range of W Omega after power_iters subspace iterations; k <= min(m, n,
 * 640).  No reference counterpart. */
int sm_range_finder(void* ctx, const double* A, int m, int n, int want_u, int k, int power_iters,
                    double* BH, void* stream);

/* FP64 products of the mixed forms (state norm, refinement, final estimate,
 * FP64 contractions): 1 (default) on the tensor cores as sm_gemm_f64tc, 0 on
 * the FP64 SIMT kernel.  SM_PRECISION_FP64 always uses the SIMT kernel. */
int sm_ctx_set_fp64_products(void* ctx, int tensor_cores);

/* The same product at FP32 accuracy: the contractions of the mixed precision
 * forms (sm_ctx_set_contraction_bits(ctx, 32)).  Real operands with
 * M, N >= 64, K >= 32 and at least 4 Mi multiply-adds run 3xTF32 on the
 * tensor cores (tcgen05, FP32 accumulation); complex operands of those shapes
 * as three real 3xTF32 products on split re / im / re+im planes (the 3M form);
 * other shapes run an FP32 SIMT kernel.  No reference counterpart (the reference
 * contracts in FP64). */
int sm_gemm_f32(void* ctx, int dtype, int opA, int opB, int M, int N, int K,
                const void* A, int lda, const void* B, int ldb, void* C, int ldc,
                void* stream);

/* _destructive_svd (cython/svd.pxi:17-83): economy SVD A[m,n] = U diag(s) Vt,
 * s descending; U is m x r, Vt is r x n, r = min(m, n).  A is not modified. */
int sm_svd(void* ctx, int dtype, const void* A, int m, int n, void* U, double* s,
           void* Vt, void* stream);

/* _left_orth_2site (cython/schmidt.pxi:123-147): AA[a,d1,d2,b] ->
 * U[a,d1,D] (left isometry) and SV[D,d2,b].  Buffers U and SV must hold
 * a*d1*r and r*d2*b elements (r = min(a*d1, d2*b)); outputs are written
 * contiguously for the kept D.  *err = sqrt(discarded weight). */
int sm_left_orth_2site(void* ctx, int dtype, const void* AA, int a, int d1, int d2,
                       int b, const sm_strategy* st, void* U, void* SV, int* D,
                       double* err, void* stream);
/* Allocation-free _left_orth_2site.  No counterpart in the reference: it is the
 * same split as sm_left_orth_2site for callers that cannot allocate device
 * memory while they run (host applications that own all device memory through
 * their own pool, plugins that are only handed buffers, loops where a
 * cudaMalloc would synchronise the device).  It needs no context and calls no
 * cudaMalloc/cudaFree or allocating library routine: its intermediates live
 * in a static device array (about 2 MiB, held by every GPU that loads the
 * library until exit).  Limit: a*d1 <= 256 and d2*b <= 256, larger inputs
 * return SM_ERR_VALUE.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress), so make that first call before any stream
 * capture.  All calls share the array and it keeps the last call's contents;
 * calls that overlap on the GPU race on it, so serialise them.  Every call
 * reads the kept rank back to the host, so it synchronises `stream` before it
 * returns.  Its Jacobi stage is a cooperative multi-CTA kernel; if kernels of
 * other streams keep its CTAs off the SMs, its bounded barrier times out and
 * the call redoes the split with a one-CTA Jacobi (slower, same result). */
int sm_left_orth_2site_noalloc(int dtype, const void* AA, int a, int d1, int d2, int b,
                               const sm_strategy* st, void* U, void* SV, int* D,
                               double* err, void* stream);
/* _right_orth_2site (cython/schmidt.pxi:150-174): -> US[a,d1,D], V[D,d2,b]. */
int sm_right_orth_2site(void* ctx, int dtype, const void* AA, int a, int d1, int d2,
                        int b, const sm_strategy* st, void* US, void* V, int* D,
                        double* err, void* stream);

/* update_left_mpo_environment (state/environments.py:19-30): out[d, e, f] =
 * sum conj(A[a, j, d]) rho[a, c, b] O[c, j, i, e] B[b, i, f] with the bra site A
 * (a, j, d), the MPO site O (c, j, i, e), the ket site B (b, i, f) and rho
 * (a, c, b). */
int sm_update_left_mpo_environment(void* ctx, int dtype, const void* rho, const void* A, int a,
                                   int j, int d, const void* O, int c, int i, int e,
                                   const void* B, int b, int f, void* out, void* stream);
/* update_right_mpo_environment (state/environments.py:33-42): out[a, c, b] =
 * sum conj(A[a, j, d]) rho[d, e, f] O[c, j, i, e] B[b, i, f] (shapes as above,
 * rho (d, e, f)). */
int sm_update_right_mpo_environment(void* ctx, int dtype, const void* rho, const void* A, int a,
                                    int j, int d, const void* O, int c, int i, int e,
                                    const void* B, int b, int f, void* out, void* stream);

/* One site of MPOList.join (operators/mpo.py:679-711) for two MPOs, A applied
 * first and B after it: C[(a c), i, k, (b d)] = sum_j B[a, i, j, b] A[c, j, k, d]
 * with B (a, i, j, b), A (c, j, k, d) and C (a*c, i, k, b*d). */
int sm_mpo_join(void* ctx, int dtype, const void* B, int a, int i, int j, int b, const void* A,
                int c, int k, int d, void* C, void* stream);

/* _update_left_environment (cython/environments.pxi:10-37):
 * out[n,k] = sum conj(B[l,j,n]) rho[l,i] A[i,j,k]; B is (l,j,n), A is (i,j,k). */
int sm_update_left_environment(void* ctx, int dtype, const void* B, int l, int j,
                               int n, const void* A, int i, int k, const void* rho,
                               void* out, void* stream);
/* _update_right_environment (cython/environments.pxi:39-67):
 * out[i,l] = sum A[i,j,k] rho[k,n] conj(B[l,j,n]). */
int sm_update_right_environment(void* ctx, int dtype, const void* B, int l, int j,
                                int n, const void* A, int i, int k, const void* rho,
                                void* out, void* stream);

/* _mpo_multiply_tensor (operators/mpo.py:26-45):
 * C[c*a, i, d*b] = sum_j B[c,j,d] O[a,i,j,b]. */
int sm_mpo_multiply_tensor(void* ctx, int dtype, const void* O, int a, int i, int j,
                           int b, const void* B, int c, int d, void* C, void* stream);

/* scprod (cython/environments.pxi:87-118) of two MPS with L sites; site
 * pointers and bonds (L+1 each) per state; result written to out[0] (and the
 * imaginary part to out[1] for complex). */
int sm_scprod(void* ctx, int dtype, int L, const int* phys, const int* bra_bonds,
              const void* const* bra, const int* ket_bonds, const void* const* ket,
              double* out, void* stream);

/* _canonicalize (cython/schmidt.pxi:109-120) in place: sites[i] buffers must
 * hold cap[i] elements; bonds (L+1) are updated; *err = summed sqrt errors. */
int sm_canonicalize(void* ctx, int dtype, int L, const int* phys, int* bonds,
                    void* const* sites, const int64_t* cap, int center,
                    const sm_strategy* st, double* err, void* stream);

/* _recanonicalize (cython/schmidt.pxi:96-106) in place: moves the centre from
 * oldcenter to newcenter one site at a time with the truncated SVD updates of
 * _update_in_canonical_form_*; same buffer rules as sm_canonicalize. */
int sm_recanonicalize(void* ctx, int dtype, int L, const int* phys, int* bonds,
                      void* const* sites, const int64_t* cap, int oldcenter, int newcenter,
                      const sm_strategy* st, double* err, void* stream);

/* __update_in_canonical_form_right (cython/schmidt.pxi:18-42, the body of
 * _update_in_canonical_form_right :45-56): SVD of A (a*i x b), truncation,
 * U -> U_out (a, i, D) and (s V) @ next -> next_out (D, j, c), where next is the
 * following site (b, j, c).  U_out holds a*i*min(a*i, b) elements, next_out
 * min(a*i, b)*j*c.  *err = sqrt(discarded weight). */
int sm_update_in_canonical_form_right(void* ctx, int dtype, const void* A, int a, int i,
                                      int b, const void* next, int j, int c,
                                      const sm_strategy* st, void* U_out, void* next_out,
                                      int* D, double* err, void* stream);
/* __update_in_canonical_form_left (cython/schmidt.pxi:59-82, body of
 * _update_in_canonical_form_left :84-93): SVD of A (a x i*b), truncation,
 * V -> V_out (D, i, b) and prev @ (U s) -> prev_out (p, j, D), where prev is the
 * preceding site (p, j, a).  V_out holds min(a, i*b)*i*b elements, prev_out
 * p*j*min(a, i*b). */
int sm_update_in_canonical_form_left(void* ctx, int dtype, const void* A, int a, int i, int b,
                                     const void* prev, int p, int j, const sm_strategy* st,
                                     void* V_out, void* prev_out, int* D, double* err,
                                     void* stream);

/* _contract_nrjl_ijk_klm (cython/contractions.pxi:102-127):
 * out[i, n, r, m] = sum U[(n r), (j l)] A[i, j, k] B[k, l, m] with A (a, d, b),
 * B (b, e, c) and U (nr x d*e), nr = d*e; out is (a, d, e, c). */
int sm_contract_nrjl_ijk_klm(void* ctx, int dtype, const void* U, int nr, const void* A,
                             int a, int d, int b, const void* B, int e, int c, void* out,
                             void* stream);

/* AntilinearForm.tensor2site (state/antilinear.py:68-98): out[l, d1, d2, r] =
 * sum L[l, i] A[i, d1, k] B[k, d2, n] R[n, r] for the environments L (l x i),
 * R (n x r) and the ket sites A (i, d1, k), B (k, d2, n). */
int sm_tensor2site(void* ctx, int dtype, const void* L, int l, int i, const void* A, int d1,
                   int k, const void* B, int d2, int n, const void* R, int r, void* out,
                   void* stream);

/* _select_svd_driver (cython/svd.pxi:25-32): "gesdd" or "gesvd", else
 * SM_ERR_VALUE.  The reference picks a LAPACK driver; the device has one SVD
 * (QR-preconditioned one-sided Jacobi) whose singular values and kept ranks
 * agree with either driver's, so the choice is recorded (sm_svd_driver: 0 =
 * gesdd, 1 = gesvd) and changes no result. */
int sm_select_svd_driver(const char* name);
int sm_svd_driver(void);

/* simplify / simplify_mps_sum (state/simplification.py:32-280) of
 * sum_t w_t |psi_t> (nterms >= 1; weights as (re, im) pairs).  ket_bonds holds
 * nterms*(L+1) ints, ket_sites nterms*L pointers, term_errors the nterms
 * accumulated errors of the input states (MPS._error).  The result is written
 * into out_sites[i] (capacity out_cap[i] elements) with bonds out_bonds (L+1);
 * out_cap comes from sm_simplify_bond_caps.  A single state (nterms == 1) uses
 * its weight as given by the caller (1.0 for simplify(MPS)). */
int sm_simplify(void* ctx, int dtype, int L, const int* phys, int nterms,
                const double* weights, const int* ket_bonds,
                const void* const* ket_sites, const double* term_errors,
                const sm_strategy* st, int direction, void* const* out_sites,
                const int64_t* out_cap, int* out_bonds, sm_simplify_report* rep,
                void* stream);

/* sm_simplify with the terms' products given: gram holds nterms*nterms
 * complex pairs, gram[2*(i*nterms+j)] + 1j*gram[2*(i*nterms+j)+1] = <psi_i|psi_j>,
 * used where the reference takes scprod of the terms for the state norm
 * (state/simplification.py:101 for one state, delete_zero_components at
 * :176 for sums).  MPO.apply (operators/mpo.py:229-281) fills it from
 * sm_mpo_scprod, so the norm of the bond-(chi*D) product is never contracted.
 * Results equal sm_simplify's to FP64 rounding of the norm. */
int sm_simplify_gram(void* ctx, int dtype, int L, const int* phys, int nterms,
                     const double* weights, const int* ket_bonds,
                     const void* const* ket_sites, const double* term_errors,
                     const double* gram, const sm_strategy* st, int direction,
                     void* const* out_sites, const int64_t* out_cap, int* out_bonds,
                     sm_simplify_report* rep, void* stream);

/* sm_simplify (gram may be null, else as for sm_simplify_gram) starting the
 * variational sweeps from a caller's guess instead of the joined kets: the
 * `guess` argument of simplify / simplify_mps_sum (state/simplification.py:
 * 36,93-98 and :150-155,214-219).  The guess (bonds guess_bonds (L+1), sites
 * guess_sites) is copied and brought to canonical form at the start site with
 * the strategy's truncation, as CanonicalMPS(guess, center=start) does; the
 * caller's buffers are not modified.  out_cap must also cover the guess's
 * bonds.  Only the variational methods use the guess (as in the reference). */
int sm_simplify_guess(void* ctx, int dtype, int L, const int* phys, int nterms,
                      const double* weights, const int* ket_bonds,
                      const void* const* ket_sites, const double* term_errors,
                      const double* gram, const int* guess_bonds,
                      const void* const* guess_sites, const sm_strategy* st, int direction,
                      void* const* out_sites, const int64_t* out_cap, int* out_bonds,
                      sm_simplify_report* rep, void* stream);

/* <O bra|O ket> for an MPO O (site i: mpo_bonds[i] x dout[i] x din[i] x
 * mpo_bonds[i+1]) and two MPS with physical dimensions din: the scprod
 * (cython/environments.pxi:87-118) of the products O|bra>, O|ket>
 * (_mpo_multiply_tensor, operators/mpo.py:26-45) computed from the factors
 * with environments E[x, alpha, beta, y], 4 d D^2 chi^3 flops per site instead
 * of 4 d (D chi)^3.  out[0] (+ out[1] for complex) as for sm_scprod. */
int sm_mpo_scprod(void* ctx, int dtype, int L, const int* dout, const int* din,
                  const int* mpo_bonds, const void* const* mpo, const int* bra_bonds,
                  const void* const* bra, const int* ket_bonds, const void* const* ket,
                  double* out, void* stream);

/* Two-site effective-Hamiltonian matvec of DMRG (QuadraticForm.two_site_operator
 * ._matvec, operators/quadratic.py:187-237):
 *   out[a, ko, lo, g] = sum L[a, c, b] v[b, k, l, f] H[c, ko, k, lo, l, e] R[g, e, f]
 * with L (a, c, b) the left MPO environment (bra, MPO, ket), H (c, p1, p1, p2,
 * p2, e) the two-site MPO (_contract_last_and_first of the two sites' MPO
 * tensors), R (g, e, f) the right environment, v (b, p1, p2, f) and out (a,
 * p1, p2, g).  dims = {a, c, b, p1, p2, e, g, f}.  precision: SM_MATVEC_FP64
 * (SIMT FP64, the reference's arithmetic), SM_MATVEC_FP64TC (FP64-accurate on
 * the BF16 tensor cores), SM_MATVEC_TF32X3 (FP32-accurate, 3xTF32) or
 * SM_MATVEC_BF16 (one BF16 product, FP32 accumulation); real operands only on
 * the tensor cores (complex ones use the SIMT kernels of the same accuracy
 * class).  No reference counterpart for the reduced precisions. */
enum { SM_MATVEC_FP64 = 0, SM_MATVEC_FP64TC = 1, SM_MATVEC_TF32X3 = 2, SM_MATVEC_BF16 = 3 };
int sm_two_site_matvec(void* ctx, int dtype, const int* dims, const void* L, const void* H,
                       const void* R, const void* v, void* out, int precision, void* stream);

/* Prepared two-site matvec for a Lanczos run (real FP64 operands; precision
 * SM_MATVEC_TF32X3 or SM_MATVEC_BF16).  sm_two_site_prepare converts L and R
 * (dims as above) into tensor-core operand planes held by the context; the
 * caller keeps L and R alive and unchanged until the next prepare.
 * sm_two_site_matvec_prepared then computes out from H and v with only v
 * converted per call, X1 kept in FP32 and the MPO step writing the second
 * product's operand directly (the same operator as sm_two_site_matvec; the
 * reference applies its matvec to a fixed operator in the same way,
 * operators/quadratic.py:187-237 inside eigsh, optimization/dmrg.py:15-23). */
int sm_two_site_prepare(void* ctx, const int* dims, const void* L, const void* R, int precision,
                        void* stream);
int sm_two_site_matvec_prepared(void* ctx, const void* H, const void* v, void* out,
                                void* stream);

/* Upper bound on the bond dimensions a simplify of these kets can produce:
 * min(max_bond_dimension, summed ket bond); fills cap_bonds (L+1). */
int sm_simplify_bond_caps(int L, const int* phys, int nterms, const int* ket_bonds,
                          const sm_strategy* st, int* cap_bonds);

/* Split trace.  While enabled, every SVD split run by this context appends a
 * record: its singular values (all of them, descending), the kept rank and
 * the squared discarded weight.  sm_trace_enable clears the trace.
 * sm_trace_read with null buffers returns the record count and the total
 * number of singular values; with buffers it copies them out. */
int sm_trace_enable(void* ctx, int on);
int sm_trace_read(void* ctx, int* count, int64_t* total_s, int* ranks, int* lens,
                  double* err2, double* svals);

/* Counters of this context.  Launch counts are always kept; per-kernel device
 * times (CUDA events around each Jacobi SVD launch and each GEMM) are only
 * recorded while timing is enabled.  Algorithmic flops follow the usual
 * convention: 2MNK per real GEMM (x4 complex), 4mn^2 + 8n^3 per m x n SVD
 * (m >= n, x4 complex). */
typedef struct sm_stats {
  int64_t launches;        /* kernels launched by this library */
  int64_t jacobi_launches;
  int64_t jacobi_sweeps;   /* Jacobi sweeps summed over launches */
  int64_t gemm_launches;
  int64_t splits;          /* SVD splits */
  double jacobi_ms;        /* event-timed device time of the Jacobi kernels */
  double jacobi_flops;     /* algorithmic SVD flops of those launches */
  double gemm_ms;          /* event-timed device time of the GEMMs */
  double gemm_flops;
  int64_t mixed_splits;    /* splits attempted in SM_PRECISION_MIXED */
  int64_t mixed_fallbacks; /* of those, redone by the FP64 path */
  int64_t mixed_rows;      /* rows of R carried into the cluster Jacobi, summed */
  double cluster_ms;       /* event-timed device time of the cluster kernel */
  double cluster_qr_ms;    /* of which: load + FP32 QR (device timer) */
  double cluster_jacobi_ms;/* of which: FP32 Jacobi + store (device timer) */
  int64_t mixed_fallback_cut;  /* fallbacks: kept/dropped coupling left after refinement */
  int64_t mixed_fallback_fp32; /* fallbacks: FP32 stage (convergence, resolution, weight) */
  int64_t mixed_capped;      /* mixed splits whose QR the predicted rank capped */
  int64_t mixed_cap_redone; /* capped QR left weight: redone without the cap */
  int64_t rank_predicted_sum;  /* predicted kept ranks, summed */
  int64_t gemm32_launches;     /* contractions computed in FP32 (mixed forms) */
  double gemm32_flops;
  double gemm32_ms;            /* event-timed (stats timing on) */
  int64_t gemm_tc_launches;    /* of those, on the tensor cores (3xTF32, tcgen05) */
  double gemm_tc_flops;        /* 2 M N K of those (the MMAs run 3x this) */
  double gemm_tc_ms;           /* event-timed (stats timing on), split + MMA + reduce */
  int64_t mixed_fallback_over; /* of the FP32 fallbacks: exact discarded weight over tolerance */
  int64_t mixed_fallback_unconverged; /* of the FP32 fallbacks: FP32 iteration did not converge */
  int64_t gemm_oz_launches;    /* FP64 products on the BF16 tensor cores (mixed forms) */
  double gemm_oz_flops;        /* 2 M N K of those */
  double gemm_oz_ms;           /* event-timed (stats timing on), slicing + MMA + reduce */
  double cluster_flops;        /* FP32 work of the cluster kernel as run: QR 4 (kw-j)(l-j-1) per
                                  reflector j, Jacobi 12 l per pair and sweep (x4 complex) */
  double cluster_alg_flops;    /* algorithmic SVD work of the cluster launches: 4mn^2 + 8n^3 per
                                  m x n split (m >= n, x4 complex) */
  double cluster_bytes;        /* algorithmic bytes of the cluster launches: the split matrix read
                                  once and the converged rows written */
  int64_t rf_splits;           /* mixed splits that ran the randomized range finder */
  int64_t mixed_ns_steps;      /* Newton-Schulz steps of the mixed splits (one, or two for rows
                                  below FP32 resolution) */
  int64_t rank_predictions;    /* splits whose kept rank the predictor (or a rank hint) gave */
} sm_stats;
int sm_stats_reset(void* ctx, int timing);
int sm_stats_read(void* ctx, sm_stats* out);

#ifdef __cplusplus
}
#endif

#endif /* SEEMPS_GB300_H */
