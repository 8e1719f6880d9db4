// Internal (C++) interface between the kernels, the sweep driver and the C ABI.
#pragma once

#include <map>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"

namespace sm {

// ---------------------------------------------------------------------------
// Context: scratch device buffers (grown on demand, reused across calls) and a
// small pinned host block for reading back ranks / scalars.
// ---------------------------------------------------------------------------
// BF16 copy of the rank predictor (sm_rank_model_set), used for inference.
struct RankModel {
  bool loaded = false;
  int layers = 0;
  int dims[9] = {};
  __nv_bfloat16* w = nullptr;
  float* b = nullptr;
};

// Prepared DMRG matvec (sm_two_site_prepare): dimensions, the caller's L and
// R (kept alive by the caller), and their tensor-core operand planes.
struct MatvecPrep {
  int precision = -1;  // none prepared
  int a = 0, c = 0, b = 0, p1 = 0, p2 = 0, e = 0, g = 0, f = 0;
  bool tc = false;     // both products on the tensor cores (else the generic path)
  int kpL = 0, kpR = 0;
  const double* L = nullptr;
  const double* R = nullptr;
  void* Lh = nullptr;
  float* Ll = nullptr;
  void* Rh = nullptr;
  float* Rl = nullptr;
};

struct Ctx {
  int device = 0;
  int num_sms = 0;
  int precision = 0;  // SM_PRECISION_FP64, SM_PRECISION_MIXED or SM_PRECISION_MIXED_LEARNED
  // rank features: position of the split being made (set by the sweep
  // driver), the previous split's kept rank and leading singular values,
  // the model, and the recorder (features, kept rank) of every split
  bool contract32 = false;  // mixed forms: sweep contractions in FP32 arithmetic
  bool fp64_tc = true;      // mixed forms: FP64 products on the tensor cores (gemm_oz)
  bool concurrent = false;  // shares the device with other streams: no multi-CTA grid barriers
  // learned rank cap of the FP32 QR: ceil(cap_margin * predicted) + cap_extra rows
  double cap_margin = 1.15;
  int cap_extra = 10;
  // learned form: the predicted rank (or rf_rank_hint > 0 in its place) sizes a
  // randomized range finder of rank + rf_oversample columns and rf_power
  // subspace iterations instead of capping the QR
  bool range_finder = false;
  int rf_oversample = 10;
  int rf_power = 0;
  int rf_rank_hint = 0;
  int split_site = -1, split_n = 0;
  int prev_rank = 0;
  std::vector<double> prev_s;
  const double* last_s = nullptr;  // device: sorted singular values of the last split
  int last_len = 0;
  double* prev_s_dev = nullptr;     // device copy of the last split's 32 largest values
  int prev_len_dev = 0;             //   (the learned form's features, read on the device)
  RankModel model;
  bool record = false;
  std::vector<float> rec_x;
  std::vector<int> rec_y;
  void* pinned = nullptr;  // 64 KB of pinned host memory
  std::map<std::string, std::pair<void*, size_t>> bufs;
  std::map<const void*, int> coop_blocks;  // per-kernel co-resident CTA limit
  // split trace (sm_trace_*): one record per SVD split, singular values included
  sm_stats stats{};
  bool timing = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  MatvecPrep mvp;
  bool trace = false;
  std::vector<int> tr_rank, tr_len;
  std::vector<double> tr_err2, tr_s;
  ~Ctx();
  // Returns a device buffer of at least `bytes` bytes for `name`.  A buffer
  // only grows; growing it synchronises the device (cudaFree).
  int scratch(const std::string& name, size_t bytes, void** out);
  template <typename P>
  int scratch(const std::string& name, size_t count, P** out) {
    return scratch(name, count * sizeof(P), reinterpret_cast<void**>(out));
  }
};

// Raises kernel `fn`'s dynamic shared-memory limit to at least `bytes` (never
// lowers it), under a process-wide lock: contexts on different host threads
// launch the same kernels with different sizes concurrently.
int raise_smem_limit(const void* fn, size_t bytes);
template <typename K>
int raise_smem_limit(K* fn, size_t bytes) {
  return raise_smem_limit(reinterpret_cast<const void*>(fn), bytes);
}

// Cooperative (grid-barrier) launch on `st`.  A multi-CTA grid returns once
// the kernel has completed, holding a process-wide lock meanwhile, so no two
// such kernels of this process overlap.  That alone does not make a grid
// barrier safe next to other streams' work (their kernels can keep the grid's
// remaining CTAs from becoming resident): contexts that share the device set
// `concurrent` and launch these kernels as one CTA.
int coop_launch(const void* fn, dim3 grid, dim3 block, void** args, cudaStream_t st);

// Kernel launches issued by this library in this process (all contexts).
void note_launch(int n = 1);
long long launches_total();

// Kept size and squared discarded weight of a split.
struct SplitResult {
  int D;
  int status;
  double err2;
  int sweeps;
  int pad;
};

// Control block of one Jacobi iteration: grid-barrier words, convergence
// status (DevStatus bits) and the sweep count.
struct JacobiCtl {
  unsigned int bar_count;
  unsigned int bar_gen;
  unsigned int rot[2];
  int status;
  int sweeps;
  int nact;  // rows still taking part in the iteration (deflation / rank)
  int nkeep;  // mixed split: FP32 rows heavy enough to take into the FP64 refinement
  int cap;    // mixed split: the QR cap the cluster kernel used (0: none)
  int pred;   // mixed split: the predicted rank behind a device-side cap (0: none)
};

// Output forms of the two factors of a split A = U diag(s) Vt.
enum { OUT_NONE = 0, OUT_U = 1, OUT_US = 2 };
enum { OUT_VT = 1, OUT_SVT = 2 };

// --- gemm.cu ---------------------------------------------------------------
// GEMM through the context: counts the launch and, when timing is enabled,
// measures it with CUDA events.
template <typename T>
int gemm_ctx(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, T alpha, const T* A,
             int lda, const T* B, int ldb, T beta, T* C, int ldc);
// allow_tc = false keeps the product on the FP64 SIMT kernel in every mode
template <typename T>
int gemm_ctx_sel(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, T alpha,
                 const T* A, int lda, const T* B, int ldb, T beta, T* C, int ldc, bool allow_tc);
template <typename T>
int gemm(cudaStream_t st, int opA, int opB, int M, int N, int K, T alpha, const T* A, int lda,
         const T* B, int ldb, T beta, T* C, int ldc);
// Same contract with FP32 arithmetic (FP64 operands rounded on load, FP32
// accumulation): the contractions of the mixed forms.
template <typename T>
int gemm_ctx_f32(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, T alpha,
                 const T* A, int lda, const T* B, int ldb, T beta, T* C, int ldc);

// --- gemm_tc.cu -------------------------------------------------------------
// Real GEMM at FP32 accuracy on the tensor cores (3xTF32, tcgen05): used by
// gemm_ctx_f32 for shapes gemm_tc_eligible accepts.  Pipeline waits that time
// out set bits of a device status word; tc_status_check reads (and clears) it
// and returns SM_ERR_CUDA when one did.
bool gemm_tc_eligible(int M, int N, int K);
// bf16 = true: one BF16 product (kind::f16, FP32 accumulation) instead of 3xTF32
int gemm_tc(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, double alpha,
            const double* A, int lda, const double* B, int ldb, double beta, double* C, int ldc,
            bool bf16 = false);
// Operands already in tensor-core form: K-contiguous planes of M x kp and
// N x kp (kp a multiple of tc_kslab(bf16)): one BF16 plane, or FP32 hi and lo
// planes for 3xTF32.  tc_planes writes them from an FP64 op(X) (trans as in
// gemm_tc's operand rule); gemm_tc_planes multiplies them, C (double or float)
// = alpha A_planes B_planes^T + beta C.
int tc_kslab(bool bf16);
int tc_planes(Ctx& ctx, cudaStream_t st, const double* X, int ldx, int rows, int K, int kp,
              int trans, bool bf16, void* hi, float* lo);
template <typename OutT>
int gemm_tc_planes(Ctx& ctx, cudaStream_t st, int M, int N, int kp, bool bf16, const void* ah,
                   const float* al, const void* bh, const float* bl, double alpha, double beta,
                   OutT* C, int ldc);
int tc_status(Ctx& ctx, unsigned int** out);
int tc_status_check(Ctx& ctx, cudaStream_t st);

// --- gemm_oz.cu -------------------------------------------------------------
// Real GEMM at FP64 accuracy on the BF16 tensor cores (error-free slicing of
// the operands into 7-bit integer slices); gemm_ctx<double> uses it in the
// mixed forms (ctx.fp64_tc) for shapes gemm_oz_eligible accepts.
bool gemm_oz_eligible(int M, int N, int K);
int gemm_oz(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, double alpha,
            const double* A, int lda, const double* B, int ldb, double beta, double* C, int ldc);

// --- gemm_cplx.cu -------------------------------------------------------------
// Complex product as three real products (3M) on split re / im / re+im planes:
// on the 3xTF32 tensor-core GEMM, or the FP64-accurate one (fp64_accurate).
// Callers check gemm_cplx_tc_eligible / gemm_cplx_oz_eligible on (M, N, K).
bool gemm_cplx_tc_eligible(int M, int N, int K);
bool gemm_cplx_oz_eligible(int M, int N, int K);
int gemm_cplx_3m(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, cplx alpha,
                 const cplx* A, int lda, const cplx* B, int ldb, cplx beta, cplx* C, int ldc,
                 bool fp64_accurate);
// --- rangefinder.cu -------------------------------------------------------------
// BH (l x k) = W^T Q for an orthonormal basis Q of range(W Omega) after
// power_iters subspace iterations (W = A^T if want_u, else A; real); *status
// becomes 1 if a Cholesky pivot was not positive.  k <= range_finder_max_k().
int range_finder_max_k();
int range_finder_bh(Ctx& ctx, cudaStream_t st, const double* A, int m, int n, bool want_u, int k,
                    int power_iters, double* BH, int* status);
// --- dmrg.cu -----------------------------------------------------------------
template <typename T>
int two_site_matvec(Ctx& ctx, cudaStream_t st, int a, int c, int b, int p1, int p2, int e, int g,
                    int f, const T* L, const T* H, const T* R, const T* v, T* out, int precision);
// Prepared form (real, SM_MATVEC_TF32X3 / SM_MATVEC_BF16): L and R become
// operand planes once; ctx.mvp holds them until the next prepare.
int two_site_prepare(Ctx& ctx, cudaStream_t st, int a, int c, int b, int p1, int p2, int e,
                     int g, int f, const double* L, const double* R, int precision);
int two_site_matvec_prepared(Ctx& ctx, cudaStream_t st, const double* H, const double* v,
                             double* out);

// --- mpo_env.cu --------------------------------------------------------------
// Three-leg MPO environments (bra A (a, j, d), MPO O (c, j, i, e), ket B (b, i, f)):
// left rho (a, c, b) -> out (d, e, f); right rho (d, e, f) -> out (a, c, b).
template <typename T>
int mpo_env_left(Ctx& ctx, cudaStream_t st, const T* rho, const T* A, int a, int j, int d,
                 const T* O, int c, int i, int e, const T* B, int b, int f, T* out);
template <typename T>
int mpo_env_right(Ctx& ctx, cudaStream_t st, const T* rho, const T* A, int a, int j, int d,
                  const T* O, int c, int i, int e, const T* B, int b, int f, T* out);
// --- mps_ops.cu ------------------------------------------------------------
template <typename T>
int scale_matrix(cudaStream_t st, int M, int N, T beta, T* C, int ldc);
template <typename T>
int scale_vector(cudaStream_t st, size_t n, double factor, T* x);
template <typename T>
int fill_zero(cudaStream_t st, size_t n, T* x);
template <typename T>
int mpo_multiply_tensor(cudaStream_t st, const T* O, int a, int i, int j, int b, const T* B,
                        int c, int d, T* C);
// C[(a c), i, k, (b d)] = sum_j B[a, i, j, b] A[c, j, k, d] (A applied first, then B)
template <typename T>
int mpo_join(cudaStream_t st, const T* B, int a, int i, int j, int b, const T* A, int c, int k,
             int d, T* C);
// out[0] (+ out[1] for complex) = sum conj(x) y, deterministic two-pass reduction
template <typename T>
int vdot(Ctx& ctx, cudaStream_t st, size_t n, const T* x, const T* y, double* out_dev);
template <typename T>
int transpose(cudaStream_t st, int m, int n, const T* A, int lda, T* B, int ldb);
template <typename T>
int set_identity(cudaStream_t st, int k, T* X, int ldx);
// Copy `n` elements of the mixed-dtype buffers used by the joined MPSSum guess.
template <typename T>
int copy_block3(cudaStream_t st, const T* src, int a, int d, int b, T* dst, int A, int B,
                int off_a, int off_b, T w);

// --- svd.cu ----------------------------------------------------------------
// Exact reference truncation rule on device values s_dev[0..n) (descending).
int truncate_device(Ctx& ctx, cudaStream_t st, const double* s_dev, int n,
                    const sm_strategy& strat, int* rank, double* err2);

// SVD of A (m x n, row-major, leading dim n) followed by truncation with
// `strat`.  Writes the left factor (m x D, mode OUT_U / OUT_US) into `left`
// and the right factor (D x n, mode OUT_VT / OUT_SVT) into `right`; optional
// `s_out` receives all min(m,n) singular values (descending).  The kept size
// D and err^2 are returned on the host (one stream synchronisation).
template <typename T>
int svd_split(Ctx& ctx, cudaStream_t st, const T* A, int m, int n, const sm_strategy& strat,
              int left_mode, T* left, int right_mode, T* right, double* s_out,
              SplitResult* res);

// --- mlp.cu ----------------------------------------------------------------
// The SM_RANK_FEATURES features of a split of size k about to be made.
void rank_features(const Ctx& ctx, int k, const sm_strategy& st, float* f);
// Kept rank of that split predicted by the context's model (1..k).
int rank_predict(Ctx& ctx, cudaStream_t st, int k, const sm_strategy& strat, int* out);
// The same prediction without a host round trip: features from the previous
// split's values on the device, the network, and the QR cap it gives,
// out[0] = cap (0 when above useful min(m, n)), out[1] = the predicted rank.
int rank_predict_dev(Ctx& ctx, cudaStream_t st, int k, const sm_strategy& strat, double useful,
                     int* out);

// --- svd_mixed.cu ------------------------------------------------------------
// Whether the 16-CTA cluster factorisation holds W (kw x l) on this GPU.
// Splits with min(m, n) below this stay on the FP64 path in the mixed forms.
constexpr int kMixedMinRank = 24;
template <typename T>
bool split_cluster_size_ok(int kw, int l);
template <typename T>
bool split_cluster_fits(int kw, int l);
// FP32 rank-revealing QR + one-sided Jacobi of W = (want_u ? A^T : A) in one
// cluster.  Writes kcap rows (FP64, ld = l, zero past the iteration's rows)
// and their norms; ctl receives status / sweeps / nact = rows of R kept;
// info[0] = |A|_F^2 (FP64), info[1] = trailing weight dropped by the QR.
// qr_cap > 0 stops the QR after that many steps (a predicted rank) even if
// the trailing weight is still above the threshold; info[1] then holds the
// weight it left behind.  info needs 7 doubles; vbuf (device) needs
// split_cluster_vbuf_floats(kw) floats, kw = n when U is wanted, else m.
template <typename T>
int split_cluster_f32(cudaStream_t st, const T* A, int m, int n, bool want_u, double thr_rel,
                      double thr_abs, int max_sweeps, T* out_rows, double* out_nrm, int kcap,
                      JacobiCtl* ctl, double* info, int qr_cap, float* vbuf, bool pivot = true,
                      const int* cap_dev = nullptr);
size_t split_cluster_vbuf_floats(int kw);

}  // namespace sm
