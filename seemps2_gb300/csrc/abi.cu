// extern "C" boundary of libseemps_gb300.so (declared in include/seemps_gb300.h).
#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <cmath>
#include <string>

#include "kernels.cuh"

namespace sm {

template <typename T>
int simplify_impl(Ctx&, cudaStream_t, int, const int*, int, const double*, const double*,
                  const int*, const void* const*, const sm_strategy&, int, void* const*,
                  const int64_t*, int*, sm_simplify_report*, const double*, const int*,
                  const void* const*);
template <typename T>
int mpo_scprod_impl(Ctx&, cudaStream_t, int, const int*, const int*, const int*,
                    const void* const*, const int*, const void* const*, const int*,
                    const void* const*, double*);
template <typename T>
int canonicalize_impl(Ctx&, cudaStream_t, int, const int*, int*, void* const*, const int64_t*,
                      int, const sm_strategy&, double*);
template <typename T>
int scprod_impl(Ctx&, cudaStream_t, int, const int*, const int*, const void* const*, const int*,
                const void* const*, double*);
template <typename T>
int recanonicalize_impl(Ctx&, cudaStream_t, int, const int*, int*, void* const*, const int64_t*,
                        int, int, const sm_strategy&, double*);

static thread_local std::string g_error;
static std::atomic<long long> g_launches{0};
void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int coop_launch(const void* fn, dim3 grid, dim3 block, void** args, cudaStream_t st) {
  if (grid.x * grid.y * grid.z == 1) {  // one CTA: its barrier waits for no one
    SM_CUDA_CHECK(cudaLaunchCooperativeKernel(fn, grid, block, args, 0, st));
    return SM_OK;
  }
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  SM_CUDA_CHECK(cudaLaunchCooperativeKernel(fn, grid, block, args, 0, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  return SM_OK;
}

int raise_smem_limit(const void* fn, size_t bytes) {
  static std::mutex mu;
  static std::map<const void*, size_t> limit;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = limit[fn];
  if (bytes <= cur) return SM_OK;
  SM_CUDA_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
  return SM_OK;
}
long long launches_total() { return g_launches.load(std::memory_order_relaxed); }
void set_error(const std::string& msg) { g_error = msg; }
const char* last_error() { return g_error.c_str(); }

Ctx::~Ctx() {
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  for (auto& kv : bufs)
    if (kv.second.first) cudaFree(kv.second.first);
  if (pinned) cudaFreeHost(pinned);
}

int Ctx::scratch(const std::string& name, size_t bytes, void** out) {
  bytes = std::max<size_t>(bytes, 16);
  auto it = bufs.find(name);
  if (it != bufs.end() && it->second.second >= bytes) {
    *out = it->second.first;
    return SM_OK;
  }
  if (it != bufs.end() && it->second.first) {
    cudaError_t e = cudaFree(it->second.first);  // synchronises the device
    it->second = {nullptr, 0};
    if (e != cudaSuccess) {
      set_error(std::string("cudaFree: ") + cudaGetErrorString(e));
      return SM_ERR_CUDA;
    }
  }
  // round up to reduce regrowth
  size_t alloc = bytes + bytes / 8;
  alloc = (alloc + 255) & ~size_t(255);
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, alloc);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaMalloc of " + std::to_string(alloc) + " bytes for '" + name + "' failed: " +
              cudaGetErrorString(e));
    return SM_ERR_NOMEM;
  }
  bufs[name] = {p, alloc};
  *out = p;
  return SM_OK;
}

static int check_strategy(const sm_strategy* st) {
  if (!st) {
    set_error("null strategy");
    return SM_ERR_VALUE;
  }
  if (st->tolerance < 0 || st->tolerance >= 1.0) {
    set_error("Invalid tolerance argument passed to Strategy");
    return SM_ERR_STRATEGY;
  }
  if (st->max_bond_dimension <= 0) {
    set_error("Invalid bond dimension in Strategy");
    return SM_ERR_STRATEGY;
  }
  if (st->method < 0 || st->method > 3) {
    set_error("Invalid method argument passed to Strategy");
    return SM_ERR_STRATEGY;
  }
  if (st->simplify < 0 || st->simplify > 3) {
    set_error("Invalid simplify argument passed to Strategy");
    return SM_ERR_STRATEGY;
  }
  if (st->max_sweeps < 0) {
    set_error("Negative or zero number of sweeps in Strategy");
    return SM_ERR_STRATEGY;
  }
  return SM_OK;
}

static int check_dtype(int dtype) {
  if (dtype != SM_FLOAT64 && dtype != SM_COMPLEX128) {
    set_error("dtype must be SM_FLOAT64 or SM_COMPLEX128");
    return SM_ERR_VALUE;
  }
  return SM_OK;
}

static Ctx* as_ctx(void* c) { return reinterpret_cast<Ctx*>(c); }
static cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

#define SM_GUARD_CTX(c)                  \
  if (!(c)) {                            \
    ::sm::set_error("null context");     \
    return SM_ERR_VALUE;                 \
  }

template <typename T>
static int split2(Ctx* ctx, cudaStream_t st, const void* AA, int a, int d1, int d2, int b,
                  const sm_strategy* s, int lmode, void* L, int rmode, void* R, int* D,
                  double* err) {
  SplitResult r;
  SM_CHECK(svd_split<T>(*ctx, st, reinterpret_cast<const T*>(AA), a * d1, d2 * b, *s, lmode,
                        reinterpret_cast<T*>(L), rmode, reinterpret_cast<T*>(R), nullptr, &r));
  *D = r.D;
  *err = std::sqrt(r.err2);
  return SM_OK;
}

template <typename T>
static int env_left(Ctx* ctx, cudaStream_t st, const void* B, int l, int j, int n, const void* A,
                    int i, int k, const void* rho, void* out) {
  T* tmp;
  SM_CHECK(ctx->scratch("abi.env", (size_t)l * j * k, &tmp));
  const T one = S<T>::one(), zero = S<T>::zero();
  SM_CHECK(gemm_ctx<T>(*ctx, st, SM_OP_N, SM_OP_N, l, j * k, i, one, (const T*)rho, i, (const T*)A,
                       j * k, zero, tmp, j * k));
  return gemm_ctx<T>(*ctx, st, SM_OP_C, SM_OP_N, n, k, l * j, one, (const T*)B, n, tmp, k, zero,
                     (T*)out, k);
}

template <typename T>
static int env_right(Ctx* ctx, cudaStream_t st, const void* B, int l, int j, int n,
                     const void* A, int i, int k, const void* rho, void* out) {
  T* tmp;
  SM_CHECK(ctx->scratch("abi.env", (size_t)i * j * n, &tmp));
  const T one = S<T>::one(), zero = S<T>::zero();
  SM_CHECK(gemm_ctx<T>(*ctx, st, SM_OP_N, SM_OP_N, i * j, n, k, one, (const T*)A, k, (const T*)rho,
                       n, zero, tmp, n));
  return gemm_ctx<T>(*ctx, st, SM_OP_N, SM_OP_C, i, l, j * n, one, tmp, j * n, (const T*)B, j * n,
                     zero, (T*)out, l);
}

// out[j][i][k] = in[i][j][k] for an n0 x n1 x n2 array (swap of the first two axes).
template <typename T>
__global__ void k_swap01(const T* __restrict__ in, int n0, int n1, int n2, T* __restrict__ out) {
  const size_t total = (size_t)n0 * n1 * n2;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < total;
       x += (size_t)gridDim.x * blockDim.x) {
    const size_t k = x % n2;
    const size_t r = x / n2;
    const size_t j = r % n1;
    const size_t i = r / n1;
    out[(j * n0 + i) * n2 + k] = in[x];
  }
}

template <typename T>
static int swap01(cudaStream_t st, const T* in, int n0, int n1, int n2, T* out) {
  const size_t total = (size_t)n0 * n1 * n2;
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>((total + 255) / 256, 152 * 16));
  k_swap01<T><<<blocks, 256, 0, st>>>(in, n0, n1, n2, out);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

// _update_in_canonical_form_right (cython/schmidt.pxi:18-42): split A (a*i x b),
// U -> U_out (a, i, D), (s V) @ next -> next_out (D, j, c).
template <typename T>
static int canon_update_right(Ctx* ctx, cudaStream_t st, const T* A, int a, int i, int b,
                              const T* next, int j, int c, const sm_strategy& s, T* U,
                              T* next_out, int* D, double* err) {
  const int r = std::min(a * i, b);
  T* sv;
  SM_CHECK(ctx->scratch("kt.sv", (size_t)r * b, &sv));
  SplitResult res;
  SM_CHECK(svd_split<T>(*ctx, st, A, a * i, b, s, OUT_U, U, OUT_SVT, sv, nullptr, &res));
  SM_CHECK(gemm_ctx<T>(*ctx, st, SM_OP_N, SM_OP_N, res.D, j * c, b, S<T>::one(), sv, b, next,
                       j * c, S<T>::zero(), next_out, j * c));
  *D = res.D;
  *err = std::sqrt(res.err2);
  return SM_OK;
}

// _update_in_canonical_form_left (cython/schmidt.pxi:59-82): split A (a x i*b),
// V -> V_out (D, i, b), prev @ (U s) -> prev_out (p, j, D).
template <typename T>
static int canon_update_left(Ctx* ctx, cudaStream_t st, const T* A, int a, int i, int b,
                             const T* prev, int p, int j, const sm_strategy& s, T* V,
                             T* prev_out, int* D, double* err) {
  const int r = std::min(a, i * b);
  T* us;
  SM_CHECK(ctx->scratch("kt.us", (size_t)a * r, &us));
  SplitResult res;
  SM_CHECK(svd_split<T>(*ctx, st, A, a, i * b, s, OUT_US, us, OUT_VT, V, nullptr, &res));
  SM_CHECK(gemm_ctx<T>(*ctx, st, SM_OP_N, SM_OP_N, p * j, res.D, a, S<T>::one(), prev, a, us,
                       res.D, S<T>::zero(), prev_out, res.D));
  *D = res.D;
  *err = std::sqrt(res.err2);
  return SM_OK;
}

// _contract_nrjl_ijk_klm (cython/contractions.pxi:102-127):
// out[i, x, m] = sum_y U[x, y] (A B)[i, y, m], with (A B)[i, (j l), m] =
// sum_k A[i, j, k] B[k, l, m].  Formed as one product A B, a swap of its first
// two axes, one product with U and the swap back.
template <typename T>
static int contract_nrjl(Ctx* ctx, cudaStream_t st, const T* U, int nr, const T* A, int a, int d,
                         int b, const T* B, int e, int c, T* out) {
  const int de = d * e;
  const size_t n = (size_t)a * de * c;
  T *ab, *sw;
  SM_CHECK(ctx->scratch("kt.ab", n, &ab));
  SM_CHECK(ctx->scratch("kt.sw", n, &sw));
  const T one = S<T>::one(), zero = S<T>::zero();
  SM_CHECK(gemm_ctx<T>(*ctx, st, SM_OP_N, SM_OP_N, a * d, e * c, b, one, A, b, B, e * c, zero, ab,
                       e * c));
  SM_CHECK(swap01<T>(st, ab, a, de, c, sw));                     // (de, a, c)
  SM_CHECK(gemm_ctx<T>(*ctx, st, SM_OP_N, SM_OP_N, nr, a * c, de, one, U, de, sw, a * c, zero, ab,
                       a * c));                                    // (nr, a, c)
  return swap01<T>(st, ab, nr, a, c, out);                         // (a, nr, c)
}

// AntilinearForm.tensor2site (state/antilinear.py:68-98): out[l, d1, d2, r] =
// sum L[l, i] A[i, d1, k] B[k, d2, n] R[n, r].
template <typename T>
static int tensor2site(Ctx* ctx, cudaStream_t st, const T* L, int l, int i, const T* A, int d1,
                       int k, const T* B, int d2, int n, const T* R, int r, T* out) {
  T *la, *br;
  SM_CHECK(ctx->scratch("kt.la", (size_t)l * d1 * k, &la));
  SM_CHECK(ctx->scratch("kt.br", (size_t)k * d2 * r, &br));
  const T one = S<T>::one(), zero = S<T>::zero();
  SM_CHECK(gemm_ctx<T>(*ctx, st, SM_OP_N, SM_OP_N, l, d1 * k, i, one, L, i, A, d1 * k, zero, la,
                       d1 * k));
  SM_CHECK(gemm_ctx<T>(*ctx, st, SM_OP_N, SM_OP_N, k * d2, r, n, one, B, n, R, r, zero, br, r));
  return gemm_ctx<T>(*ctx, st, SM_OP_N, SM_OP_N, l * d1, d2 * r, k, one, la, k, br, d2 * r, zero,
                     out, d2 * r);
}

static std::atomic<int> g_svd_driver{0};  // 0 = gesdd, 1 = gesvd (the reference's default: gesdd)

}  // namespace sm

using namespace sm;

extern "C" {

int sm_abi_version(void) { return SM_ABI_VERSION; }

const char* sm_last_error(void) { return sm::last_error(); }

int sm_ctx_create(void** out, int device) {
  if (!out) return SM_ERR_VALUE;
  *out = nullptr;
  SM_CUDA_CHECK(cudaSetDevice(device));
  Ctx* c = new Ctx();
  c->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaHostAlloc(&c->pinned, 64 * 1024, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e != cudaSuccess) {
    set_error(std::string("context creation: ") + cudaGetErrorString(e));
    delete c;
    return SM_ERR_CUDA;
  }
  *out = c;
  return SM_OK;
}

int sm_ctx_destroy(void* ctx) {
  if (!ctx) return SM_OK;
  cudaDeviceSynchronize();
  delete as_ctx(ctx);
  return SM_OK;
}

int sm_ctx_set_precision(void* ctx, int precision) {
  SM_GUARD_CTX(ctx);
  if (precision != SM_PRECISION_FP64 && precision != SM_PRECISION_MIXED &&
      precision != SM_PRECISION_MIXED_LEARNED) {
    set_error("sm_ctx_set_precision: unknown precision mode");
    return SM_ERR_VALUE;
  }
  as_ctx(ctx)->precision = precision;
  return SM_OK;
}

int sm_split_rows_f32(void* ctx, int dtype, const void* A, int m, int n, int want_u,
                      double thr_rel, double thr_abs, void* rows, double* nrm, int kcap,
                      int* keff, int* sweeps, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (!A || !rows || !nrm || !keff || !sweeps || m < 1 || n < 1 || kcap < std::min(m, n) + 32) {
    set_error("sm_split_rows_f32: need m, n >= 1, kcap >= min(m, n) + 32 and non-null pointers");
    return SM_ERR_VALUE;
  }
  Ctx& c = *as_ctx(ctx);
  cudaStream_t st = as_stream(stream);
  const int kw = want_u ? n : m, l = want_u ? m : n;
  const bool fits = dtype == SM_FLOAT64 ? split_cluster_fits<double>(kw, l)
                                        : split_cluster_fits<cplx>(kw, l);
  if (!fits) {
    set_error("sm_split_rows_f32: matrix exceeds the cluster's capacity");
    return SM_ERR_VALUE;
  }
  JacobiCtl* ctl;
  double* info;
  float* vbuf;
  SM_CHECK(c.scratch("rows.ctl", 1, &ctl));
  SM_CHECK(c.scratch("rows.info", 8, &info));
  SM_CHECK(c.scratch("rows.vbuf", split_cluster_vbuf_floats(kw), &vbuf));
  SM_CUDA_CHECK(cudaMemsetAsync(ctl, 0, sizeof(JacobiCtl), st));
  if (dtype == SM_FLOAT64)
    SM_CHECK(split_cluster_f32<double>(st, (const double*)A, m, n, want_u != 0, thr_rel, thr_abs,
                                       60, (double*)rows, nrm, kcap, ctl, info, 0, vbuf));
  else
    SM_CHECK(split_cluster_f32<cplx>(st, (const cplx*)A, m, n, want_u != 0, thr_rel, thr_abs, 60,
                                     (cplx*)rows, nrm, kcap, ctl, info, 0, vbuf));
  JacobiCtl* h = reinterpret_cast<JacobiCtl*>(c.pinned);
  SM_CUDA_CHECK(cudaMemcpyAsync(h, ctl, sizeof(JacobiCtl), cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  *keff = h->nact;
  *sweeps = h->sweeps;
  if (h->status != 0) {
    set_error("sm_split_rows_f32: the FP32 Jacobi iteration did not converge");
    return SM_ERR_LINALG;
  }
  return SM_OK;
}

int sm_ctx_set_contraction_bits(void* ctx, int bits) {
  SM_GUARD_CTX(ctx);
  if (bits != 32 && bits != 64) {
    set_error("sm_ctx_set_contraction_bits: bits must be 32 or 64");
    return SM_ERR_VALUE;
  }
  as_ctx(ctx)->contract32 = bits == 32;
  return SM_OK;
}

int sm_truncate(void* ctx, const double* s_dev, int n, const sm_strategy* st, int* rank,
                double* err2, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_strategy(st));
  if (n < 1 || !s_dev || !rank || !err2) {
    set_error("sm_truncate: need n >= 1 and non-null pointers");
    return SM_ERR_VALUE;
  }
  return truncate_device(*as_ctx(ctx), as_stream(stream), s_dev, n, *st, rank, err2);
}

int sm_gemm(void* ctx, int dtype, int opA, int opB, int M, int N, int K, const void* A, int lda,
            const void* B, int ldb, void* C, int ldc, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (opA < 0 || opA > 2 || opB < 0 || opB > 2) {
    set_error("sm_gemm: invalid op flag");
    return SM_ERR_VALUE;
  }
  // through the context (split-K for small outputs, counted in the stats), on
  // the FP64 SIMT kernel in every precision mode
  if (dtype == SM_FLOAT64)
    return gemm_ctx_sel<double>(*as_ctx(ctx), as_stream(stream), opA, opB, M, N, K, 1.0,
                                (const double*)A, lda, (const double*)B, ldb, 0.0, (double*)C, ldc,
                                false);
  return gemm_ctx_sel<cplx>(*as_ctx(ctx), as_stream(stream), opA, opB, M, N, K, cplx{1.0, 0.0},
                            (const cplx*)A, lda, (const cplx*)B, ldb, cplx{0.0, 0.0}, (cplx*)C, ldc,
                            false);
}

int sm_gemm_ex(void* ctx, int dtype, int opA, int opB, int M, int N, int K, const double* alpha,
               const void* A, int lda, const void* B, int ldb, const double* beta, void* C, int ldc,
               void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (opA < 0 || opA > 2 || opB < 0 || opB > 2 || M < 0 || N < 0 || K < 0 || !alpha || !beta) {
    set_error("sm_gemm_ex: invalid op flag, size or scalar");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return gemm_ctx_sel<double>(*as_ctx(ctx), as_stream(stream), opA, opB, M, N, K, alpha[0],
                                (const double*)A, lda, (const double*)B, ldb, beta[0], (double*)C,
                                ldc, false);
  return gemm_ctx_sel<cplx>(*as_ctx(ctx), as_stream(stream), opA, opB, M, N, K,
                            cplx{alpha[0], alpha[1]}, (const cplx*)A, lda, (const cplx*)B, ldb,
                            cplx{beta[0], beta[1]}, (cplx*)C, ldc, false);
}

int sm_gemm_f64tc(void* ctx, int dtype, int opA, int opB, int M, int N, int K, const void* A,
                  int lda, const void* B, int ldb, void* C, int ldc, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (opA < 0 || opA > 2 || opB < 0 || opB > 2 || M < 0 || N < 0 || K < 0) {
    set_error("sm_gemm_f64tc: invalid op flag or size");
    return SM_ERR_VALUE;
  }
  Ctx& c = *as_ctx(ctx);
  cudaStream_t s = as_stream(stream);
  if (dtype == SM_FLOAT64 && M && N && K && gemm_oz_eligible(M, N, K)) {
    c.stats.gemm_oz_launches += 1;
    c.stats.gemm_oz_flops += 2.0 * M * N * K;
    SM_CHECK(gemm_oz(c, s, opA, opB, M, N, K, 1.0, (const double*)A, lda, (const double*)B, ldb,
                     0.0, (double*)C, ldc));
    return tc_status_check(c, s);
  }
  if (dtype == SM_COMPLEX128 && M && N && K && gemm_cplx_oz_eligible(M, N, K)) {
    c.stats.gemm_oz_launches += 3;
    c.stats.gemm_oz_flops += 6.0 * M * N * K;
    SM_CHECK(gemm_cplx_3m(c, s, opA, opB, M, N, K, cplx{1.0, 0.0}, (const cplx*)A, lda,
                          (const cplx*)B, ldb, cplx{0.0, 0.0}, (cplx*)C, ldc, true));
    return tc_status_check(c, s);
  }
  return sm_gemm(ctx, dtype, opA, opB, M, N, K, A, lda, B, ldb, C, ldc, stream);
}

int sm_two_site_matvec(void* ctx, int dtype, const int* dims, const void* L, const void* H,
                       const void* R, const void* v, void* out, int precision, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (!dims || !L || !H || !R || !v || !out || precision < SM_MATVEC_FP64 ||
      precision > SM_MATVEC_BF16) {
    set_error("two_site_matvec: null argument or unknown precision");
    return SM_ERR_VALUE;
  }
  for (int i = 0; i < 8; ++i)
    if (dims[i] <= 0) {
      set_error("two_site_matvec: non-positive dimension");
      return SM_ERR_VALUE;
    }
  Ctx& c = *as_ctx(ctx);
  cudaStream_t s = as_stream(stream);
  int rc;
  if (dtype == SM_FLOAT64)
    rc = two_site_matvec<double>(c, s, dims[0], dims[1], dims[2], dims[3], dims[4], dims[5],
                                 dims[6], dims[7], (const double*)L, (const double*)H,
                                 (const double*)R, (const double*)v, (double*)out, precision);
  else
    rc = two_site_matvec<cplx>(c, s, dims[0], dims[1], dims[2], dims[3], dims[4], dims[5], dims[6],
                               dims[7], (const cplx*)L, (const cplx*)H, (const cplx*)R,
                               (const cplx*)v, (cplx*)out, precision);
  SM_CHECK(rc);
  return precision == SM_MATVEC_FP64 ? SM_OK : tc_status_check(c, s);
}

int sm_two_site_prepare(void* ctx, const int* dims, const void* L, const void* R, int precision,
                        void* stream) {
  SM_GUARD_CTX(ctx);
  if (!dims || !L || !R) {
    set_error("two_site_prepare: null argument");
    return SM_ERR_VALUE;
  }
  for (int i = 0; i < 8; ++i)
    if (dims[i] <= 0) {
      set_error("two_site_prepare: non-positive dimension");
      return SM_ERR_VALUE;
    }
  Ctx& c = *as_ctx(ctx);
  return two_site_prepare(c, as_stream(stream), dims[0], dims[1], dims[2], dims[3], dims[4],
                          dims[5], dims[6], dims[7], (const double*)L, (const double*)R,
                          precision);
}

int sm_two_site_matvec_prepared(void* ctx, const void* H, const void* v, void* out,
                                void* stream) {
  SM_GUARD_CTX(ctx);
  if (!H || !v || !out) {
    set_error("two_site_matvec_prepared: null argument");
    return SM_ERR_VALUE;
  }
  Ctx& c = *as_ctx(ctx);
  cudaStream_t s = as_stream(stream);
  SM_CHECK(two_site_matvec_prepared(c, s, (const double*)H, (const double*)v, (double*)out));
  return tc_status_check(c, s);
}

int sm_ctx_set_rank_cap(void* ctx, double margin, int extra) {
  SM_GUARD_CTX(ctx);
  if (!(margin >= 1.0) || extra < 0) {
    set_error("sm_ctx_set_rank_cap: margin must be >= 1 and extra >= 0");
    return SM_ERR_VALUE;
  }
  as_ctx(ctx)->cap_margin = margin;
  as_ctx(ctx)->cap_extra = extra;
  return SM_OK;
}

int sm_range_finder(void* ctx, const double* A, int m, int n, int want_u, int k, int power_iters,
                    double* BH, void* stream) {
  SM_GUARD_CTX(ctx);
  if (!A || !BH || m < 1 || n < 1 || power_iters < 0 || power_iters > 8) {
    set_error("sm_range_finder: invalid argument");
    return SM_ERR_VALUE;
  }
  Ctx& c = *as_ctx(ctx);
  cudaStream_t s = as_stream(stream);
  int* status;
  SM_CHECK(c.scratch("rf.status", 1, &status));
  SM_CHECK(range_finder_bh(c, s, A, m, n, want_u != 0, k, power_iters, BH, status));
  int* h = reinterpret_cast<int*>(c.pinned);
  SM_CUDA_CHECK(cudaMemcpyAsync(h, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  SM_CUDA_CHECK(cudaStreamSynchronize(s));
  if (*h) {
    set_error("sm_range_finder: Cholesky pivot not positive");
    return SM_ERR_LINALG;
  }
  return SM_OK;
}

int sm_ctx_set_range_finder(void* ctx, int on, int oversample, int power_iters, int rank_hint) {
  SM_GUARD_CTX(ctx);
  if (oversample < 0 || power_iters < 0 || power_iters > 8 || rank_hint < 0) {
    set_error("sm_ctx_set_range_finder: oversample >= 0, 0 <= power_iters <= 8, rank_hint >= 0");
    return SM_ERR_VALUE;
  }
  Ctx* c = as_ctx(ctx);
  c->range_finder = on != 0;
  c->rf_oversample = oversample;
  c->rf_power = power_iters;
  c->rf_rank_hint = rank_hint;
  return SM_OK;
}

int sm_ctx_set_concurrent(void* ctx, int on) {
  SM_GUARD_CTX(ctx);
  as_ctx(ctx)->concurrent = on != 0;
  return SM_OK;
}

int sm_ctx_set_fp64_products(void* ctx, int tensor_cores) {
  SM_GUARD_CTX(ctx);
  as_ctx(ctx)->fp64_tc = tensor_cores != 0;
  return SM_OK;
}

int sm_gemm_f32(void* ctx, int dtype, int opA, int opB, int M, int N, int K, const void* A,
                int lda, const void* B, int ldb, void* C, int ldc, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (opA < 0 || opA > 2 || opB < 0 || opB > 2 || M < 0 || N < 0 || K < 0) {
    set_error("sm_gemm_f32: invalid op flag or size");
    return SM_ERR_VALUE;
  }
  Ctx& c = *as_ctx(ctx);
  cudaStream_t s = as_stream(stream);
  int rc;
  if (dtype == SM_FLOAT64)
    rc = gemm_ctx_f32<double>(c, s, opA, opB, M, N, K, 1.0, (const double*)A, lda,
                              (const double*)B, ldb, 0.0, (double*)C, ldc);
  else
    rc = gemm_ctx_f32<cplx>(c, s, opA, opB, M, N, K, cplx{1.0, 0.0}, (const cplx*)A, lda,
                            (const cplx*)B, ldb, cplx{0.0, 0.0}, (cplx*)C, ldc);
  SM_CHECK(rc);
  return tc_status_check(c, s);
}

int sm_svd(void* ctx, int dtype, const void* A, int m, int n, void* U, double* s, void* Vt,
           void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  sm_strategy st{};
  st.method = SM_DO_NOT_TRUNCATE;
  st.max_bond_dimension = 0x7fffffff;
  SplitResult r;
  if (dtype == SM_FLOAT64)
    return svd_split<double>(*as_ctx(ctx), as_stream(stream), (const double*)A, m, n, st, OUT_U,
                             (double*)U, OUT_VT, (double*)Vt, s, &r);
  return svd_split<cplx>(*as_ctx(ctx), as_stream(stream), (const cplx*)A, m, n, st, OUT_U, (cplx*)U,
                         OUT_VT, (cplx*)Vt, s, &r);
}

int sm_left_orth_2site(void* ctx, int dtype, const void* AA, int a, int d1, int d2, int b,
                       const sm_strategy* st, void* U, void* SV, int* D, double* err,
                       void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  SM_CHECK(check_strategy(st));
  if (dtype == SM_FLOAT64)
    return split2<double>(as_ctx(ctx), as_stream(stream), AA, a, d1, d2, b, st, OUT_U, U, OUT_SVT,
                          SV, D, err);
  return split2<cplx>(as_ctx(ctx), as_stream(stream), AA, a, d1, d2, b, st, OUT_U, U, OUT_SVT, SV,
                      D, err);
}

int sm_right_orth_2site(void* ctx, int dtype, const void* AA, int a, int d1, int d2, int b,
                        const sm_strategy* st, void* US, void* V, int* D, double* err,
                        void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  SM_CHECK(check_strategy(st));
  if (dtype == SM_FLOAT64)
    return split2<double>(as_ctx(ctx), as_stream(stream), AA, a, d1, d2, b, st, OUT_US, US, OUT_VT,
                          V, D, err);
  return split2<cplx>(as_ctx(ctx), as_stream(stream), AA, a, d1, d2, b, st, OUT_US, US, OUT_VT, V,
                      D, err);
}

int sm_update_left_environment(void* ctx, int dtype, const void* B, int l, int j, int n,
                               const void* A, int i, int k, const void* rho, void* out,
                               void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (l <= 0 || j <= 0 || n <= 0 || i <= 0 || k <= 0) {
    set_error("Invalid arguments to _update_left_environment");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return env_left<double>(as_ctx(ctx), as_stream(stream), B, l, j, n, A, i, k, rho, out);
  return env_left<cplx>(as_ctx(ctx), as_stream(stream), B, l, j, n, A, i, k, rho, out);
}

int sm_update_right_environment(void* ctx, int dtype, const void* B, int l, int j, int n,
                                const void* A, int i, int k, const void* rho, void* out,
                                void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (l <= 0 || j <= 0 || n <= 0 || i <= 0 || k <= 0) {
    set_error("Invalid arguments to _update_right_environment");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return env_right<double>(as_ctx(ctx), as_stream(stream), B, l, j, n, A, i, k, rho, out);
  return env_right<cplx>(as_ctx(ctx), as_stream(stream), B, l, j, n, A, i, k, rho, out);
}

int sm_mpo_multiply_tensor(void* ctx, int dtype, const void* O, int a, int i, int j, int b,
                           const void* B, int c, int d, void* C, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (a <= 0 || i <= 0 || j <= 0 || b <= 0 || c <= 0 || d <= 0) {
    set_error("Invalid arguments to _mpo_multiply_tensor");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return mpo_multiply_tensor<double>(as_stream(stream), (const double*)O, a, i, j, b,
                                       (const double*)B, c, d, (double*)C);
  return mpo_multiply_tensor<cplx>(as_stream(stream), (const cplx*)O, a, i, j, b, (const cplx*)B, c,
                                   d, (cplx*)C);
}

static int check_mpo_env(int a, int j, int d, int c, int i, int e, int b, int f,
                         const void* rho, const void* A, const void* O, const void* B,
                         const void* out) {
  if (a <= 0 || j <= 0 || d <= 0 || c <= 0 || i <= 0 || e <= 0 || b <= 0 || f <= 0 || !rho || !A ||
      !O || !B || !out) {
    set_error("Invalid arguments to an MPO environment update");
    return SM_ERR_VALUE;
  }
  return SM_OK;
}

int sm_update_left_mpo_environment(void* ctx, int dtype, const void* rho, const void* A, int a,
                                   int j, int d, const void* O, int c, int i, int e, const void* B,
                                   int b, int f, void* out, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  SM_CHECK(check_mpo_env(a, j, d, c, i, e, b, f, rho, A, O, B, out));
  if (dtype == SM_FLOAT64)
    return mpo_env_left<double>(*as_ctx(ctx), as_stream(stream), (const double*)rho,
                                (const double*)A, a, j, d, (const double*)O, c, i, e,
                                (const double*)B, b, f, (double*)out);
  return mpo_env_left<cplx>(*as_ctx(ctx), as_stream(stream), (const cplx*)rho, (const cplx*)A, a,
                            j, d, (const cplx*)O, c, i, e, (const cplx*)B, b, f, (cplx*)out);
}

int sm_update_right_mpo_environment(void* ctx, int dtype, const void* rho, const void* A, int a,
                                    int j, int d, const void* O, int c, int i, int e,
                                    const void* B, int b, int f, void* out, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  SM_CHECK(check_mpo_env(a, j, d, c, i, e, b, f, rho, A, O, B, out));
  if (dtype == SM_FLOAT64)
    return mpo_env_right<double>(*as_ctx(ctx), as_stream(stream), (const double*)rho,
                                 (const double*)A, a, j, d, (const double*)O, c, i, e,
                                 (const double*)B, b, f, (double*)out);
  return mpo_env_right<cplx>(*as_ctx(ctx), as_stream(stream), (const cplx*)rho, (const cplx*)A, a,
                             j, d, (const cplx*)O, c, i, e, (const cplx*)B, b, f, (cplx*)out);
}

int sm_mpo_join(void* ctx, int dtype, const void* B, int a, int i, int j, int b, const void* A,
                int c, int k, int d, void* C, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (a <= 0 || i <= 0 || j <= 0 || b <= 0 || c <= 0 || k <= 0 || d <= 0 || !A || !B || !C) {
    set_error("Invalid arguments to MPOList.join");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return mpo_join<double>(as_stream(stream), (const double*)B, a, i, j, b, (const double*)A, c, k,
                            d, (double*)C);
  return mpo_join<cplx>(as_stream(stream), (const cplx*)B, a, i, j, b, (const cplx*)A, c, k, d,
                        (cplx*)C);
}

int sm_scprod(void* ctx, int dtype, int L, const int* phys, const int* bra_bonds,
              const void* const* bra, const int* ket_bonds, const void* const* ket, double* out,
              void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (L < 1) {
    set_error("Invalid arguments to scprod");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return scprod_impl<double>(*as_ctx(ctx), as_stream(stream), L, phys, bra_bonds, bra, ket_bonds,
                               ket, out);
  return scprod_impl<cplx>(*as_ctx(ctx), as_stream(stream), L, phys, bra_bonds, bra, ket_bonds, ket,
                           out);
}

int sm_canonicalize(void* ctx, int dtype, int L, const int* phys, int* bonds, void* const* sites,
                    const int64_t* cap, int center, const sm_strategy* st, double* err,
                    void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  SM_CHECK(check_strategy(st));
  if (L < 1 || center < 0 || center >= L) {
    set_error("canonicalize: center out of range");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return canonicalize_impl<double>(*as_ctx(ctx), as_stream(stream), L, phys, bonds, sites, cap,
                                     center, *st, err);
  return canonicalize_impl<cplx>(*as_ctx(ctx), as_stream(stream), L, phys, bonds, sites, cap,
                                 center, *st, err);
}

int sm_recanonicalize(void* ctx, int dtype, int L, const int* phys, int* bonds, void* const* sites,
                      const int64_t* cap, int oldcenter, int newcenter, const sm_strategy* st,
                      double* err, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  SM_CHECK(check_strategy(st));
  if (L < 1 || oldcenter < 0 || oldcenter >= L || newcenter < 0 || newcenter >= L || !err) {
    set_error("recanonicalize: center out of range");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return recanonicalize_impl<double>(*as_ctx(ctx), as_stream(stream), L, phys, bonds, sites, cap,
                                       oldcenter, newcenter, *st, err);
  return recanonicalize_impl<cplx>(*as_ctx(ctx), as_stream(stream), L, phys, bonds, sites, cap,
                                   oldcenter, newcenter, *st, err);
}

int sm_update_in_canonical_form_right(void* ctx, int dtype, const void* A, int a, int i, int b,
                                      const void* next, int j, int c, const sm_strategy* st,
                                      void* U, void* next_out, int* D, double* err,
                                      void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  SM_CHECK(check_strategy(st));
  if (a <= 0 || i <= 0 || b <= 0 || j <= 0 || c <= 0 || !A || !next || !U || !next_out || !D ||
      !err) {
    set_error("Invalid arguments to _update_in_canonical_form_right");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return canon_update_right<double>(as_ctx(ctx), as_stream(stream), (const double*)A, a, i, b,
                                      (const double*)next, j, c, *st, (double*)U,
                                      (double*)next_out, D, err);
  return canon_update_right<cplx>(as_ctx(ctx), as_stream(stream), (const cplx*)A, a, i, b,
                                  (const cplx*)next, j, c, *st, (cplx*)U, (cplx*)next_out, D, err);
}

int sm_update_in_canonical_form_left(void* ctx, int dtype, const void* A, int a, int i, int b,
                                     const void* prev, int p, int j, const sm_strategy* st, void* V,
                                     void* prev_out, int* D, double* err, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  SM_CHECK(check_strategy(st));
  if (a <= 0 || i <= 0 || b <= 0 || p <= 0 || j <= 0 || !A || !prev || !V || !prev_out || !D ||
      !err) {
    set_error("Invalid arguments to _update_in_canonical_form_left");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return canon_update_left<double>(as_ctx(ctx), as_stream(stream), (const double*)A, a, i, b,
                                     (const double*)prev, p, j, *st, (double*)V,
                                     (double*)prev_out, D, err);
  return canon_update_left<cplx>(as_ctx(ctx), as_stream(stream), (const cplx*)A, a, i, b,
                                 (const cplx*)prev, p, j, *st, (cplx*)V, (cplx*)prev_out, D, err);
}

int sm_contract_nrjl_ijk_klm(void* ctx, int dtype, const void* U, int nr, const void* A, int a,
                             int d, int b, const void* B, int e, int c, void* out, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (a <= 0 || d <= 0 || b <= 0 || e <= 0 || c <= 0 || nr != d * e || !U || !A || !B || !out) {
    set_error("Invalid arguments to _contract_nrjl_ijk_klm");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return contract_nrjl<double>(as_ctx(ctx), as_stream(stream), (const double*)U, nr,
                                 (const double*)A, a, d, b, (const double*)B, e, c, (double*)out);
  return contract_nrjl<cplx>(as_ctx(ctx), as_stream(stream), (const cplx*)U, nr, (const cplx*)A, a,
                             d, b, (const cplx*)B, e, c, (cplx*)out);
}

int sm_tensor2site(void* ctx, int dtype, const void* L, int l, int i, const void* A, int d1, int k,
                   const void* B, int d2, int n, const void* R, int r, void* out, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (l <= 0 || i <= 0 || d1 <= 0 || k <= 0 || d2 <= 0 || n <= 0 || r <= 0 || !L || !A || !B ||
      !R || !out) {
    set_error("Invalid arguments to tensor2site");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return tensor2site<double>(as_ctx(ctx), as_stream(stream), (const double*)L, l, i,
                               (const double*)A, d1, k, (const double*)B, d2, n, (const double*)R, r,
                               (double*)out);
  return tensor2site<cplx>(as_ctx(ctx), as_stream(stream), (const cplx*)L, l, i, (const cplx*)A, d1,
                           k, (const cplx*)B, d2, n, (const cplx*)R, r, (cplx*)out);
}

int sm_select_svd_driver(const char* name) {
  const std::string s = name ? name : "";
  if (s == "gesdd") {
    g_svd_driver = 0;
    return SM_OK;
  }
  if (s == "gesvd") {
    g_svd_driver = 1;
    return SM_OK;
  }
  set_error("Invalid LAPACK SVD driver name: " + s);
  return SM_ERR_VALUE;
}

int sm_svd_driver(void) { return g_svd_driver.load(); }

static int simplify_entry(void* ctx, int dtype, int L, const int* phys, int nterms,
                          const double* weights, const int* ket_bonds, const void* const* ket_sites,
                          const double* term_errors, const sm_strategy* st, int direction,
                          void* const* out_sites, const int64_t* out_cap, int* out_bonds,
                          sm_simplify_report* rep, const double* gram, const int* guess_bonds,
                          const void* const* guess_sites, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  SM_CHECK(check_strategy(st));
  if (L < 1 || nterms < 1 || !rep || !weights || !ket_bonds || !ket_sites) {
    set_error("simplify: need L >= 1, nterms >= 1 and non-null arguments");
    return SM_ERR_VALUE;
  }
  for (int t = 0; t < nterms; ++t) {
    const int* kb = ket_bonds + (size_t)t * (L + 1);
    for (int i = 0; i < L; ++i)
      if (kb[i] <= 0 || phys[i] <= 0) {
        set_error("simplify: non-positive dimension");
        return SM_ERR_VALUE;
      }
    if (kb[0] != 1 || kb[L] != 1) {
      set_error("simplify: open boundary bonds must be 1");
      return SM_ERR_VALUE;
    }
  }
  if (dtype == SM_FLOAT64)
    return simplify_impl<double>(*as_ctx(ctx), as_stream(stream), L, phys, nterms, weights,
                                 term_errors, ket_bonds, ket_sites, *st, direction, out_sites,
                                 out_cap, out_bonds, rep, gram, guess_bonds, guess_sites);
  return simplify_impl<cplx>(*as_ctx(ctx), as_stream(stream), L, phys, nterms, weights,
                             term_errors, ket_bonds, ket_sites, *st, direction, out_sites, out_cap,
                             out_bonds, rep, gram, guess_bonds, guess_sites);
}

int sm_simplify(void* ctx, int dtype, int L, const int* phys, int nterms, const double* weights,
                const int* ket_bonds, const void* const* ket_sites, const double* term_errors,
                const sm_strategy* st, int direction, void* const* out_sites,
                const int64_t* out_cap, int* out_bonds, sm_simplify_report* rep, void* stream) {
  return simplify_entry(ctx, dtype, L, phys, nterms, weights, ket_bonds, ket_sites, term_errors, st,
                        direction, out_sites, out_cap, out_bonds, rep, nullptr, nullptr, nullptr,
                        stream);
}

int sm_simplify_guess(void* ctx, int dtype, int L, const int* phys, int nterms,
                      const double* weights, const int* ket_bonds, const void* const* ket_sites,
                      const double* term_errors, const double* gram, const int* guess_bonds,
                      const void* const* guess_sites, const sm_strategy* st, int direction,
                      void* const* out_sites, const int64_t* out_cap, int* out_bonds,
                      sm_simplify_report* rep, void* stream) {
  if (!guess_bonds || !guess_sites) {
    set_error("simplify_guess: the guess must not be null");
    return SM_ERR_VALUE;
  }
  return simplify_entry(ctx, dtype, L, phys, nterms, weights, ket_bonds, ket_sites, term_errors, st,
                        direction, out_sites, out_cap, out_bonds, rep, gram, guess_bonds,
                        guess_sites, stream);
}

int sm_simplify_gram(void* ctx, int dtype, int L, const int* phys, int nterms,
                     const double* weights, const int* ket_bonds, const void* const* ket_sites,
                     const double* term_errors, const double* gram, const sm_strategy* st,
                     int direction, void* const* out_sites, const int64_t* out_cap, int* out_bonds,
                     sm_simplify_report* rep, void* stream) {
  if (!gram) {
    set_error("simplify_gram: gram must not be null");
    return SM_ERR_VALUE;
  }
  return simplify_entry(ctx, dtype, L, phys, nterms, weights, ket_bonds, ket_sites, term_errors, st,
                        direction, out_sites, out_cap, out_bonds, rep, gram, nullptr, nullptr,
                        stream);
}

int sm_mpo_scprod(void* ctx, int dtype, int L, const int* dout, const int* din,
                  const int* mpo_bonds, const void* const* mpo, const int* bra_bonds,
                  const void* const* bra, const int* ket_bonds, const void* const* ket,
                  double* out, void* stream) {
  SM_GUARD_CTX(ctx);
  SM_CHECK(check_dtype(dtype));
  if (L < 1 || !dout || !din || !mpo_bonds || !mpo || !bra_bonds || !bra || !ket_bonds || !ket ||
      !out) {
    set_error("mpo_scprod: need L >= 1 and non-null arguments");
    return SM_ERR_VALUE;
  }
  for (int i = 0; i <= L; ++i)
    if (mpo_bonds[i] <= 0 || bra_bonds[i] <= 0 || ket_bonds[i] <= 0 ||
        (i < L && (dout[i] <= 0 || din[i] <= 0))) {
      set_error("mpo_scprod: non-positive dimension");
      return SM_ERR_VALUE;
    }
  if (mpo_bonds[0] != 1 || mpo_bonds[L] != 1 || bra_bonds[0] != 1 || bra_bonds[L] != 1 ||
      ket_bonds[0] != 1 || ket_bonds[L] != 1) {
    set_error("mpo_scprod: open boundary bonds must be 1");
    return SM_ERR_VALUE;
  }
  if (dtype == SM_FLOAT64)
    return mpo_scprod_impl<double>(*as_ctx(ctx), as_stream(stream), L, dout, din, mpo_bonds, mpo,
                                   bra_bonds, bra, ket_bonds, ket, out);
  return mpo_scprod_impl<cplx>(*as_ctx(ctx), as_stream(stream), L, dout, din, mpo_bonds, mpo,
                               bra_bonds, bra, ket_bonds, ket, out);
}

int sm_simplify_bond_caps(int L, const int* phys, int nterms, const int* ket_bonds,
                          const sm_strategy* st, int* cap_bonds) {
  SM_CHECK(check_strategy(st));
  if (L < 1 || nterms < 1) {
    set_error("bond caps: need L >= 1 and nterms >= 1");
    return SM_ERR_VALUE;
  }
  (void)phys;
  for (int i = 0; i <= L; ++i) {
    long long K = 0;
    for (int t = 0; t < nterms; ++t) K += ket_bonds[(size_t)t * (L + 1) + i];
    if (nterms > 1 && (i == 0 || i == L)) K = 1;
    long long c = std::min<long long>(K, st->max_bond_dimension);
    if (i == 0 || i == L) c = K;
    cap_bonds[i] = (int)std::max<long long>(1, c);
  }
  return SM_OK;
}

int sm_trace_enable(void* ctx, int on) {
  SM_GUARD_CTX(ctx);
  Ctx* c = as_ctx(ctx);
  c->trace = on != 0;
  c->tr_rank.clear();
  c->tr_len.clear();
  c->tr_err2.clear();
  c->tr_s.clear();
  return SM_OK;
}

int sm_trace_read(void* ctx, int* count, int64_t* total_s, int* ranks, int* lens, double* err2,
                  double* svals) {
  SM_GUARD_CTX(ctx);
  Ctx* c = as_ctx(ctx);
  if (count) *count = (int)c->tr_rank.size();
  if (total_s) *total_s = (int64_t)c->tr_s.size();
  if (ranks) std::copy(c->tr_rank.begin(), c->tr_rank.end(), ranks);
  if (lens) std::copy(c->tr_len.begin(), c->tr_len.end(), lens);
  if (err2) std::copy(c->tr_err2.begin(), c->tr_err2.end(), err2);
  if (svals) std::copy(c->tr_s.begin(), c->tr_s.end(), svals);
  return SM_OK;
}

int sm_stats_reset(void* ctx, int timing) {
  SM_GUARD_CTX(ctx);
  Ctx* c = as_ctx(ctx);
  c->stats = sm_stats{};
  c->stats.launches = -launches_total();  // read back as a difference
  c->timing = timing != 0;
  return SM_OK;
}

int sm_stats_read(void* ctx, sm_stats* out) {
  SM_GUARD_CTX(ctx);
  if (!out) return SM_ERR_VALUE;
  *out = as_ctx(ctx)->stats;
  out->launches += launches_total();
  return SM_OK;
}

}  // extern "C"
