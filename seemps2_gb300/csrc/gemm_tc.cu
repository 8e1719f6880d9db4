// Tensor-core GEMM for FP64 operands at FP32 accuracy: 3xTF32 on tcgen05.
//
//   C[M,N] = alpha * op(A)[M,K] * op(B)[K,N] + beta * C      (real, row-major)
//
// The mixed precision forms run the sweep contractions (cython/gemm.pxi:21-122
// in the reference, FP64 there) at FP32 accuracy.  GB300's CUDA cores give
// FP32 at 64x the FP64 rate, its tensor cores TF32 at another ~15x; TF32 keeps
// 11 significant bits, so each operand is split x = hi + lo (hi = x rounded to
// TF32, lo = the FP32 rest) and the product is hi*hi + hi*lo + lo*hi
// accumulated in FP32 in tensor memory: the error of an FP32 GEMM.
//
// Data path per 128 x 128 output tile (one CTA of 128 threads, K split over
// blockIdx.z when the output has few tiles):
//   * a split kernel writes hi / lo of op(A) as M x Kp and of op(B)^T as
//     N x Kp FP32 arrays (K contiguous, Kp = K rounded up to 32, zero pad);
//   * warp 0 / lane 0 streams 32-wide K slices of the four arrays with TMA
//     (cp.async.bulk.tensor, 128-byte swizzle) into a 3-stage ring;
//   * warp 1 / lane 0 issues tcgen05.mma kind::tf32 (M=128, N=128, K=8; three
//     per K step) accumulating in 128 TMEM columns, and tcgen05.commit frees
//     each stage;
//   * all four warps read the accumulator back with tcgen05.ld (warp w owns
//     TMEM lanes 32w..32w+31 = tile rows) and write FP64 results.
// Every mbarrier wait is bounded (globaltimer): on timeout the CTA records an
// error bit, waits (bounded) for its own copies in flight, frees its TMEM and
// returns; the sweep reads the status word at its end.
#include <algorithm>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "kernels.cuh"

namespace sm {

namespace {

constexpr int TM = 128, TN = 128, TS = 3;
constexpr int kTCThreads = 128;
// Per mode: 3xTF32 (FP32 planes hi and lo of both operands, 32-wide K slabs,
// three tf32 MMAs of K = 8 per 8 of K) or BF16 (one BF16 plane per operand,
// 64-wide K slabs, one f16-kind MMA of K = 16 per 16 of K).  Either way a
// slab row is 128 bytes, the span of the 128-byte swizzle.
template <bool BF16>
struct TcMode {
  static constexpr int TK = BF16 ? 64 : 32;          // K elements per slab
  static constexpr int KMMA = BF16 ? 16 : 8;         // K per MMA instruction
  static constexpr int planes = BF16 ? 1 : 2;        // planes per operand
  static constexpr uint32_t tileA = TM * 128;        // bytes of one plane's slab
  static constexpr uint32_t tileB = TN * 128;
  static constexpr uint32_t stage = planes * (tileA + tileB);
  static constexpr size_t smem = (size_t)TS * stage + 1024 + 256;
  // instruction descriptor: D = F32 (bits 4-5 = 1), A and B TF32 (2) or BF16
  // (1) at bits 7-9 and 10-12, both K-major (bits 15, 16 = 0), N >> 3 at bits
  // 17-22, M >> 4 at bits 24-28
  static constexpr uint32_t fmt = BF16 ? 1u : 2u;
  static constexpr uint32_t idesc = (1u << 4) | (fmt << 7) | (fmt << 10) |
                                    ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
};
constexpr unsigned long long kWaitNs = 1000000000ull;  // 1 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the phase of the given parity; false after `ns` nanoseconds.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, unsigned long long ns) {
  if (mbar_try_wait(b, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (!mbar_try_wait(b, parity))
    if (gtimer() - t0 > ns) return false;
  return true;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x,
                                            int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
      "%4}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// K-major operand in the 128-byte swizzled layout TMA writes: rows of 128 B,
// 8-row atoms of 1024 B (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;              // leading byte offset (unused for this layout)
  d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;              // descriptor version
  d |= (uint64_t)2 << 61;              // 128-byte swizzle
  return d;
}
__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(TcMode<false>::idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(TcMode<true>::idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <bool BF16, typename OutT>
__global__ void __launch_bounds__(kTCThreads, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
              const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl,
              int M, int N, int ktiles, int kt_per, double alpha, double beta,
              OutT* __restrict__ C, int ldc, OutT* __restrict__ part,
              unsigned int* __restrict__ status) {
  using Md = TcMode<BF16>;
  constexpr uint32_t kStage = Md::stage, kTileA = Md::tileA, kTileB = Md::tileB;
  constexpr int TK = Md::TK;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + (size_t)TS * kStage);
  uint64_t* empty = full + TS;
  uint64_t* done = empty + TS;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const int kt0 = blockIdx.z * kt_per;
  const int nk = min(ktiles, kt0 + kt_per) - kt0;  // >= 1 (host)
  if (threadIdx.x == 0) {
    for (int s = 0; s < TS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"((uint32_t)TN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer: TMA ring
    int issued[TS] = {};
    for (int i = 0; i < nk; ++i) {
      const int s = i % TS;
      const uint32_t ph = (uint32_t)(i / TS) & 1u;
      if (i >= TS && !mbar_wait(&empty[s], ph ^ 1u, kWaitNs)) {
        atomicOr(status, 1u);
        break;
      }
      unsigned char* stg = base + (size_t)s * kStage;
      mbar_expect_tx(&full[s], kStage);
      const int x = (kt0 + i) * TK;
      if constexpr (BF16) {
        tma_load_2d(stg, &mAh, &full[s], x, m0);
        tma_load_2d(stg + kTileA, &mBh, &full[s], x, n0);
      } else {
        tma_load_2d(stg, &mAh, &full[s], x, m0);
        tma_load_2d(stg + kTileA, &mAl, &full[s], x, m0);
        tma_load_2d(stg + 2 * kTileA, &mBh, &full[s], x, n0);
        tma_load_2d(stg + 2 * kTileA + kTileB, &mBl, &full[s], x, n0);
      }
      issued[s] += 1;
    }
    // no copy of this CTA may still be landing when it exits
    for (int s = 0; s < TS; ++s)
      if (issued[s] && !mbar_wait(&full[s], (uint32_t)(issued[s] - 1) & 1u, kWaitNs))
        atomicOr(status, 4u);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    for (int i = 0; i < nk; ++i) {
      const int s = i % TS;
      const uint32_t ph = (uint32_t)(i / TS) & 1u;
      if (!mbar_wait(&full[s], ph, kWaitNs)) {
        atomicOr(status, 2u);
        break;
      }
      tc_fence_after();
      const uint32_t ah = smem_u32(base + (size_t)s * kStage);
      if constexpr (BF16) {
        const uint32_t bh = ah + kTileA;
#pragma unroll
        for (int kk = 0; kk < TK / Md::KMMA; ++kk) {
          const uint32_t off = kk * 32;  // 16 BF16 values
          umma_bf16(tmem, sdesc_sw128(ah + off), sdesc_sw128(bh + off),
                    (i > 0 || kk > 0) ? 1u : 0u);
        }
      } else {
        const uint32_t al = ah + kTileA, bh = ah + 2 * kTileA, bl = bh + kTileB;
#pragma unroll
        for (int kk = 0; kk < TK / Md::KMMA; ++kk) {
          const uint32_t off = kk * 32;  // 8 TF32 values
          const uint64_t dah = sdesc_sw128(ah + off), dal = sdesc_sw128(al + off);
          const uint64_t dbh = sdesc_sw128(bh + off), dbl = sdesc_sw128(bl + off);
          umma_tf32(tmem, dah, dbh, (i > 0 || kk > 0) ? 1u : 0u);
          umma_tf32(tmem, dah, dbl, 1u);
          umma_tf32(tmem, dal, dbh, 1u);
        }
      }
      umma_commit(&empty[s]);
    }
    umma_commit(done);  // arrives once every MMA issued above has completed
  }
  __syncwarp();
  // epilogue: the done wait outlasts the producer's and the issuer's bounds
  const bool ok = mbar_wait(done, 0u, 4 * kWaitNs);
  __syncwarp();
  tc_fence_after();
  if (ok) {
    const int row = m0 + warp * 32 + lane;
    for (int c = 0; c < TN; c += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
      if (row < M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = n0 + c + j;
          if (col < N) {
            if (part) {
              part[((size_t)blockIdx.z * M + row) * N + col] = (OutT)v[j];
            } else {
              OutT* p = C + (size_t)row * ldc + col;
              *p = beta == 0.0 ? (OutT)(alpha * (double)v[j])
                               : (OutT)fma(alpha, (double)v[j], beta * (double)*p);
            }
          }
        }
      }
    }
  } else if (threadIdx.x == 0) {
    atomicOr(status, 8u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)TN)
                 : "memory");
  }
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// hi / lo FP32 parts of op(X) as a rows x kp K-contiguous array: element
// (r, k) is X[r * ldx + k] (trans = 0) or X[k * ldx + r] (trans = 1), zero for
// k >= K.  32 x 32 tiles through shared memory so both sides stay coalesced.
__global__ void k_split_tf32(const double* __restrict__ X, int ldx, int rows, int K, int kp,
                             int trans, float* __restrict__ hi, float* __restrict__ lo) {
  __shared__ double tile[32][33];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int j = ty; j < 32; j += 8) {
    double v = 0.0;
    if (trans) {  // read along r: tile[k][r]
      const int k = k0 + j, r = r0 + tx;
      if (k < K && r < rows) v = X[(size_t)k * ldx + r];
      tile[j][tx] = v;
    } else {  // read along k: tile[r][k]
      const int r = r0 + j, k = k0 + tx;
      if (k < K && r < rows) v = X[(size_t)r * ldx + k];
      tile[j][tx] = v;
    }
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int r = r0 + j, k = k0 + tx;
    if (r < rows && k < kp) {
      const double v = trans ? tile[tx][j] : tile[j][tx];
      const float h = tf32_rna((float)v);
      hi[(size_t)r * kp + k] = h;
      lo[(size_t)r * kp + k] = (float)(v - (double)h);
    }
  }
}

// op(X) rounded to BF16 as a rows x kp K-contiguous array (same tiling and
// element rule as k_split_tf32).
__global__ void k_split_bf16(const double* __restrict__ X, int ldx, int rows, int K, int kp,
                             int trans, __nv_bfloat16* __restrict__ out) {
  __shared__ double tile[32][33];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int j = ty; j < 32; j += 8) {
    double v = 0.0;
    if (trans) {
      const int k = k0 + j, r = r0 + tx;
      if (k < K && r < rows) v = X[(size_t)k * ldx + r];
    } else {
      const int r = r0 + j, k = k0 + tx;
      if (k < K && r < rows) v = X[(size_t)r * ldx + k];
    }
    tile[j][tx] = v;
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int r = r0 + j, k = k0 + tx;
    if (r < rows && k < kp)
      out[(size_t)r * kp + k] = __float2bfloat16_rn((float)(trans ? tile[tx][j] : tile[j][tx]));
  }
}

template <typename OutT>
__global__ void k_tc_reduce(int M, int N, int nz, const OutT* __restrict__ part, double alpha,
                            double beta, OutT* __restrict__ C, int ldc) {
  const size_t mn = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < mn;
       e += (size_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int z = 0; z < nz; ++z) acc += (double)part[(size_t)z * mn + e];
    OutT* p = C + (e / N) * ldc + (e % N);
    *p = beta == 0.0 ? (OutT)(alpha * acc) : (OutT)fma(alpha, acc, beta * (double)*p);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  // looked up once (thread-safe static initialisation); null when unavailable
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
    return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
  }();
  return fn;
}

// 2-D map over a rows x kp K-contiguous plane (FP32 or BF16), box = one
// 128-byte slab row of box_rows rows, 128-byte swizzle.
int make_map(CUtensorMap* map, const void* base, bool bf16, int rows, int kp, int box_rows) {
  auto enc = encode_fn();
  if (!enc) {
    set_error("tensor-core GEMM: cuTensorMapEncodeTiled not available");
    return SM_ERR_CUDA;
  }
  const size_t es = bf16 ? 2 : 4;
  const cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kp * es};
  const cuuint32_t box[2] = {(cuuint32_t)(128 / es), (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                         2, const_cast<void*>(base), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("tensor-core GEMM: tensor map encoding failed");
    return SM_ERR_CUDA;
  }
  return SM_OK;
}

}  // namespace

bool gemm_tc_eligible(int M, int N, int K) {
  // below a few tiles of work the SIMT FP32 kernel is as fast and has no
  // split step
  return (double)M * N * K >= 4.0 * 1024 * 1024 && M >= 64 && N >= 64 && K >= 32 &&
         encode_fn() != nullptr;
}

int tc_kslab(bool bf16) { return bf16 ? TcMode<true>::TK : TcMode<false>::TK; }

int tc_planes(Ctx& ctx, cudaStream_t st, const double* X, int ldx, int rows, int K, int kp,
              int trans, bool bf16, void* hi, float* lo) {
  const dim3 sblk(32, 8), grd(kp / 32, (rows + 31) / 32);
  if (bf16)
    k_split_bf16<<<grd, sblk, 0, st>>>(X, ldx, rows, K, kp, trans,
                                       reinterpret_cast<__nv_bfloat16*>(hi));
  else
    k_split_tf32<<<grd, sblk, 0, st>>>(X, ldx, rows, K, kp, trans, reinterpret_cast<float*>(hi),
                                       lo);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  return SM_OK;
}

template <typename OutT>
int gemm_tc_planes(Ctx& ctx, cudaStream_t st, int M, int N, int kp, bool bf16, const void* ah,
                   const float* al, const void* bh, const float* bl, double alpha, double beta,
                   OutT* C, int ldc) {
  const int TK = tc_kslab(bf16);
  const int ktiles = kp / TK;
  unsigned int* status;
  SM_CHECK(tc_status(ctx, &status));
  CUtensorMap mAh, mAl, mBh, mBl;
  SM_CHECK(make_map(&mAh, ah, bf16, M, kp, TM));
  SM_CHECK(make_map(&mBh, bh, bf16, N, kp, TN));
  if (bf16) {
    mAl = mAh;
    mBl = mBh;
  } else {
    SM_CHECK(make_map(&mAl, al, false, M, kp, TM));
    SM_CHECK(make_map(&mBl, bl, false, N, kp, TN));
  }
  const int tiles = ((M + TM - 1) / TM) * ((N + TN - 1) / TN);
  int nz = std::max(1, std::min(std::max(1, ctx.num_sms) / tiles, ktiles / 2));
  const int kt_per = (ktiles + nz - 1) / nz;
  nz = (ktiles + kt_per - 1) / kt_per;
  OutT* part = nullptr;
  if (nz > 1)
    SM_CHECK(ctx.scratch(sizeof(OutT) == 8 ? "tc.part" : "tc.part32", (size_t)nz * M * N, &part));
  const dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM, nz);
  if (bf16) {
    SM_CHECK(raise_smem_limit(k_gemm_tc<true, OutT>, TcMode<true>::smem));
    k_gemm_tc<true, OutT><<<grid, kTCThreads, TcMode<true>::smem, st>>>(
        mAh, mAl, mBh, mBl, M, N, ktiles, kt_per, alpha, beta, C, ldc, part, status);
  } else {
    SM_CHECK(raise_smem_limit(k_gemm_tc<false, OutT>, TcMode<false>::smem));
    k_gemm_tc<false, OutT><<<grid, kTCThreads, TcMode<false>::smem, st>>>(
        mAh, mAl, mBh, mBl, M, N, ktiles, kt_per, alpha, beta, C, ldc, part, status);
  }
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  if (nz > 1) {
    const size_t mn = (size_t)M * N;
    k_tc_reduce<OutT><<<(int)std::min<size_t>((mn + 255) / 256, 4096), 256, 0, st>>>(
        M, N, nz, part, alpha, beta, C, ldc);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
  }
  return SM_OK;
}

template int gemm_tc_planes<double>(Ctx&, cudaStream_t, int, int, int, bool, const void*,
                                    const float*, const void*, const float*, double, double,
                                    double*, int);
template int gemm_tc_planes<float>(Ctx&, cudaStream_t, int, int, int, bool, const void*,
                                   const float*, const void*, const float*, double, double, float*,
                                   int);

int gemm_tc(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, double alpha,
            const double* A, int lda, const double* B, int ldb, double beta, double* C, int ldc,
            bool bf16) {
  const int TK = tc_kslab(bf16);
  const int kp = (K + TK - 1) / TK * TK;
  // op(A)[m][k]: A[m][k] (N) or A[k][m] (T, C: real); op(B)^T[n][k]: B[k][n]
  // (N) or B[n][k] (T, C)
  const int ta = opA == SM_OP_N ? 0 : 1, tb = opB == SM_OP_N ? 1 : 0;
  void *ah, *bh;
  float *al = nullptr, *bl = nullptr;
  const size_t es = bf16 ? 2 : 4;
  SM_CHECK(ctx.scratch(bf16 ? "tc.Abf" : "tc.Ah", es * (size_t)M * kp, &ah));
  SM_CHECK(ctx.scratch(bf16 ? "tc.Bbf" : "tc.Bh", es * (size_t)N * kp, &bh));
  if (!bf16) {
    SM_CHECK(ctx.scratch("tc.Al", (size_t)M * kp, &al));
    SM_CHECK(ctx.scratch("tc.Bl", (size_t)N * kp, &bl));
  }
  SM_CHECK(tc_planes(ctx, st, A, lda, M, K, kp, ta, bf16, ah, al));
  SM_CHECK(tc_planes(ctx, st, B, ldb, N, K, kp, tb, bf16, bh, bl));
  return gemm_tc_planes<double>(ctx, st, M, N, kp, bf16, ah, al, bh, bl, alpha, beta, C, ldc);
}

int tc_status(Ctx& ctx, unsigned int** out) {
  auto it = ctx.bufs.find("tc.status");
  const bool fresh = it == ctx.bufs.end();
  SM_CHECK(ctx.scratch("tc.status", sizeof(unsigned int), reinterpret_cast<void**>(out)));
  if (fresh) SM_CUDA_CHECK(cudaMemset(*out, 0, sizeof(unsigned int)));
  return SM_OK;
}

int tc_status_check(Ctx& ctx, cudaStream_t st) {
  if (ctx.bufs.find("tc.status") == ctx.bufs.end()) return SM_OK;
  unsigned int* status;
  SM_CHECK(tc_status(ctx, &status));
  unsigned int* h = reinterpret_cast<unsigned int*>(ctx.pinned) + 1000;
  SM_CUDA_CHECK(cudaMemcpyAsync(h, status, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
  SM_CUDA_CHECK(cudaStreamSynchronize(st));
  if (*h) {
    SM_CUDA_CHECK(cudaMemsetAsync(status, 0, sizeof(unsigned int), st));
    set_error("tensor-core GEMM: a pipeline wait timed out (status " + std::to_string(*h) + ")");
    return SM_ERR_CUDA;
  }
  return SM_OK;
}

}  // namespace sm
