// FP64-accurate GEMM on the BF16 tensor cores (error-free slicing).
//
//   C[M,N] = alpha * op(A)[M,K] * op(B)[K,N] + beta * C      (real, row-major)
//
// GB300 runs FP64 on the CUDA cores only (~1.2 TFLOP/s); its BF16 tensor cores
// run ~2 PFLOP/s dense.  Following the error-free transformation of matrix
// products of Ozaki, Ogita, Oishi and Rump (Numer. Algorithms 59, 2012), each
// row of op(A) and each column of op(B) is scaled by a power of two to
// (-1, 1) and cut into S = 8 slices of 7-bit integers,
//   x = 2^(e - 7) * sum_i a_i 2^(-7 i),   a_i in [-127, 127],
// which BF16 holds exactly (stored pre-scaled: a_i 2^(-7 i)).  The product is
//   C = 2^(e_m + e_n - 14) * sum_{i + j <= S - 1} A_i B_j^T
// with the slice products on tcgen05 (kind::f16, BF16 in, FP32 accumulate).
// Each t = i + j has its own FP32 accumulator: over a K chunk of 256,
// sum_{i + j = t} A_i B_j^T is an integer times 2^(-7 t) below
// 4 * 256 * 127^2 < 2^24 for t <= 3, so those four are exact; t = 4..7 (below
// 2^-28 of the leading term) lose at most a bit or two of their own 24.  (The
// tensor cores add an MMA result into an accumulator of a different scale with
// only ~17 bits: one accumulator per scale keeps every addition aligned.)
// After each chunk the exact t = 0..4 (integers in units of 2^(-7 t)) are
// added into one int64 per element (units of 2^-28) and t = 5..7 (below 2^-31
// of the leading term) into an FP32 sum; the two become FP64 once, at the end.
// No FP64 arithmetic runs per chunk (GB300's FP64 pipe would bound it).  The
// truncation after 8 slices (56 bits of each row's range) and the dropped
// products (i + j >= 8) are below 2^-56 of the row / column maxima, so the
// result has the accuracy of an FP64 GEMM.
//
// One CTA (10 warps) per 128 x 64 output tile and K range (split over
// blockIdx.z for small outputs):
//   warp 8 / lane 0: TMA, one 3-D box per operand and stage holding all 8
//            slices of a 32-wide K slab (64-byte swizzle), 2 stages;
//   warp 9 / lane 0: 2 x 36 tcgen05.mma (M=128, N=64, K=16) per slab into
//            8 x 64 TMEM columns, a commit per stage and per chunk;
//   warps 0-7: per chunk, tcgen05.ld of the 8 accumulators (warp w owns tile
//            rows 32 (w % 4) .. +31, columns 32 (w / 4) .. +31) into 32 int64
//            + 32 FP32 registers per thread; at the end the scaled FP64 tile
//            (or a split-K partial).
// Every mbarrier wait is bounded; a timeout sets a bit of the status word
// shared with the TF32 path (read by tc_status_check), waits for the CTA's
// copies in flight, frees TMEM and returns.
#include <algorithm>
#include <cfloat>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "kernels.cuh"

namespace sm {

namespace {

constexpr int OM = 128, ON = 64, OK = 32, OS = 2;  // tile M, N, K slab (BF16), stages
constexpr int kSlices = 8;
constexpr int kChunkSlabs = 8;  // 256 of K per exact chunk
constexpr int kGroups = 8;      // one accumulator per t = i + j
constexpr int kOzThreads = 320;  // 8 flush warps, TMA, MMA
constexpr uint32_t kSliceA = OM * OK * 2;  // 8 KB: one slice of A, one slab
constexpr uint32_t kSliceB = ON * OK * 2;  // 4 KB
constexpr uint32_t kOzStage = kSlices * (kSliceA + kSliceB);  // 96 KB
constexpr size_t kOzSmem = (size_t)OS * kOzStage + 1024 + 256;
constexpr uint32_t kOzCols = 512;  // TMEM allocation: 8 accumulators of 64 columns
// instruction descriptor: D = F32, A = B = BF16, K-major, N = 64, M = 128
constexpr uint32_t kOzIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(ON >> 3) << 17) |
                              ((uint32_t)(OM >> 4) << 24);
constexpr unsigned long long kOzWaitNs = 1000000000ull;

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
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
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
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, unsigned long long ns) {
  if (mbar_try_wait(b, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (!mbar_try_wait(b, parity))
    if (gtimer() - t0 > ns) return false;
  return true;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x,
                                            int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
      "%4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// K-major operand, 64-byte swizzle: rows of 64 B, 8-row atoms of 512 B.
__device__ __forceinline__ uint64_t sdesc_sw64(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for this layout)
  d |= (uint64_t)(512 >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)4 << 61;            // 64-byte swizzle
  return d;
}
__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(kOzIdesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
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

__global__ void __launch_bounds__(kOzThreads, 1)
    k_gemm_oz(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB,
              const int* __restrict__ ea, const int* __restrict__ eb, int M, int N, int nslabs,
              int slabs_per, double alpha, double beta, double* __restrict__ C, int ldc,
              double* __restrict__ part, unsigned int* __restrict__ status) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + (size_t)OS * kOzStage);
  uint64_t* empty = full + OS;
  uint64_t* acc_full = empty + OS;
  uint64_t* acc_empty = acc_full + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_empty + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * OM, n0 = blockIdx.x * ON;
  const int s0 = blockIdx.z * slabs_per;
  const int nk = min(nslabs, s0 + slabs_per) - s0;  // >= 1 (host)
  const int nchunks = (nk + kChunkSlabs - 1) / kChunkSlabs;
  if (threadIdx.x == 0) {
    for (int s = 0; s < OS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(acc_full, 1);
    mbar_init(acc_empty, 8);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kOzCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 8) {
    if (lane == 0) {  // producer
      int issued[OS] = {};
      for (int i = 0; i < nk; ++i) {
        const int s = i % OS;
        const uint32_t ph = (uint32_t)(i / OS) & 1u;
        if (i >= OS && !mbar_wait(&empty[s], ph ^ 1u, kOzWaitNs)) {
          atomicOr(status, 16u);
          break;
        }
        unsigned char* stg = base + (size_t)s * kOzStage;
        mbar_expect_tx(&full[s], kOzStage);
        const int x = (s0 + i) * OK;
        tma_load_3d(stg, &mA, &full[s], x, m0, 0);
        tma_load_3d(stg + kSlices * kSliceA, &mB, &full[s], x, n0, 0);
        issued[s] += 1;
      }
      for (int s = 0; s < OS; ++s)
        if (issued[s] && !mbar_wait(&full[s], (uint32_t)(issued[s] - 1) & 1u, kOzWaitNs))
          atomicOr(status, 64u);
    }
  } else if (warp == 9) {
    if (lane == 0) {  // MMA issuer
      bool failed = false;
      for (int i = 0; i < nk; ++i) {
        const int s = i % OS;
        const uint32_t ph = (uint32_t)(i / OS) & 1u;
        const int c = i / kChunkSlabs, first = (i % kChunkSlabs) == 0;
        // the flush of the previous chunk must have read the accumulators
        if (first && c > 0 && !mbar_wait(acc_empty, (uint32_t)(c - 1) & 1u, kOzWaitNs)) {
          atomicOr(status, 32u);
          failed = true;
          break;
        }
        if (!mbar_wait(&full[s], ph, kOzWaitNs)) {
          atomicOr(status, 32u);
          failed = true;
          break;
        }
        tc_fence_after();
        const uint32_t a0 = smem_u32(base + (size_t)s * kOzStage);
        const uint32_t b0 = a0 + kSlices * kSliceA;
        bool written[kGroups] = {};
        if (!first) {
#pragma unroll
          for (int g = 0; g < kGroups; ++g) written[g] = true;
        }
#pragma unroll
        for (int kk = 0; kk < OK / 16; ++kk) {
#pragma unroll
          for (int t = 0; t < kSlices; ++t) {
            const int g = t;
#pragma unroll
            for (int ia = 0; ia <= t; ++ia) {
              const int jb = t - ia;
              const uint64_t da = sdesc_sw64(a0 + ia * kSliceA + kk * 32);
              const uint64_t db = sdesc_sw64(b0 + jb * kSliceB + kk * 32);
              umma_bf16(tmem + (uint32_t)(g * ON), da, db, written[g] ? 1u : 0u);
              written[g] = true;
            }
          }
        }
        umma_commit(&empty[s]);
        if ((i % kChunkSlabs) == kChunkSlabs - 1 || i == nk - 1) umma_commit(acc_full);
      }
      // after a failed wait the flush still learns when the MMAs issued so far
      // have completed (its next wait then runs out and the CTA returns)
      if (failed) umma_commit(acc_full);
    }
  } else {
    // warps 0-7: per chunk, the exact accumulators t = 0..4 (integers in
    // units of 2^(-7 t)) go into one int64 per element in units of 2^-28;
    // t = 5..7 into an FP32 sum (below 2^-31 of the leading term).  Warp w
    // reads TMEM lanes 32 (w % 4) .. +31 (its lane quadrant), columns
    // 32 (w / 4) .. +31 of each accumulator.
    constexpr int HC = ON / 2;
    const int quad = warp & 3, c0 = (warp >> 2) * HC;
    long long S[HC];
    float small[HC];
#pragma unroll
    for (int j = 0; j < HC; ++j) {
      S[j] = 0;
      small[j] = 0.f;
    }
    bool ok = true;
    for (int c = 0; c < nchunks; ++c) {
      ok = mbar_wait(acc_full, (uint32_t)c & 1u, 4 * kOzWaitNs);
      __syncwarp();
      if (!ok) break;
      tc_fence_after();
      const uint32_t lane_base = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0;
#pragma unroll
      for (int cb = 0; cb < HC; cb += 16) {
        float v[16];
#pragma unroll
        for (int g = 7; g >= 5; --g) {
          tmem_ld16(lane_base + (uint32_t)(g * ON + cb), v);
#pragma unroll
          for (int j = 0; j < 16; ++j) small[cb + j] += v[j];
        }
#pragma unroll
        for (int g = 4; g >= 0; --g) {
          tmem_ld16(lane_base + (uint32_t)(g * ON + cb), v);
          const float up = (float)(1u << (7 * g));  // 2^(7 g): v * up is an integer below 2^25
#pragma unroll
          for (int j = 0; j < 16; ++j)
            S[cb + j] += (long long)__float2int_rn(v[j] * up) << (28 - 7 * g);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty);
    }
    if (!ok) {
      if (lane == 0) atomicOr(status, 128u);
    } else {
      const int row = m0 + quad * 32 + lane;
      if (row < M) {
        const int er = max(ea[row], -1100) - 14;
#pragma unroll
        for (int j = 0; j < HC; ++j) {
          const int col = n0 + c0 + j;
          if (col < N) {
            const double acc = fma((double)S[j], 3.725290298461914e-09 /* 2^-28 */,
                                   (double)small[j]);
            // 2^e from its exponent bits (one FP64 multiply; GB300's FP64 pipe
            // makes ldexp's general path expensive), ldexp outside that range
            const int e = er + max(eb[col], -1100);
            const double v = (e > -1022 && e < 1024) ? acc * __hiloint2double((e + 1023) << 20, 0)
                                                     : ldexp(acc, e);
            if (part) {
              part[((size_t)blockIdx.z * M + row) * N + col] = v;
            } else {
              double* p = C + (size_t)row * ldc + col;
              *p = beta == 0.0 ? alpha * v : fma(alpha, v, beta * *p);
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kOzCols)
                 : "memory");
  }
}

// One operand of the preparation kernels: op(X) is rows x K with element
// (r, k) = X[r * ldx + k] (trans = 0) or X[k * ldx + r] (trans = 1).
constexpr int kOzNoExp = (int)0x80808080;  // exponent of an all-zero row

struct OzOperand {
  const double* X;
  int ldx, rows, trans;
  int* ex;
  __nv_bfloat16* out;
};

// Exponent e (x = f 2^e, f in [0.5, 1)) of the largest |element| of each row
// of op(X) into ex; the bytes 0x80 (kOzNoExp) for an all-zero (or non-finite)
// row.  32 x 32 threads per 32 rows over the whole of K; lanes run along the
// contiguous index; blockIdx.z picks the operand.
__global__ void __launch_bounds__(1024) k_oz_exp(OzOperand A, OzOperand B, int K) {
  const OzOperand& o = blockIdx.z ? B : A;
  __shared__ double red[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 32
  const int r0 = blockIdx.x * 32;
  if (r0 >= o.rows) return;  // uniform over the block
  const int k0 = 0, k1 = K;
  double m = 0.0;
  if (o.trans) {  // tx = row, ty strides over k
    const int r = r0 + tx;
    if (r < o.rows)
      for (int k = k0 + ty; k < k1; k += 32) m = fmax(m, fabs(o.X[(size_t)k * o.ldx + r]));
    red[ty][tx] = m;
  } else {  // ty = row, tx strides over k
    const int r = r0 + ty;
    if (r < o.rows)
      for (int k = k0 + tx; k < k1; k += 32) m = fmax(m, fabs(o.X[(size_t)r * o.ldx + k]));
    red[tx][ty] = m;
  }
  __syncthreads();
  if (ty == 0) {  // column tx of red: the 32 partial maxima of row r0 + tx
    double v = 0.0;
    for (int j = 0; j < 32; ++j) v = fmax(v, red[j][tx]);
    const int r = r0 + tx;
    if (r < o.rows) {
      int e = kOzNoExp;
      if (v > 0.0 && v <= DBL_MAX) frexp(v, &e);
      o.ex[r] = e;
    }
  }
}

// The 8 slices of op(X) scaled by 2^-ex[r]: out[(i * rows + r) * kp + k] =
// sign(x) a_i 2^(-7 i) (BF16, exact), zero for k >= K, where a_0 a_1 ... a_7
// are the base-128 digits of |x| 2^-ex[r] < 1, i.e. 7-bit fields of the 56-bit
// fixed-point value F = floor(|x| 2^(56 - ex[r])) taken from the FP64
// significand with integer shifts.  32 x 32 tiles through shared memory so
// reads and writes stay coalesced; blockIdx.z picks the operand.
__global__ void k_oz_slice(OzOperand A, OzOperand B, int K, int kp) {
  const OzOperand& o = blockIdx.z ? B : A;
  __shared__ double tile[32][33];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  if (r0 >= o.rows) return;  // uniform over the block
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int j = ty; j < 32; j += 8) {
    double v = 0.0;
    if (o.trans) {
      const int k = k0 + j, r = r0 + tx;
      if (k < K && r < o.rows) v = o.X[(size_t)k * o.ldx + r];
    } else {
      const int r = r0 + j, k = k0 + tx;
      if (k < K && r < o.rows) v = o.X[(size_t)r * o.ldx + k];
    }
    tile[j][tx] = v;
  }
  __syncthreads();
  const size_t plane = (size_t)o.rows * kp;
  for (int j = ty; j < 32; j += 8) {
    const int r = r0 + j, k = k0 + tx;
    if (r >= o.rows || k >= kp) continue;
    const unsigned long long bits =
        (unsigned long long)__double_as_longlong(o.trans ? tile[tx][j] : tile[j][tx]);
    const int bexp = (int)((bits >> 52) & 0x7FF);
    unsigned long long m = bits & ((1ull << 52) - 1);
    int ev = -1022;  // subnormal
    if (bexp) {
      m |= 1ull << 52;
      ev = bexp - 1023;
    }
    unsigned long long F = 0;
    if (m) {  // |x| = m 2^(ev - 52) < 2^ex[r], so the shift is at most 3
      const int sh = ev - o.ex[r] + 4;
      F = sh >= 0 ? m << sh : (sh > -64 ? m >> (-sh) : 0ull);
    }
    const bool neg = (bits >> 63) != 0;
    float scale = 1.f;
#pragma unroll
    for (int i = 0; i < kSlices; ++i) {
      const float a = (float)(unsigned)((F >> (49 - 7 * i)) & 127ull) * scale;
      o.out[i * plane + (size_t)r * kp + k] = __float2bfloat16_rn(neg ? -a : a);
      scale *= 0.0078125f;  // 2^-7
    }
  }
}

__global__ void k_oz_reduce(int M, int N, int nz, const double* __restrict__ part, double alpha,
                            double beta, double* __restrict__ C, int ldc) {
  const size_t mn = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < mn;
       e += (size_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int z = 0; z < nz; ++z) acc += part[(size_t)z * mn + e];
    double* p = C + (e / N) * ldc + (e % N);
    *p = beta == 0.0 ? alpha * acc : fma(alpha, acc, beta * *p);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 oz_encode_fn() {
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

// 3-D map over the slices: (k, row, slice), box (32, box_rows, 8), 64-byte swizzle
int make_slice_map(CUtensorMap* map, const __nv_bfloat16* base, int rows, int kp, int box_rows) {
  auto enc = oz_encode_fn();
  if (!enc) {
    set_error("FP64 tensor-core GEMM: cuTensorMapEncodeTiled not available");
    return SM_ERR_CUDA;
  }
  const cuuint64_t dims[3] = {(cuuint64_t)kp, (cuuint64_t)rows, (cuuint64_t)kSlices};
  const cuuint64_t strides[2] = {(cuuint64_t)kp * 2, (cuuint64_t)rows * kp * 2};
  const cuuint32_t box[3] = {(cuuint32_t)OK, (cuuint32_t)box_rows, (cuuint32_t)kSlices};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                         const_cast<__nv_bfloat16*>(base), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("FP64 tensor-core GEMM: tensor map encoding failed");
    return SM_ERR_CUDA;
  }
  return SM_OK;
}

}  // namespace

bool gemm_oz_eligible(int M, int N, int K) {
  return (double)M * N * K >= 2.0 * 1024 * 1024 && M >= 32 && N >= 32 && K >= 32 &&
         oz_encode_fn() != nullptr;
}

int gemm_oz(Ctx& ctx, cudaStream_t st, int opA, int opB, int M, int N, int K, double alpha,
            const double* A, int lda, const double* B, int ldb, double beta, double* C, int ldc) {
  const int kp = (K + OK - 1) / OK * OK;
  const int nslabs = kp / OK;
  __nv_bfloat16 *sa, *sb;
  int *ea, *eb;
  unsigned int* status;
  SM_CHECK(ctx.scratch("oz.A", (size_t)kSlices * M * kp, &sa));
  SM_CHECK(ctx.scratch("oz.B", (size_t)kSlices * N * kp, &sb));
  SM_CHECK(ctx.scratch("oz.ea", (size_t)M, &ea));
  SM_CHECK(ctx.scratch("oz.eb", (size_t)N, &eb));
  SM_CHECK(tc_status(ctx, &status));
  // op(A)[m][k] = A[m][k] (N) or A[k][m] (T, C: real); op(B)^T[n][k] = B[k][n]
  // (N) or B[n][k] (T, C)
  const int ta = opA == SM_OP_N ? 0 : 1, tb = opB == SM_OP_N ? 1 : 0;
  const OzOperand oa{A, lda, M, ta, ea, sa}, ob{B, ldb, N, tb, eb, sb};
  const int rb = (std::max(M, N) + 31) / 32;
  k_oz_exp<<<dim3(rb, 1, 2), dim3(32, 32), 0, st>>>(oa, ob, K);
  k_oz_slice<<<dim3(kp / 32, rb, 2), dim3(32, 8), 0, st>>>(oa, ob, K, kp);
  note_launch(2);
  SM_CUDA_CHECK(cudaGetLastError());
  CUtensorMap mA, mB;
  SM_CHECK(make_slice_map(&mA, sa, M, kp, OM));
  SM_CHECK(make_slice_map(&mB, sb, N, kp, ON));
  const int tiles = ((M + OM - 1) / OM) * ((N + ON - 1) / ON);
  // split K over CTAs while the output has fewer tiles than SMs, in whole
  // 32-wide slabs, at least two per CTA (each CTA's range is accumulated in
  // exact chunks of at most 256, so any slab split is exact)
  int nz = std::max(1, std::min(std::max(1, ctx.num_sms) / tiles, nslabs / 2));
  const int slabs_per = (nslabs + nz - 1) / nz;
  nz = (nslabs + slabs_per - 1) / slabs_per;
  double* part = nullptr;
  if (nz > 1) SM_CHECK(ctx.scratch("oz.part", (size_t)nz * M * N, &part));
  SM_CHECK(raise_smem_limit(k_gemm_oz, kOzSmem));
  const dim3 grid((N + ON - 1) / ON, (M + OM - 1) / OM, nz);
  k_gemm_oz<<<grid, kOzThreads, kOzSmem, st>>>(mA, mB, ea, eb, M, N, nslabs, slabs_per, alpha,
                                               beta, C, ldc, part, status);
  note_launch();
  SM_CUDA_CHECK(cudaGetLastError());
  if (nz > 1) {
    const size_t mn = (size_t)M * N;
    k_oz_reduce<<<(int)std::min<size_t>((mn + 255) / 256, 4096), 256, 0, st>>>(M, N, nz, part,
                                                                               alpha, beta, C, ldc);
    note_launch();
    SM_CUDA_CHECK(cudaGetLastError());
  }
  return SM_OK;
}

}  // namespace sm
