// Mixed-precision split: rank-revealing QR + one-sided Jacobi in FP32 inside
// ONE thread-block cluster of 16 CTAs.
//
// The FP64 iteration (svd.cu) spreads every Jacobi round over the whole GPU
// and pays a grid barrier plus a round trip through L2 per round; at the
// sizes of the two-site splits (<= 768 x 512) that latency, not the FP64
// pipe, is the bound.  Here the whole factorisation of one split runs on 16
// SMs that talk through distributed shared memory (DSMEM) and the hardware
// cluster barrier:
//
//   phase 0  |W|_F^2 in FP64; W / |W|_F is stored in FP32, column c of W in
//            the shared memory of CTA c % 16 (so FP32 cannot overflow even
//            for operators with 1/h^2 ~ 1e18 entries).
//   phase 1  blocked Householder QR of W (reflectors act on the columns,
//            length kw).  The columns are dealt out in blocks of qb (<= 8):
//            block g lives in CTA g % 16.  One cluster barrier per block
//            step: every CTA applies the block's qb reflectors to its columns
//            beyond it in compact WY form (two passes over the rows; lanes
//            own columns and warps own rows, so every reflector-row load is a
//            shared-memory broadcast); then the CTA owning the next block
//            factors that block's columns (its "panel") with all its threads:
//            each holds two rows of the panel in registers, and a reflector
//            costs one CTA-wide sum.  Before that, block column pivoting puts
//            the 8 live columns of largest remaining weight into the panel's
//            positions (every CTA sends its heaviest to the owner, which
//            swaps the winners' data in over DSMEM and records the swap in
//            CTA 0's permutation; phase 4 undoes it).  The owner writes the
//            reflector block
//            and its T factor once to global memory; after the barrier every
//            other CTA copies them from L2 into its shared memory (a DSMEM
//            broadcast from one SM to 15 is bound by that SM's outgoing
//            stores, measured at ~46 bytes per clock).  The factorisation
//            stops at the first step whose trailing block holds at most thr
//            of |W|_F^2 (rank revealing), leaving keff rows of R; the
//            trailing weights of all qb steps of a block come from the column
//            weights after the block (the later reflectors of a block leave
//            the weight below each earlier step unchanged).
//   phase 2  the rows of R are cut into 32 blocks of r = ceil(keff / 32) rows;
//            CTA c holds block positions c and 31 - c in shared memory.
//   phase 3  block-cyclic one-sided Jacobi: per sweep, the pairs inside each
//            block once, then 31 block rounds in which each CTA rotates all
//            r x r pairs between its two blocks (r local rounds of r disjoint
//            pairs, one warp per pair, CTA barriers only) and passes its
//            blocks to the neighbouring CTAs through double-buffered DSMEM
//            mailboxes.  One cluster barrier per block round (31 per sweep).
//   phase 4  the rows (= diag(s) V^H of the rows of R, i.e. of W, in W's own
//            column order) go back to global memory in FP64, rescaled by
//            |W|_F, with their FP64 norms.
//
// Only the accuracy of the iteration changes: the rows of V^H are accurate
// to FP32 rounding.  The caller re-orthonormalises them in FP64 and forms the
// other factor with an FP64 GEMM from the exact matrix, so the split it
// returns is an exact FP64 factorisation of a rank-D approximation whose
// discarded weight is computed exactly (|A|^2 - |kept factor|^2).
#include <cooperative_groups.h>

#include <algorithm>
#include <cfloat>
#include <cmath>

#include "kernels.cuh"

namespace cg = cooperative_groups;

namespace sm {

namespace {

constexpr int kCW = 16;            // CTAs per cluster
constexpr int kCNT = 512;          // threads per CTA
constexpr int kCNW = kCNT / 32;    // warps per CTA
constexpr int kMaxRows = 512;      // rows of R the Jacobi phase takes (32 blocks of <= 16)
// Jacobi: a sweep whose rotations all start below cosine 1e-2 ends the iteration
constexpr float kStopC2 = 1e-4f;
constexpr int kQB = 8;             // widest column block of the QR (reflectors per cluster barrier)
constexpr int kPanelRP = 2;        // rows per thread of the QR panel in registers (kw <= 1024)
// Scale floors (W is held as W / |W|_F, so these are relative to |W|):
// a QR column whose part below its pivot has norm <= kTinyCol gets no
// reflector (the part, weight <= 1e-30, is dropped; its tau would approach
// the FP32 range); the QR also stops once the trailing weight is below
// kQrFloor whatever the threshold asked; the Jacobi leaves rows of squared
// norm below kTinyRow2 alone and rotates only pairs whose normalised |g|^2
// is above kTinyG2 (clear of the SFU's subnormal flush).
constexpr float kTinyCol = 1e-15f;
constexpr float kQrFloor = 1e-24f;
constexpr float kTinyRow2 = 1e-30f;
constexpr float kTinyG2 = 1e-36f;

// column slots per CTA for l columns in blocks of qb
__host__ __device__ inline int qr_slots(int l, int qb) {
  return ((l + qb * kCW - 1) / (qb * kCW)) * qb;
}
// Shared memory of the QR phase: the columns [ncs][ks] (ks = kw | 1: an odd
// stride keeps lanes that own different columns on different banks; padded
// to 16 bytes), two reflector blocks [kwp][qb] (kwp = kw rounded up to a
// multiple of 4, so each block is a multiple of 16 bytes), two T factors
// [8][8], and the block update's scratch:
// y partials [16][qb][32] and sums [qb][32] (F), row weights [qb][32] and
// tail weights [16][32] (float).
template <typename F>
__host__ __device__ inline size_t qr_cols_elems(int ncs, int kw) {
  const size_t per16 = 16 / sizeof(F);
  return ((size_t)ncs * (kw | 1) + per16 - 1) / per16 * per16;
}
template <typename F>
__host__ __device__ inline size_t qr_bytes(int ncs, int kw, int qb) {
  const size_t kwp = (size_t)((kw + 3) & ~3);
  const size_t slab =
      sizeof(F) * (size_t)(kCNW + 1) * qb * 32 + sizeof(float) * (size_t)(qb + kCNW) * 32;
  return sizeof(F) * (qr_cols_elems<F>(ncs, kw) + 2 * kwp * qb + 2 * kQB * kQB) + slab;
}

// ---- FP32 element helpers ----------------------------------------------------
template <typename T> struct F32;
template <> struct F32<double> {
  using type = float;
  __device__ static float from(double x, double s) { return (float)(x * s); }
  __device__ static double to(float x, double s) { return (double)x * s; }
  __device__ static float zero() { return 0.0f; }
};
template <> struct F32<cplx> {
  using type = float2;
  __device__ static float2 from(cplx x, double s) {
    return make_float2((float)(x.re * s), (float)(x.im * s));
  }
  __device__ static cplx to(float2 x, double s) { return cplx{(double)x.x * s, (double)x.y * s}; }
  __device__ static float2 zero() { return make_float2(0.f, 0.f); }
};

__device__ __forceinline__ float f_abs2(float x) { return x * x; }
__device__ __forceinline__ float f_abs2(float2 x) { return fmaf(x.x, x.x, x.y * x.y); }
// acc += conj(u) v
__device__ __forceinline__ void f_dotc(float u, float v, float& gr, float&) { gr = fmaf(u, v, gr); }
__device__ __forceinline__ void f_dotc(float2 u, float2 v, float& gr, float& gi) {
  gr = fmaf(u.x, v.x, fmaf(u.y, v.y, gr));
  gi = fmaf(u.x, v.y, fmaf(-u.y, v.x, gi));
}
// c -= (wr + i wi) v
__device__ __forceinline__ void f_axpy(float wr, float, float v, float& c) { c = fmaf(-wr, v, c); }
__device__ __forceinline__ void f_axpy(float wr, float wi, float2 v, float2& c) {
  c.x = fmaf(-wr, v.x, fmaf(wi, v.y, c.x));
  c.y = fmaf(-wr, v.y, fmaf(-wi, v.x, c.y));
}
__device__ __forceinline__ float f_re(float x) { return x; }
__device__ __forceinline__ float f_re(float2 x) { return x.x; }
__device__ __forceinline__ float f_im(float) { return 0.f; }
__device__ __forceinline__ float f_im(float2 x) { return x.y; }
__device__ __forceinline__ void f_set(float& x, float re, float) { x = re; }
__device__ __forceinline__ void f_set(float2& x, float re, float im) { x = make_float2(re, im); }

// the elements of a float4 as F values
__device__ __forceinline__ void unpack4(float4 t, float* v) {
  v[0] = t.x;
  v[1] = t.y;
  v[2] = t.z;
  v[3] = t.w;
}
__device__ __forceinline__ void unpack4(float4 t, float2* v) {
  v[0] = make_float2(t.x, t.y);
  v[1] = make_float2(t.z, t.w);
}

// tan of the Jacobi angle, 1 / (|zeta| + sqrt(1 + zeta^2)), with the SFU's
// approximate reciprocal square root and reciprocal (a few ulp; the rotation
// built from it is orthogonal to FP32 rounding whatever the angle's error)
__device__ __forceinline__ float rot_tan(float az) {
  const float q = fmaf(az, az, 1.0f);
  return __fdividef(1.0f, fmaf(q, rsqrtf(q), az));
}

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Control words of one CTA (after the data region of its shared memory).
struct CtrlS {
  int flag[2];                 // CTA 0: a rotation happened in the sweep of this parity
  int c2max[2];                // CTA 0: largest rotated cos^2 of that sweep (float bits)
  float2 gram[kQB][kQB];       // panel reflector Gram matrix v_i^H v_k (i < k; re, im)
  float2 prow[2][kQB];         // the panel's pivot row (re, im), by reflector parity
  float rsq[kQB][kQB];         // |R|^2 of the rows just below the panel's first row
  float pred[kCNW][16];        // CTA-sum partials
  float pfin[16];
  float part[2][kCW][kQB];     // trailing-weight partials of all CTAs, by block-step parity
  float inpanel[kQB][kQB];     // owner of a panel: weight of panel column k below step i
  double part64[kCW];          // |W|^2 partials of all CTAs
  float cn[64];                // remaining squared norm of each column slot (-1: not a candidate)
  float cand_v[kCW][kQB];      // next panel's owner: every CTA's heaviest columns (value,
  int cand_p[kCW][kQB];        //   position; -1: none)
  int cand_n[kCW];             //   valid entries per CTA
  int sel[kQB];                // next panel's owner: the chosen positions, heaviest first
  int nsel;
  int swp[2][kQB];             // next panel's owner: positions swapped (chosen, panel)
  unsigned short perm[768];    // CTA 0: original column of each position
  float red[kCNW][kQB];        // CTA-local reduction scratch
  double red64[kCNW];
};

// CTA-wide sum of 16 floats (entries n.. must be zero; every thread gets the
// sums; fixed order).  Within a warp a butterfly that halves the values it
// carries at each level (16 shuffles for the 16 sums): lanes 2a and 2a+1 end
// with the warp's sum of value a.
__device__ __forceinline__ void cta_sum(CtrlS* ctrl, float (&v)[16], int n) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int h = 8, o = 16; h >= 1; h >>= 1, o >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      if (a < h) {
        const float keep = up ? v[a + h] : v[a];
        const float send = up ? v[a] : v[a + h];
        v[a] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
    }
  }
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
  if ((lane & 1) == 0 && (lane >> 1) < n) ctrl->pred[warp][lane >> 1] = v[0];
  __syncthreads();
  if (tid < n) {
    float t = 0.f;
    for (int w = 0; w < kCNW; ++w) t += ctrl->pred[w][tid];
    ctrl->pfin[tid] = t;
  }
  __syncthreads();
#pragma unroll
  for (int a = 0; a < 16; ++a)
    if (a < n) v[a] = ctrl->pfin[a];
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Shared memory (bytes) for a k_split_cluster launch.
template <typename T, int E>
size_t cluster_smem(int kw, int l, int qb) {
  using F = typename F32<T>::type;
  const size_t qr = qr_bytes<F>(qr_slots(l, qb), kw, qb);
  const size_t rmax = (size_t)(std::min(std::min(kw, l), kMaxRows) + 2 * kCW - 1) / (2 * kCW);
  const size_t jb = sizeof(F) * 6 * rmax * 32 * E;  // 2 blocks + 2 x 2 mailboxes
  return ((std::max(qr, jb) + 15) / 16) * 16 + sizeof(CtrlS);
}

// W (kw x l) is A (m x n) itself (trans = 0) or A^T (trans = 1).  Writes kcap
// rows (FP64, ld = l) and their norms; rows past the Jacobi's are zero.
template <typename T, int E>
__global__ void __launch_bounds__(kCNT, 1)
    k_split_cluster(const T* __restrict__ A, int n_a, int trans, int kw, int l, double thr_rel,
                    double thr_abs, float tol2, int max_sweeps, T* __restrict__ out_rows,
                    double* __restrict__ out_nrm, int kcap, JacobiCtl* ctl_out,
                    double* __restrict__ info, int qr_cap, int qb, float* __restrict__ vbuf,
                    int pivot, const int* __restrict__ cap_dev) {
  using F = typename F32<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int gw = rank * kCNW + warp;
  // column c: block c / qb, held by CTA (c / qb) % 16 in slot
  // ((c / qb) / 16) qb + c % qb
  const int ncs = qr_slots(l, qb);  // column slots per CTA
  const int kmax = min(kw, l);
  // a learned rank caps the QR steps (0: the trailing weight alone decides);
  // a cap computed on the device by the rank predictor replaces qr_cap
  if (cap_dev) qr_cap = cap_dev[0];
  const int qsteps = qr_cap > 0 ? min(kmax, qr_cap) : kmax;
  constexpr int LP = 32 * E;

  F* cols = reinterpret_cast<F*>(smem_raw);        // [ncs][kw], phase 1
  F* refl = cols + qr_cols_elems<F>(ncs, kw);      // reflector blocks, see phase 1
  const int ks = kw | 1;                           // column stride
  const size_t qr = qr_bytes<F>(ncs, kw, qb);
  auto col_of = [&](int s) { return ((s / qb) * kCW + rank) * qb + s % qb; };
  const size_t rmax = (size_t)(min(kmax, kMaxRows) + 2 * kCW - 1) / (2 * kCW);
  const size_t jb = sizeof(F) * 6 * rmax * LP;
  CtrlS* ctrl = reinterpret_cast<CtrlS*>(smem_raw + ((max(qr, jb) + 15) / 16) * 16);
  CtrlS* ctrl0 = cluster.map_shared_rank(ctrl, 0);

  auto Wat = [&](int i, int c) -> T {  // W[i][c]
    return trans ? A[(size_t)c * n_a + i] : A[(size_t)i * n_a + c];
  };

  // ---- phase 0: |W|^2 (FP64) and the scaled FP32 copy ------------------------
  const unsigned long long t_start = global_ns();
  if (tid < 2) {
    ctrl->flag[tid] = 0;
    ctrl->c2max[tid] = 0;
  }
  {
    double acc = 0.0;
    for (int s = warp; s < ncs; s += kCNW) {
      const int c = col_of(s);
      if (c >= l) break;
      for (int i = lane; i < kw; i += 32) acc += S<T>::abs2(Wat(i, c));
    }
    acc = warp_sum(acc);
    if (lane == 0) ctrl->red64[warp] = acc;
    __syncthreads();
    if (tid < kCW) {  // every CTA receives every partial
      double t = 0.0;
      for (int w = 0; w < kCNW; ++w) t += ctrl->red64[w];
      cluster.map_shared_rank(ctrl, tid)->part64[rank] = t;
    }
  }
  cluster.sync();
  double norm2 = 0.0;
  for (int r = 0; r < kCW; ++r) norm2 += ctrl->part64[r];
  const double nrm = sqrt(norm2);
  const double scale = nrm > 0.0 ? 1.0 / nrm : 1.0;
  // stop once the trailing block holds at most max(thr_rel |W|^2, thr_abs)
  const float thr =
      fmaxf((float)fmax(thr_rel, norm2 > 0.0 ? thr_abs / norm2 : 0.0), kQrFloor);
  for (int s = warp; s < ncs; s += kCNW) {
    const int c = col_of(s);
    if (c >= l) break;
    for (int i = lane; i < kw; i += 32) cols[(size_t)s * ks + i] = F32<T>::from(Wat(i, c), scale);
  }
  if (rank == 0)
    for (int c = tid; c < l; c += kCNT) ctrl->perm[c] = (unsigned short)c;
  __syncthreads();
  // squared column norms: the candidates for the first panel
  for (int s = warp; s < 64; s += kCNW) {
    const int c = s < ncs ? col_of(s) : l;
    float a = 0.f;
    if (c < l)
      for (int i = lane; i < kw; i += 32) a += f_abs2(cols[(size_t)s * ks + i]);
    a = warp_sum(a);
    if (lane == 0) ctrl->cn[s] = c < l ? a : -1.f;
  }
  __syncthreads();

  // ---- phase 1: rank-revealing blocked Householder QR -------------------------
  // Row `row` of a block of reflectors (qb entries, 128-bit loads when qb = 8).
  constexpr int NV4 = kQB * (int)sizeof(F) / 16;
  auto load_vrow = [&](const F* Vp, int row, F* v) {
    if (qb == kQB) {
      const float4* s4 = reinterpret_cast<const float4*>(Vp + (size_t)row * kQB);
#pragma unroll
      for (int u = 0; u < NV4; ++u) unpack4(s4[u], v + u * (4 / (int)(sizeof(F) / 4)));
    } else {
#pragma unroll
      for (int i = 0; i < kQB; ++i) v[i] = i < qb ? Vp[(size_t)row * qb + i] : F32<T>::zero();
    }
  };
  const int kwp = (kw + 3) & ~3;  // rows of a reflector block buffer (16-byte multiple)
  F* Vb = refl;                              // [2][kwp][qb]
  F* Tm = Vb + (size_t)2 * kwp * qb;         // [2][kQB][kQB]
  F* ys = Tm + (size_t)2 * kQB * kQB;        // [16][qb][32]: y partials of the block update
  F* ysum = ys + (size_t)kCNW * qb * 32;     // [qb][32]
  float* ebin = reinterpret_cast<float*>(ysum + (size_t)qb * 32);  // [qb][32]
  float* tl = ebin + (size_t)qb * 32;                                // [16][32]
  // Every live column of this CTA (col >= c0 + nb) through the block of nb
  // reflectors in compact WY form (H_{nb-1} .. H_0 = I - V T^H V^H, Vp
  // row-major [row][qb], Tp = T [8][8] upper triangular): y = V^H col,
  // z = T^H y, col -= V z on rows c0..kw-1.  Lane j owns column slot 32 g + j,
  // warp w the rows c0 + w + 16 t.  acc[i] (all lanes of warp 0) gains the
  // weights below the block's steps, the sum over the live columns of
  // |col[c0+i+1:kw)|^2.  All threads; ends with a CTA barrier.
  auto update_block = [&](const F* Vp, const F* Tp, int c0, int nb, float* acc) {
    for (int g = 0; g * 32 < ncs; ++g) {
      const int sl = g * 32 + lane;
      const int c = sl < ncs ? col_of(sl) : l;
      const bool live = c < l && c >= c0 + nb;
      F* col = cols + (size_t)(live ? sl : 0) * ks;
      float yr[kQB], yi[kQB];
#pragma unroll
      for (int i = 0; i < kQB; ++i) yr[i] = yi[i] = 0.f;
#pragma unroll 2
      for (int row = c0 + warp; row < kw; row += kCNW) {
        F v[kQB];
        load_vrow(Vp, row, v);
        const F x = live ? col[row] : F32<T>::zero();
#pragma unroll
        for (int i = 0; i < kQB; ++i)
          if (i < nb) f_dotc(v[i], x, yr[i], yi[i]);
      }
#pragma unroll
      for (int i = 0; i < kQB; ++i)
        if (i < nb) f_set(ys[((size_t)warp * qb + i) * 32 + lane], yr[i], yi[i]);
      __syncthreads();
      if (tid < nb * 32) {  // fixed-order sum over the warps
        float sr = 0.f, si = 0.f;
        for (int w = 0; w < kCNW; ++w) {
          const F t = ys[(size_t)w * qb * 32 + tid];
          sr += f_re(t);
          si += f_im(t);
        }
        f_set(ysum[tid], sr, si);
      }
      __syncthreads();
      float zr[kQB], zi[kQB];  // z_k = sum_{i <= k} conj(T_ik) y_i
#pragma unroll
      for (int k = 0; k < kQB; ++k) {
        zr[k] = zi[k] = 0.f;
#pragma unroll
        for (int i = 0; i <= k; ++i) {
          if (i < nb && k < nb) {
            const F t = Tp[i * kQB + k];
            const F y = ysum[i * 32 + lane];
            zr[k] = fmaf(f_re(t), f_re(y), fmaf(f_im(t), f_im(y), zr[k]));
            zi[k] = fmaf(f_re(t), f_im(y), fmaf(-f_im(t), f_re(y), zi[k]));
          }
        }
      }
      float tail = 0.f;
#pragma unroll 2
      for (int row = c0 + warp; row < kw; row += kCNW) {
        F v[kQB];
        load_vrow(Vp, row, v);
        F x = live ? col[row] : F32<T>::zero();
#pragma unroll
        for (int i = 0; i < kQB; ++i)
          if (i < nb) f_axpy(zr[i], zi[i], v[i], x);
        if (live) col[row] = x;
        const float x2 = f_abs2(x);
        if (row >= c0 + nb) tail += x2;
        else if (row > c0) ebin[(row - c0) * 32 + lane] = x2;  // rows c0+1 .. c0+nb-1
      }
      tl[warp * 32 + lane] = tail;
      __syncthreads();
      if (warp == 0) {
        float run = 0.f;  // S(nb-1) = the tail, S(i) = S(i+1) + |col[c0+i+1]|^2
        for (int w = 0; w < kCNW; ++w) run += tl[w * 32 + lane];
        // the column's weight below the block, |col[c0+nb:kw)|^2: its pivot
        // candidate value for the next panel
        ctrl->cn[g * 32 + lane] = live ? run : -1.f;
        float sv[kQB];  // this lane's S(i), then the nb independent warp sums
#pragma unroll
        for (int i = kQB - 1; i >= 0; --i) {
          sv[i] = i < nb ? run : 0.f;
          if (i >= 1 && i < nb) run += ebin[i * 32 + lane];
        }
#pragma unroll
        for (int i = 0; i < kQB; ++i)
          if (i < nb) acc[i] += warp_sum(sv[i]);
      }
      __syncthreads();
    }
  };
  auto Vpar = [&](int p) { return Vb + (size_t)p * kwp * qb; };
  auto Tpar = [&](int p) { return Tm + (size_t)p * kQB * kQB; };
  // Panel of the owner CTA: columns cp .. cp+nbp-1 (slots sp ..), factored by
  // the whole CTA.  Thread t holds rows t and t + 512 of the panel's columns
  // in registers; each reflector is two CTA-wide sums (the column norm with
  // the reflector Gram entries it completes, then v^H of the later columns).
  // Reflector i (pivot row j = cp + i): v = x + nu e_j, nu = (x_j/|x_j|)|x|,
  // tau = 1/(|x|(|x|+|x_j|)), x_j <- -nu, x = rows j..kw-1 of column i; v is
  // zero above row j.  Writes the block of reflectors into Vpar(p), its T
  // factor into Tpar(p), the R entries back into the columns, and the
  // in-panel weights inpanel[k][i] = |R[cp+i+1 .. cp+k, cp+k]|^2 (i < k).
  auto factor_panel = [&](int cp, int nbp, int sp, int p) {
    F x[kPanelRP][kQB];
    F v0s[kQB];
    float taus[kQB];
#pragma unroll
    for (int pr = 0; pr < kPanelRP; ++pr) {
      const int row = tid + kCNT * pr;
#pragma unroll
      for (int k = 0; k < kQB; ++k)
        x[pr][k] = (k < nbp && row >= cp && row < kw) ? cols[(size_t)(sp + k) * ks + row]
                                                      : F32<T>::zero();
    }
#pragma unroll
    for (int i = 0; i < kQB; ++i) {
      v0s[i] = F32<T>::zero();
      taus[i] = 0.f;
    }
    // Reflectors one by one (v_m on a row below its pivot is the column's
    // stored value), one CTA-wide sum each: with the pivot row's values
    // broadcast first, the column norm, the Gram entries v_m^H v_i (m < i) and
    // the products d_k = v_i^H x_k (k > i) all come from sums over the rows
    // below the pivot, v_i being x_i there (d_k adds conj(v0_i) x_k[j] after
    // the sum).  The pivot values alternate between two buffers, so a step's
    // writes never meet the previous step's reads (one barrier apart).
#pragma unroll
    for (int i = 0; i < kQB; ++i) {
      if (i < nbp) {
        const int j = cp + i;
        float2* prw = ctrl->prow[i & 1];
#pragma unroll
        for (int pr = 0; pr < kPanelRP; ++pr)
          if (tid + kCNT * pr == j) {
#pragma unroll
            for (int m = 0; m < kQB; ++m)
              if (m < nbp) prw[m] = make_float2(f_re(x[pr][m]), f_im(x[pr][m]));
          }
        // red[0] = |x_i|^2 over rows >= j; over rows > j, slots 1 + 2 s, 2 + 2 s:
        // conj(x_m) x_i for m < i (s = m), conj(x_i) x_k for k > i (s = k - 1)
        float red[16];
#pragma unroll
        for (int a = 0; a < 16; ++a) red[a] = 0.f;
#pragma unroll
        for (int pr = 0; pr < kPanelRP; ++pr) {
          const int row = tid + kCNT * pr;
          if (row >= j && row < kw) red[0] += f_abs2(x[pr][i]);
          if (row > j && row < kw) {
#pragma unroll
            for (int m = 0; m < kQB; ++m) {
              if (m < i) {
                float gr = 0.f, gi = 0.f;
                f_dotc(x[pr][m], x[pr][i], gr, gi);
                red[1 + 2 * m] += gr;
                red[2 + 2 * m] += gi;
              } else if (m > i && m < nbp) {
                float gr = 0.f, gi = 0.f;
                f_dotc(x[pr][i], x[pr][m], gr, gi);
                red[2 * m - 1] += gr;
                red[2 * m] += gi;
              }
            }
          }
        }
        cta_sum(ctrl, red, 2 * nbp - 1);
        const float2 xp = prw[i];
        F x0;
        f_set(x0, xp.x, xp.y);
        const float xn = sqrtf(red[0]);
        const float a0 = sqrtf(f_abs2(x0));
        float pr_ = 1.f, pi_ = 0.f;  // phase of x_j
        if (a0 > 0.f) {
          pr_ = f_re(x0) / a0;
          pi_ = f_im(x0) / a0;
        }
        // no reflector for a column that is already zero to the noise floor
        const bool refl = xn > kTinyCol;
        if (refl) f_set(v0s[i], f_re(x0) + pr_ * xn, f_im(x0) + pi_ * xn);
        taus[i] = refl ? 1.0f / (xn * (xn + a0)) : 0.f;
        const float v0r = f_re(v0s[i]), v0i = f_im(v0s[i]);
        // Gram entries v_m^H v_i = (rows > j) + conj(v_m[j]) v0_i
        if (tid == 0) {
#pragma unroll
          for (int m = 0; m < i; ++m) {
            const float2 vm = prw[m];
            const float gr = red[1 + 2 * m] + vm.x * v0r + vm.y * v0i;
            const float gi = red[2 + 2 * m] + vm.x * v0i - vm.y * v0r;
            ctrl->gram[m][i] = make_float2(gr, gi);
          }
        }
        // v_i on this thread's rows; the pivot row of column i becomes -nu
        F vi[kPanelRP];
#pragma unroll
        for (int pr = 0; pr < kPanelRP; ++pr) {
          const int row = tid + kCNT * pr;
          vi[pr] = !refl ? F32<T>::zero()
                         : (row > j && row < kw) ? x[pr][i] : (row == j ? v0s[i] : F32<T>::zero());
          if (row == j && refl) f_set(x[pr][i], -pr_ * xn, -pi_ * xn);
        }
        // x_k -= tau d_k v_i, d_k = v_i^H x_k = (rows > j) + conj(v0_i) x_k[j]
#pragma unroll
        for (int k = i + 1; k < kQB; ++k) {
          if (k < nbp) {
            const float2 xk = prw[k];
            const float dr = red[2 * k - 1] + v0r * xk.x + v0i * xk.y;
            const float di = red[2 * k] + v0r * xk.y - v0i * xk.x;
            const float wr = taus[i] * dr, wi = taus[i] * di;
#pragma unroll
            for (int pr = 0; pr < kPanelRP; ++pr) f_axpy(wr, wi, vi[pr], x[pr][k]);
          }
        }
      }
    }
    // R entries and reflectors back to shared memory
    F* Vp = Vpar(p);
#pragma unroll
    for (int pr = 0; pr < kPanelRP; ++pr) {
      const int row = tid + kCNT * pr;
      if (row >= cp && row < kw) {
#pragma unroll
        for (int k = 0; k < kQB; ++k) {
          if (k < nbp) cols[(size_t)(sp + k) * ks + row] = x[pr][k];
          if (k < qb) {
            const int jk = cp + k;
            const F v = (k >= nbp || taus[k] == 0.f)
                            ? F32<T>::zero()
                            : (row > jk ? x[pr][k] : (row == jk ? v0s[k] : F32<T>::zero()));
            Vp[(size_t)row * qb + k] = v;
          }
        }
        // |R[row][cp+k]|^2 for the rows just below the block's first row
        const int rr = row - cp;
        if (rr >= 1 && rr < kQB) {
#pragma unroll
          for (int k = 0; k < kQB; ++k)
            ctrl->rsq[rr][k] = (k < nbp && k >= rr) ? f_abs2(x[pr][k]) : 0.f;
        }
      }
    }
    __syncthreads();
    // inpanel[k][i] = sum_{r=i+1}^{k} |R[cp+r][cp+k]|^2 ; T row i (lane i of warp 0):
    // T_kk = tau_k, T[0:k, k] = -tau_k T[0:k, 0:k] gram[0:k, k]
    if (warp == 0 && lane < kQB) {
      const int i = lane;
#pragma unroll
      for (int k = 0; k < kQB; ++k) {
        float t = 0.f;
        for (int r = i + 1; r <= k && r < kQB; ++r) t += ctrl->rsq[r][k];
        ctrl->inpanel[k][i] = (k < nbp && i < k) ? t : 0.f;
      }
      F* Tp = Tpar(p);
      float tre[kQB], tim[kQB];
#pragma unroll
      for (int k = 0; k < kQB; ++k) {
        float tr = 0.f, ti = 0.f;
        if (k < nbp) {
          if (i == k) {
            tr = taus[k];
          } else if (i < k) {
            float sr = 0.f, si = 0.f;  // sum_{m=i}^{k-1} T_im gram_mk
#pragma unroll
            for (int m = 0; m < k; ++m) {
              if (m >= i) {
                const float2 g = ctrl->gram[m][k];
                sr += tre[m] * g.x - tim[m] * g.y;
                si += tre[m] * g.y + tim[m] * g.x;
              }
            }
            tr = -taus[k] * sr;
            ti = -taus[k] * si;
          }
        }
        tre[k] = tr;
        tim[k] = ti;
        f_set(Tp[i * kQB + k], tr, ti);
      }
    }
  };
  // The owner of a block writes its reflector block (rows from the block's
  // first row) and T to the global buffer of that parity; every other CTA
  // copies them into its own shared memory after the barrier (L2 loads: the
  // buffer is rewritten every other block).
  F* vg = reinterpret_cast<F*>(vbuf);
  auto Gpar = [&](int p) { return vg + (size_t)p * ((size_t)kwp * qb + kQB * kQB); };
  const int nt4 = kQB * kQB * (int)sizeof(F) / 16;
  auto publish = [&](int cp, int p) {  // all threads of the owner CTA
    const int b0 = (int)((size_t)cp * qb * sizeof(F) / 16);
    const int b1 = (int)((size_t)kwp * qb * sizeof(F) / 16);
    float4* g = reinterpret_cast<float4*>(Gpar(p));
    const float4* src = reinterpret_cast<const float4*>(Vpar(p));
    for (int f = b0 + tid; f < b1; f += kCNT) g[f] = src[f];
    float4* gt = reinterpret_cast<float4*>(Gpar(p) + (size_t)kwp * qb);
    if (tid < nt4) gt[tid] = reinterpret_cast<const float4*>(Tpar(p))[tid];
  };
  auto fetch = [&](int cp, int p) {  // all threads of every other CTA
    const int b0 = (int)((size_t)cp * qb * sizeof(F) / 16);
    const int b1 = (int)((size_t)kwp * qb * sizeof(F) / 16);
    const float4* g = reinterpret_cast<const float4*>(Gpar(p));
    float4* dst = reinterpret_cast<float4*>(Vpar(p));
    for (int f = b0 + tid; f < b1; f += kCNT) dst[f] = __ldcg(g + f);
    const float4* gt = reinterpret_cast<const float4*>(Gpar(p) + (size_t)kwp * qb);
    if (tid < nt4) reinterpret_cast<float4*>(Tpar(p))[tid] = __ldcg(gt + tid);
    __syncthreads();
  };
  auto slot_of = [&](int c) { return ((c / qb) / kCW) * qb + c % qb; };
  // Block column pivoting: the columns of the panel at positions cp ..
  // cp+nbp-1 become the nbp live columns of largest remaining weight (cn, set
  // from the columns' current values below row cp).  Every CTA sends its own
  // heaviest nbp (value, position) to the panel's owner; after a cluster
  // barrier the owner picks the heaviest nbp of all, swaps their column data
  // (all kw rows) with the panel's positions over DSMEM and records the swaps
  // in CTA 0's permutation.  The other CTAs wait at the step's barrier while
  // their columns move.  All threads of all CTAs.
  auto pivot_panel = [&](int cp, int nbp, int owner) {
    CtrlS* co = cluster.map_shared_rank(ctrl, owner);
    if (warp == 0) {  // this CTA's heaviest nbp slots, largest first (ties: smaller slot)
      float v0 = lane < ncs ? ctrl->cn[lane] : -1.f;
      float v1 = lane + 32 < ncs ? ctrl->cn[lane + 32] : -1.f;
      float myv = -1.f;  // lane k keeps the k-th result
      int myp = -1, nv = 0;
#pragma unroll 1
      for (int k = 0; k < nbp; ++k) {
        float bv = v0 >= v1 ? v0 : v1;
        int bs = v0 >= v1 ? lane : lane + 32;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
          const int os = __shfl_xor_sync(0xffffffffu, bs, o);
          if (ov > bv || (ov == bv && os < bs)) {
            bv = ov;
            bs = os;
          }
        }
        if (bv < 0.f) break;  // uniform over the warp
        if (lane == k) {
          myv = bv;
          myp = col_of(bs);
        }
        ++nv;
        if (bs == lane) v0 = -1.f;
        else if (bs == lane + 32) v1 = -1.f;
      }
      // one store per array to the owner (lanes k < nv)
      if (lane < nv) {
        co->cand_v[rank][lane] = myv;
        co->cand_p[rank][lane] = myp;
      }
      if (lane == 0) co->cand_n[rank] = nv;
    }
    cluster.sync();
    if (rank != owner) return;
    if (warp == 0) {  // merge of the 16 descending lists: lane c holds list c's head
      const int c = lane & (kCW - 1);
      const int nc = ctrl->cand_n[c];
      int head = 0;
      float hv = (lane < kCW && nc > 0) ? ctrl->cand_v[c][0] : -1.f;
      int hp = (lane < kCW && nc > 0) ? ctrl->cand_p[c][0] : 0x7fffffff;
      int ns = 0;
#pragma unroll 1
      for (int k = 0; k < nbp; ++k) {
        float bv = hv;
        int bp = hp, bl = lane;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {  // largest value, then smallest position
          const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
          const int op = __shfl_xor_sync(0xffffffffu, bp, o);
          const int ol = __shfl_xor_sync(0xffffffffu, bl, o);
          if (ov > bv || (ov == bv && op < bp)) {
            bv = ov;
            bp = op;
            bl = ol;
          }
        }
        if (bv < 0.f) break;  // uniform over the warp
        if (lane == 0) ctrl->sel[k] = bp;
        ++ns;
        if (lane == bl) {  // the winning list advances
          ++head;
          hv = head < nc ? ctrl->cand_v[c][head] : -1.f;
          hp = head < nc ? ctrl->cand_p[c][head] : 0x7fffffff;
        }
      }
      if (lane == 0) ctrl->nsel = ns;
    }
    __syncthreads();
    const int nsel = ctrl->nsel;
    // chosen columns already inside the panel stay; the others are paired in
    // order with the panel positions that were not chosen
    bool outside = false, freep = false;
    if (tid < nsel) {
      const int c = ctrl->sel[tid];
      outside = c < cp || c >= cp + nbp;
    }
    if (tid >= 32 && tid < 32 + nbp) {
      const int pp = cp + tid - 32;
      freep = true;
      for (int k = 0; k < nsel; ++k) freep = freep && ctrl->sel[k] != pp;
    }
    const int ns = __syncthreads_count(outside);
    if (outside) {
      int oi = 0;
      for (int k = 0; k < tid; ++k) {
        const int c = ctrl->sel[k];
        oi += (c < cp || c >= cp + nbp) ? 1 : 0;
      }
      ctrl->swp[0][oi] = ctrl->sel[tid];
    }
    if (freep) {
      int fi = 0;
      for (int j = 0; j < tid - 32; ++j) {
        bool f = true;
        for (int k = 0; k < nsel; ++k) f = f && ctrl->sel[k] != cp + j;
        fi += f ? 1 : 0;
      }
      if (fi < ns) ctrl->swp[1][fi] = cp + tid - 32;
    }
    __syncthreads();
    // swap the column data: pair k, row i for f = k * kw + i (independent
    // items), two per thread at a time so that their DSMEM loads overlap
    for (int f = tid; f < ns * kw; f += 2 * kCNT) {
      const int g = f + kCNT;
      const bool two = g < ns * kw;
      const int k = f / kw, i = f % kw, k2 = two ? g / kw : k, i2 = two ? g % kw : i;
      F* pa = cluster.map_shared_rank(cols + (size_t)slot_of(ctrl->swp[0][k]) * ks,
                                      (ctrl->swp[0][k] / qb) % kCW);
      F* pa2 = cluster.map_shared_rank(cols + (size_t)slot_of(ctrl->swp[0][k2]) * ks,
                                       (ctrl->swp[0][k2] / qb) % kCW);
      F* pb = cols + (size_t)slot_of(ctrl->swp[1][k]) * ks;  // the panel's positions are the owner's
      F* pb2 = cols + (size_t)slot_of(ctrl->swp[1][k2]) * ks;
      const F ta = pa[i], ta2 = pa2[i2];
      const F tb = pb[i], tb2 = pb2[i2];
      pa[i] = tb;
      pb[i] = ta;
      if (two) {
        pa2[i2] = tb2;
        pb2[i2] = ta2;
      }
    }
    if (tid < ns) {
      unsigned short* pm = cluster.map_shared_rank(ctrl, 0)->perm;
      const int a = ctrl->swp[0][tid], b = ctrl->swp[1][tid];
      const unsigned short t = pm[a];
      pm[a] = pm[b];
      pm[b] = t;
    }
    __syncthreads();
  };
  // block 0: pivoted and factored by CTA 0 before the first step's barrier
  const int nb0 = min(qb, qsteps);
  if (pivot && nb0 > 0) pivot_panel(0, nb0, 0);
  if (rank == 0 && nb0 > 0) {
    factor_panel(0, nb0, 0, 0);
    __syncthreads();
    publish(0, 0);
  }
  cluster.sync();
  int keff = qsteps;
  float trail = 0.f;
  for (int q = 0; q * qb < qsteps; ++q) {
    const int par = q & 1;
    const int c0 = q * qb, nb = min(qb, qsteps - c0);
    const int c1 = c0 + qb, nb1 = min(qb, qsteps - c1);  // next block (nb1 <= 0: none)
    const bool owner1 = nb1 > 0 && rank == (q + 1) % kCW;
    const int sp1 = owner1 ? slot_of(c1) : -1;
    if (rank != q % kCW) fetch(c0, par);
    const F* Vq = Vpar(par);
    const F* Tq = Tpar(par);
    float acc[kQB];
#pragma unroll
    for (int i = 0; i < kQB; ++i) acc[i] = 0.f;
    update_block(Vq, Tq, c0, nb, acc);
    if (tid == 0) {
#pragma unroll
      for (int i = 0; i < kQB; ++i) ctrl->red[0][i] = acc[i];
    }
    // the next panel: its columns chosen by weight, now up to date
    if (pivot && nb1 > 0) pivot_panel(c1, nb1, (q + 1) % kCW);
    if (owner1) {
      factor_panel(c1, nb1, sp1, par ^ 1);
      __syncthreads();
      publish(c1, par ^ 1);
    } else {
      __syncthreads();
    }
    if (tid < kCW * kQB) {  // every CTA receives every partial
      const int dst = tid / kQB, i = tid % kQB;
      float t = 0.f;
      if (i < nb) {
        t = ctrl->red[0][i];
        // the block's own panel (factored by this CTA in the previous step)
        if (rank == q % kCW)
          for (int k = 0; k < nb; ++k) t += ctrl->inpanel[k][i];
      }
      cluster.map_shared_rank(ctrl, dst)->part[par][rank][i] = t;
    }
    cluster.sync();
    bool stop = false;
    for (int i = 0; i < nb; ++i) {
      float t = 0.f;
      for (int r = 0; r < kCW; ++r) t += ctrl->part[par][r][i];
      trail = t;
      if (t <= thr) {
        keff = c0 + i + 1;
        stop = true;
        break;
      }
    }
    if (stop) break;
  }
  const unsigned long long t_qr = global_ns();

  // ---- phase 2: rows of R into the row blocks ---------------------------------
  // 32 block positions of r rows (zero rows past keff); CTA c holds position c
  // ("top") and position 31 - c ("bottom").  The rows are gathered into
  // registers first: the block storage reuses the column storage, which other
  // CTAs read until the barrier.
  const int r = max(1, (keff + 2 * kCW - 1) / (2 * kCW));
  const int blk = r * LP;  // elements of one block
  F* Tb = reinterpret_cast<F*>(smem_raw);
  F* Bb = Tb + blk;
  F* mbox = Bb + blk;  // [slot 0 top / 1 bottom][parity][blk]
  {
    F tmp[2 * E];
    const int tot = 2 * blk;
#pragma unroll
    for (int u = 0; u < 2 * E; ++u) {
      const int f = tid + u * kCNT;
      tmp[u] = F32<T>::zero();
      if (f < tot) {
        const int half = f / blk, ri = (f % blk) / LP, x = f % LP;
        const int i = (half ? 2 * kCW - 1 - rank : rank) * r + ri;
        if (i < keff && x < l && x >= i)
          tmp[u] = cluster.map_shared_rank(cols + (size_t)slot_of(x) * ks, (x / qb) % kCW)[i];
      }
    }
    cluster.sync();  // column storage is dead from here on
#pragma unroll
    for (int u = 0; u < 2 * E; ++u) {
      const int f = tid + u * kCNT;
      if (f < tot) Tb[f] = tmp[u];
    }
    __syncthreads();
  }

  // ---- phase 3: block-cyclic one-sided Jacobi ------------------------------
  // A lane holds NV float4 of a row (elements 4 lane + 128 e .. + 3, natural
  // order), loaded and stored as 128-bit shared-memory accesses.
  constexpr int NV = (E * (int)sizeof(F)) / 16;
  auto load_row = [&](const F* row, float4* x) {
    const float4* r4 = reinterpret_cast<const float4*>(row);
#pragma unroll
    for (int e = 0; e < NV; ++e) x[e] = r4[lane + 32 * e];
  };
  auto store_row = [&](F* row, const float4* x) {
    float4* r4 = reinterpret_cast<float4*>(row);
#pragma unroll
    for (int e = 0; e < NV; ++e) r4[lane + 32 * e] = x[e];
  };
  // Squared norms and conj(u) v of the register rows u, v (warp sums).
  auto pair_gram = [&](const float4* u, const float4* v, float& a_, float& b_, float& gr_,
                       float& gi_) {
    float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f, gr0 = 0.f, gr1 = 0.f, gi0 = 0.f, gi1 = 0.f;
#pragma unroll
    for (int e = 0; e < NV; ++e) {
      const float4 p = u[e], q = v[e];
      a0 = fmaf(p.x, p.x, fmaf(p.y, p.y, a0));
      a1 = fmaf(p.z, p.z, fmaf(p.w, p.w, a1));
      b0 = fmaf(q.x, q.x, fmaf(q.y, q.y, b0));
      b1 = fmaf(q.z, q.z, fmaf(q.w, q.w, b1));
      if constexpr (sizeof(F) == 4) {
        gr0 = fmaf(p.x, q.x, fmaf(p.y, q.y, gr0));
        gr1 = fmaf(p.z, q.z, fmaf(p.w, q.w, gr1));
      } else {  // (x, y) and (z, w) are complex numbers: conj(p) q
        gr0 = fmaf(p.x, q.x, fmaf(p.y, q.y, gr0));
        gi0 = fmaf(p.x, q.y, fmaf(-p.y, q.x, gi0));
        gr1 = fmaf(p.z, q.z, fmaf(p.w, q.w, gr1));
        gi1 = fmaf(p.z, q.w, fmaf(-p.w, q.z, gi1));
      }
    }
    a_ = warp_sum(a0 + a1);
    b_ = warp_sum(b0 + b1);
    gr_ = warp_sum(gr0 + gr1);
    gi_ = 0.f;
    if constexpr (sizeof(F) != 4) gi_ = warp_sum(gi0 + gi1);
  };
  // Rotates the register rows u, v of this warp; true if it rotated.
  float c2w = 0.f;  // this warp's largest rotated cos^2 in the sweep
  auto rotate_regs = [&](float4* u, float4* v) -> bool {
    float a_, b_, gr_, gi_;
    pair_gram(u, v, a_, b_, gr_, gi_);
    // The rotation depends on a : b : g only, so it is decided on the pair's
    // Gram entries divided by max(a, b): rows far below |W| (1e-14 of it and
    // less) have products a b and g^2 below the FP32 range, and left unrotated
    // they stay nearly parallel, which no later FP64 step separates.  Rows
    // whose squared norm is itself near the bottom of the range (< 1e-30 |W|^2,
    // weight no rank rule can see) are left alone.
    if (!(fminf(a_, b_) >= kTinyRow2)) return false;
    const float sc = __fdividef(1.0f, fmaxf(a_, b_));
    const float a = a_ * sc, b = b_ * sc, gr = gr_ * sc, gi = gi_ * sc;
    const float g2 = fmaf(gr, gr, gi * gi);
    if (!(g2 > kTinyG2 && g2 > tol2 * a * b)) return false;
    c2w = fmaxf(c2w, __fdividef(g2, a * b));
    const float rg = rsqrtf(g2);
    const float zeta = 0.5f * (b - a) * rg;
    const float az = fabsf(zeta);
    const float tt =
        copysignf(az < 1e18f ? rot_tan(az) : 0.5f / az, zeta);
    const float c = rsqrtf(fmaf(tt, tt, 1.0f));
    const float sn = c * tt;
    const float ar = sn * gr * rg, ai = sn * gi * rg;  // s e
#pragma unroll
    for (int e = 0; e < NV; ++e) {
      const float4 p = u[e], q = v[e];
      float4 np, nq;
      if constexpr (sizeof(F) == 4) {
        np = make_float4(fmaf(c, p.x, -ar * q.x), fmaf(c, p.y, -ar * q.y), fmaf(c, p.z, -ar * q.z),
                         fmaf(c, p.w, -ar * q.w));
        nq = make_float4(fmaf(ar, p.x, c * q.x), fmaf(ar, p.y, c * q.y), fmaf(ar, p.z, c * q.z),
                         fmaf(ar, p.w, c * q.w));
      } else {  // p' = c p - conj(s e) q ; q' = (s e) p + c q
        np = make_float4(c * p.x - (ar * q.x + ai * q.y), c * p.y - (ar * q.y - ai * q.x),
                         c * p.z - (ar * q.z + ai * q.w), c * p.w - (ar * q.w - ai * q.z));
        nq = make_float4((ar * p.x - ai * p.y) + c * q.x, (ar * p.y + ai * p.x) + c * q.y,
                         (ar * p.z - ai * p.w) + c * q.z, (ar * p.w + ai * p.z) + c * q.w);
      }
      u[e] = np;
      v[e] = nq;
    }
    return true;
  };
  auto mark = [&](int sweep) {
    if (lane == 0) ctrl0->flag[sweep & 1] = 1;
  };
  int status = DEV_NOT_CONVERGED, sweeps = max_sweeps;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    c2w = 0.f;
    // pairs inside each block (circle method over r positions, padded to even)
    {
      const int rp2 = r + (r & 1);
      const int half = rp2 / 2;
      for (int t = 0; t < rp2 - 1; ++t) {
        const int side = warp / 8, w8 = warp % 8;
        if (w8 < half) {
          int p, q;
          if (w8 == 0) { p = rp2 - 1; q = t; }
          else { p = (t + w8) % (rp2 - 1); q = (t + rp2 - 1 - w8) % (rp2 - 1); }
          if (p < r && q < r) {
            F* base = side ? Bb : Tb;
            float4 u[NV], v[NV];
            load_row(base + (size_t)p * LP, u);
            load_row(base + (size_t)q * LP, v);
            if (rotate_regs(u, v)) {
              store_row(base + (size_t)p * LP, u);
              store_row(base + (size_t)q * LP, v);
              mark(sweep);
            }
          }
        }
        __syncthreads();
      }
    }
    // 31 block rounds: top x bottom pairs (warp w keeps top row w in
    // registers, the bottom rows come by), then the blocks move
    for (int br = 0; br < 2 * kCW - 1; ++br) {
      float4 tr[NV];
      if (warp < r) load_row(Tb + (size_t)warp * LP, tr);
      bool trot = false;
      for (int t = 0; t < r; ++t) {
        if (warp < r) {
          F* brow = Bb + (size_t)((warp + t) % r) * LP;
          float4 v[NV];
          load_row(brow, v);
          if (rotate_regs(tr, v)) {
            store_row(brow, v);
            trot = true;
          }
        }
        __syncthreads();
      }
      if (trot) {
        store_row(Tb + (size_t)warp * LP, tr);
        mark(sweep);
      }
      __syncthreads();
      const int par = br & 1;
      const int n4 = blk * (int)sizeof(F) / 16;
      auto send = [&](const F* src, int dst_rank, int slot) {
        float4* d = reinterpret_cast<float4*>(
            cluster.map_shared_rank(mbox + (size_t)(slot * 2 + par) * blk, dst_rank));
        const float4* s4 = reinterpret_cast<const float4*>(src);
        for (int f = tid; f < n4; f += kCNT) d[f] = s4[f];
      };
      if (rank == 0) send(Bb, 1, 0);
      else {
        if (rank + 1 < kCW) send(Tb, rank + 1, 0);
        send(Bb, rank - 1, 1);
      }
      // end of the sweep: the largest rotated cos^2 goes to CTA 0
      if (br == 2 * kCW - 2 && lane == 0 && c2w > 0.f)
        atomicMax(&ctrl0->c2max[sweep & 1], __float_as_int(c2w));
      cluster.sync();
      const float4* mt = reinterpret_cast<const float4*>(mbox + (size_t)(0 * 2 + par) * blk);
      const float4* mb = reinterpret_cast<const float4*>(mbox + (size_t)(1 * 2 + par) * blk);
      float4* T4 = reinterpret_cast<float4*>(Tb);
      float4* B4 = reinterpret_cast<float4*>(Bb);
      if (rank == kCW - 1) {
        for (int f = tid; f < n4; f += kCNT) B4[f] = T4[f];
        __syncthreads();
        for (int f = tid; f < n4; f += kCNT) T4[f] = mt[f];
      } else if (rank == 0) {
        for (int f = tid; f < n4; f += kCNT) B4[f] = mb[f];
      } else {
        for (int f = tid; f < n4; f += kCNT) {
          T4[f] = mt[f];
          B4[f] = mb[f];
        }
      }
      __syncthreads();
      // the previous sweep's flag was read by every CTA before this barrier
      if (br == 0 && sweep > 0 && rank == 0 && tid == 0) {
        ctrl->flag[(sweep + 1) & 1] = 0;
        ctrl->c2max[(sweep + 1) & 1] = 0;
      }
    }
    // Converged when nothing rotated, or when every rotation of the sweep
    // started from a cosine below 1e-2: the iteration converges
    // quadratically, so the rows leave such a sweep orthogonal to ~1e-4 / gap,
    // which the two quadratically convergent FP64 refinement steps take to
    // ~1e-16 / gap; a further FP32 sweep would cost as much as both of them
    // (on the 512 x 512 workload split: 10 sweeps instead of 11 for the 2e-3
    // rule, the same split, no fallback).
    const int rotated = ctrl0->flag[sweep & 1];
    if (!rotated || __int_as_float(ctrl0->c2max[sweep & 1]) < kStopC2) {
      status = 0;
      sweeps = sweep + 1;
      break;
    }
  }

  // ---- phase 4: rows back to global memory (FP64, rescaled) ------------------
  const unsigned short* perm0 = cluster.map_shared_rank(ctrl, 0)->perm;
  for (int j = warp; j < 2 * r; j += kCNW) {
    const int row = (j < r ? rank : 2 * kCW - 1 - rank) * r + (j % r);
    if (row >= kcap) continue;
    const F* src = Tb + (size_t)j * LP;  // Bb == Tb + blk: rows j >= r are the bottom block
    double acc = 0.0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int c = lane + 32 * e;  // a position of the pivoted QR: column perm[c] of W
      if (c < l) {
        const T x = F32<T>::to(src[c], nrm);
        out_rows[(size_t)row * l + perm0[c]] = x;
        acc += S<T>::abs2(x);
      }
    }
    acc = warp_sum(acc);
    if (lane == 0) out_nrm[row] = sqrt(acc);
  }
  // zero rows 32 r .. kcap-1
  for (int row = 2 * kCW * r + gw; row < kcap; row += kCW * kCNW) {
    for (int c = lane; c < l; c += 32) out_rows[(size_t)row * l + c] = S<T>::zero();
    if (lane == 0) out_nrm[row] = 0.0;
  }
  if (rank == 0 && tid == 0) {
    ctl_out->status = status;
    ctl_out->sweeps = sweeps;
    ctl_out->nact = keff;
    ctl_out->cap = qr_cap;
    ctl_out->pred = cap_dev ? cap_dev[1] : 0;
    info[0] = norm2;
    info[1] = (double)trail * norm2;
    info[5] = 1e-6 * (double)(t_qr - t_start);       // ms: load + QR
    info[6] = 1e-6 * (double)(global_ns() - t_qr);   // ms: gather + Jacobi + store
  }
  cluster.sync();  // no CTA leaves while another may still read its shared memory
}

// The widest QR column block (8, 4, 2 or 1) whose shared memory fits.
template <typename T, int E>
int pick_qb(int kw, int l) {
  for (int qb = kQB; qb >= 1; qb /= 2)
    if (cluster_smem<T, E>(kw, l, qb) <= 227 * 1024) return qb;
  return 0;
}

template <typename T, int E>
bool cluster_config(int kw, int l, size_t* smem_out, int* qb_out) {
  const int qb = pick_qb<T, E>(kw, l);
  if (qb == 0) return false;
  const size_t smem = cluster_smem<T, E>(kw, l, qb);
  *qb_out = qb;
  auto fn = k_split_cluster<T, E>;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      raise_smem_limit(fn, smem) != SM_OK) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kCW);
  cfg.blockDim = dim3(kCNT);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kCW;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nc = 0;
  if (cudaOccupancyMaxActiveClusters(&nc, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  *smem_out = smem;
  return nc > 0;
}

template <typename T, int E>
int launch_split_cluster(cudaStream_t st, const T* A, int n_a, int trans, int kw, int l,
                         double thr_rel, double thr_abs, int max_sweeps, T* out_rows,
                         double* out_nrm, int kcap, JacobiCtl* ctl, double* info, int qr_cap,
                         float* vbuf, int pivot, const int* cap_dev) {
  size_t smem = 0;
  int qb = 0;
  if (!cluster_config<T, E>(kw, l, &smem, &qb)) {
    set_error("mixed split: cluster configuration not available");
    return SM_ERR_VALUE;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kCW);
  cfg.blockDim = dim3(kCNT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kCW;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const float eps = FLT_EPSILON;
  const float tol2 = (float)l * eps * eps;
  SM_CUDA_CHECK(cudaLaunchKernelEx(&cfg, k_split_cluster<T, E>, A, n_a, trans, kw, l, thr_rel,
                                   thr_abs, tol2, max_sweeps, out_rows, out_nrm, kcap, ctl,
                                   info, qr_cap, qb, vbuf, pivot, cap_dev));
  note_launch();
  return SM_OK;
}

// Elements per lane of a row (a multiple of 4: rows move as float4).
inline int e_bucket(int l) {
  const int need = (l + 31) / 32;
  if (need <= 4) return 4;
  if (need <= 8) return 8;
  if (need <= 12) return 12;
  if (need <= 16) return 16;
  if (need <= 24) return 24;
  return 0;
}

}  // namespace

// The sizes the cluster kernel takes (shared memory and registers aside).
template <typename T>
bool split_cluster_size_ok(int kw, int l) {
  if (std::min(kw, l) > kMaxRows || kw > kCNT * kPanelRP) return false;
  const int e = e_bucket(l);
  return e != 0 && (sizeof(T) == sizeof(double) || e <= 16);
}

template <typename T>
bool split_cluster_fits(int kw, int l) {
  // the QR panel holds kPanelRP rows per thread in registers
  if (std::min(kw, l) > kMaxRows || kw > kCNT * kPanelRP) return false;
  const int e = e_bucket(l);
  if (e == 0) return false;
  if (sizeof(T) != sizeof(double) && e > 16) return false;  // complex rows beyond 512 spill
  // Residency is checked once per (dtype, E): the answer does not depend on
  // the sizes beyond the shared-memory amount, which is re-checked below.
  size_t smem = 0;
  int qb = 0;
  switch (e) {
    case 4: return cluster_config<T, 4>(kw, l, &smem, &qb);
    case 8: return cluster_config<T, 8>(kw, l, &smem, &qb);
    case 12: return cluster_config<T, 12>(kw, l, &smem, &qb);
    case 16: return cluster_config<T, 16>(kw, l, &smem, &qb);
    default: return cluster_config<T, 24>(kw, l, &smem, &qb);
  }
}

template <typename T>
int split_cluster_f32(cudaStream_t st, const T* A, int m, int n, bool want_u, double thr_rel,
                      double thr_abs, int max_sweeps, T* out_rows, double* out_nrm, int kcap,
                      JacobiCtl* ctl, double* info, int qr_cap, float* vbuf, bool pivot,
                      const int* cap_dev) {
  // W = A^T (kw = n, l = m) when U is wanted, else W = A (kw = m, l = n)
  const int kw = want_u ? n : m;
  const int l = want_u ? m : n;
  const int trans = want_u ? 1 : 0;
  switch (e_bucket(l)) {
#define SM_C(EV)                                                                              \
  case EV:                                                                                    \
    return launch_split_cluster<T, EV>(st, A, n, trans, kw, l, thr_rel, thr_abs, max_sweeps, \
                                       out_rows, out_nrm, kcap, ctl, info, qr_cap, vbuf,  \
                                       pivot ? 1 : 0, cap_dev)
    SM_C(4);
    SM_C(8);
    SM_C(12);
    SM_C(16);
    SM_C(24);
#undef SM_C
    default:
      break;
  }
  set_error("mixed split: row length beyond the cluster kernel's limit");
  return SM_ERR_VALUE;
}

template bool split_cluster_size_ok<double>(int, int);
template bool split_cluster_size_ok<cplx>(int, int);
template bool split_cluster_fits<double>(int, int);
template bool split_cluster_fits<cplx>(int, int);
template int split_cluster_f32<double>(cudaStream_t, const double*, int, int, bool, double,
                                       double, int, double*, double*, int, JacobiCtl*, double*,
                                       int, float*, bool, const int*);
template int split_cluster_f32<cplx>(cudaStream_t, const cplx*, int, int, bool, double, double,
                                     int, cplx*, double*, int, JacobiCtl*, double*, int, float*,
                                     bool, const int*);

size_t split_cluster_vbuf_floats(int kw) {
  // two parities of a reflector block [kwp][8] and its T [8][8], complex
  return (size_t)2 * (((size_t)(kw + 3) & ~(size_t)3) * kQB + kQB * kQB) * 2;
}

}  // namespace sm
