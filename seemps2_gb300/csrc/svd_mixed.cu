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
//   phase 1  Householder QR of W (reflectors act on the columns, length kw),
//            one cluster barrier per step; the warp that owns column j + 1
//            forms the next reflector in the same step and its CTA pushes it
//            into every other CTA before the barrier (no read after the
//            barrier leaves the SM).  The factorisation stops once the
//            trailing block holds at most thr of |W|_F^2 (rank revealing),
//            leaving keff rows of R.
//   phase 2  the rows of R are cut into 32 blocks of r = ceil(keff / 32) rows;
//            CTA c holds block positions c and 31 - c in shared memory.
//   phase 3  block-cyclic one-sided Jacobi: per sweep, the pairs inside each
//            block once, then 31 block rounds in which each CTA rotates all
//            r x r pairs between its two blocks (r local rounds of r disjoint
//            pairs, one warp per pair, CTA barriers only) and passes its
//            blocks to the neighbouring CTAs through double-buffered DSMEM
//            mailboxes.  One cluster barrier per block round (31 per sweep).
//   phase 4  the rows (= diag(s) V^H of the rows of R, i.e. of W) go back to
//            global memory in FP64, rescaled by |W|_F, with their FP64 norms.
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

// Rotation of a row pair: p' = c p - s conj(e) q ; q' = s e p + c q, with e
// the phase of g = <p, q>.
__device__ __forceinline__ void f_rot(float& p, float& q, float c, float s, float er, float) {
  const float np = fmaf(c, p, -s * er * q);
  const float nq = fmaf(s * er, p, c * q);
  p = np;
  q = nq;
}
__device__ __forceinline__ void f_rot(float2& p, float2& q, float c, float s, float er, float ei) {
  const float ar = s * er, ai = s * ei;
  const float2 np = make_float2(c * p.x - (ar * q.x + ai * q.y), c * p.y - (ar * q.y - ai * q.x));
  const float2 nq = make_float2((ar * p.x - ai * p.y) + c * q.x, (ar * p.y + ai * p.x) + c * q.y);
  p = np;
  q = nq;
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
  int flag[2];        // CTA 0: a rotation happened in the sweep of this parity
  float tau[2];       // reflector tau, by step parity (pushed by the owner)
  float part[2][kCW]; // trailing-weight partials of all CTAs, by step parity
  double part64[kCW]; // |W|^2 partials of all CTAs
  float red[kCNW];    // CTA-local reduction scratch
  double red64[kCNW];
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Shared memory (bytes) for a k_split_cluster launch.
template <typename T, int E>
size_t cluster_smem(int kw, int l) {
  using F = typename F32<T>::type;
  const size_t ncs = (size_t)(l + kCW - 1) / kCW;
  const size_t qr = sizeof(F) * (ncs * (size_t)kw + 2 * (size_t)kw);
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
                    double* __restrict__ info, int qr_cap) {
  using F = typename F32<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int gw = rank * kCNW + warp;
  const int ncs = (l + kCW - 1) / kCW;  // column slots per CTA
  const int kmax = min(kw, l);
  // a learned rank caps the QR steps (0: the trailing weight alone decides)
  const int qsteps = qr_cap > 0 ? min(kmax, qr_cap) : kmax;
  constexpr int LP = 32 * E;

  F* cols = reinterpret_cast<F*>(smem_raw);        // [ncs][kw], phase 1
  F* refl = cols + (size_t)ncs * kw;               // [2][kw]
  const size_t qr = sizeof(F) * ((size_t)ncs * kw + 2 * (size_t)kw);
  const size_t rmax = (size_t)(min(kmax, kMaxRows) + 2 * kCW - 1) / (2 * kCW);
  const size_t jb = sizeof(F) * 6 * rmax * LP;
  CtrlS* ctrl = reinterpret_cast<CtrlS*>(smem_raw + ((max(qr, jb) + 15) / 16) * 16);
  CtrlS* ctrl0 = cluster.map_shared_rank(ctrl, 0);

  auto Wat = [&](int i, int c) -> T {  // W[i][c]
    return trans ? A[(size_t)c * n_a + i] : A[(size_t)i * n_a + c];
  };

  // ---- phase 0: |W|^2 (FP64) and the scaled FP32 copy ------------------------
  const unsigned long long t_start = global_ns();
  if (tid < 2) ctrl->flag[tid] = 0;
  {
    double acc = 0.0;
    for (int s = warp; s < ncs; s += kCNW) {
      const int c = rank + s * kCW;
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
  const float thr = (float)fmax(thr_rel, norm2 > 0.0 ? thr_abs / norm2 : 0.0);
  for (int s = warp; s < ncs; s += kCNW) {
    const int c = rank + s * kCW;
    if (c >= l) break;
    for (int i = lane; i < kw; i += 32) cols[(size_t)s * kw + i] = F32<T>::from(Wat(i, c), scale);
  }
  __syncthreads();

  // ---- phase 1: rank-revealing Householder QR --------------------------------
  // Reflector from x = col[j:kw): v = x + nu e1, nu = (x0/|x0|)|x|,
  // tau = 1/(|x|(|x|+|x0|)); col[j] <- -nu.  `xn2` = |x|^2.  One warp.
  auto make_reflector = [&](F* col, int j, float xn2, F* vdst, float* tau_dst) {
    const float xn = sqrtf(xn2);
    const F x0 = col[j];
    const float a0 = sqrtf(f_abs2(x0));
    float pr = 1.f, pi = 0.f;  // phase of x0
    if (a0 > 0.f) {
      pr = f_re(x0) / a0;
      pi = f_im(x0) / a0;
    }
    for (int i = j + 1 + lane; i < kw; i += 32) vdst[i] = col[i];
    __syncwarp();  // every lane has read x0 before lane 0 overwrites it
    if (lane == 0) {
      F v0;
      f_set(v0, f_re(x0) + pr * xn, f_im(x0) + pi * xn);
      vdst[j] = v0;
      *tau_dst = xn > 0.f ? 1.0f / (xn * (xn + a0)) : 0.f;
      F d;
      f_set(d, -pr * xn, -pi * xn);
      col[j] = d;
    }
  };
  // The owner CTA of the next reflector pushes it (and tau) into every other
  // CTA's buffer of that parity before the barrier; the trailing-weight
  // partials are pushed to every CTA the same way, so after the barrier all
  // reads are local.
  auto push_reflector = [&](int j, int par) {  // all threads of the owner CTA
    F* v = refl + (size_t)par * kw;
    for (int r = 0; r < kCW; ++r) {
      if (r == rank) continue;
      F* d = cluster.map_shared_rank(v, r);
      for (int i = j + tid; i < kw; i += kCNT) d[i] = v[i];
    }
    if (tid < kCW && tid != rank) cluster.map_shared_rank(ctrl, tid)->tau[par] = ctrl->tau[par];
  };
  if (rank == 0 && warp == 0 && l > 0) {
    float xn2 = 0.f;
    for (int i = lane; i < kw; i += 32) xn2 += f_abs2(cols[i]);
    xn2 = warp_sum(xn2);
    make_reflector(cols, 0, xn2, refl, &ctrl->tau[0]);
  }
  __syncthreads();
  if (rank == 0 && l > 0) push_reflector(0, 0);
  cluster.sync();
  int keff = qsteps;
  float trail = 0.f;
  for (int j = 0; j < qsteps; ++j) {
    const int par = j & 1;
    const F* v = refl + (size_t)par * kw;
    const float tau = ctrl->tau[par];
    float tw = 0.f;  // this warp's trailing weight
    for (int s = warp; s < ncs; s += kCNW) {
      const int c = rank + s * kCW;
      if (c >= l) break;
      if (c <= j) continue;
      F* col = cols + (size_t)s * kw;
      float dr = 0.f, di = 0.f;
      for (int i = j + lane; i < kw; i += 32) f_dotc(v[i], col[i], dr, di);
      dr = warp_sum(dr);
      di = warp_sum(di);
      const float wr = tau * dr, wi = tau * di;
      float cn = 0.f;
      for (int i = j + lane; i < kw; i += 32) {
        F x = col[i];
        f_axpy(wr, wi, v[i], x);
        col[i] = x;
        if (i > j) cn += f_abs2(x);
      }
      cn = warp_sum(cn);
      tw += cn;
      if (c == j + 1 && j + 1 < kmax) {
        __syncwarp();
        make_reflector(col, j + 1, cn, refl + (size_t)(par ^ 1) * kw, &ctrl->tau[par ^ 1]);
      }
    }
    if (lane == 0) ctrl->red[warp] = tw;
    __syncthreads();
    if (j + 1 < kmax && rank == (j + 1) % kCW) push_reflector(j + 1, par ^ 1);
    if (tid < kCW) {
      float t = 0.f;
      for (int w = 0; w < kCNW; ++w) t += ctrl->red[w];
      cluster.map_shared_rank(ctrl, tid)->part[par][rank] = t;
    }
    cluster.sync();
    float t = 0.f;
    for (int r = 0; r < kCW; ++r) t += ctrl->part[par][r];
    trail = t;
    if (t <= thr) {
      keff = j + 1;
      break;
    }
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
          tmp[u] = cluster.map_shared_rank(cols + (size_t)(x / kCW) * kw, x % kCW)[i];
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
  // Rotates the register rows u, v of this warp; true if it rotated.
  auto rotate_regs = [&](float4* u, float4* v) -> bool {
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
    const float a = warp_sum(a0 + a1), b = warp_sum(b0 + b1), gr = warp_sum(gr0 + gr1);
    float gi = 0.f;
    if constexpr (sizeof(F) != 4) gi = warp_sum(gi0 + gi1);
    const float g2 = fmaf(gr, gr, gi * gi);
    if (!(g2 > 0.f && g2 > tol2 * a * b)) return false;
    const float rg = rsqrtf(g2);
    const float zeta = 0.5f * (b - a) * rg;
    const float az = fabsf(zeta);
    const float tt =
        copysignf(az < 1e18f ? __frcp_rn(az + sqrtf(fmaf(az, az, 1.0f))) : 0.5f / az, zeta);
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
      if (br == 0 && sweep > 0 && rank == 0 && tid == 0) ctrl->flag[(sweep + 1) & 1] = 0;
    }
    const int rotated = ctrl0->flag[sweep & 1];
    if (!rotated) {
      status = 0;
      sweeps = sweep + 1;
      break;
    }
  }

  // ---- phase 4: rows back to global memory (FP64, rescaled) ------------------
  for (int j = warp; j < 2 * r; j += kCNW) {
    const int row = (j < r ? rank : 2 * kCW - 1 - rank) * r + (j % r);
    if (row >= kcap) continue;
    const F* src = Tb + (size_t)j * LP;  // Bb == Tb + blk: rows j >= r are the bottom block
    double acc = 0.0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int c = lane + 32 * e;
      if (c < l) {
        const T x = F32<T>::to(src[c], nrm);
        out_rows[(size_t)row * l + c] = x;
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
    info[0] = norm2;
    info[1] = (double)trail * norm2;
    info[5] = 1e-6 * (double)(t_qr - t_start);       // ms: load + QR
    info[6] = 1e-6 * (double)(global_ns() - t_qr);   // ms: gather + Jacobi + store
  }
  cluster.sync();  // no CTA leaves while another may still read its shared memory
}

template <typename T, int E>
bool cluster_config(int kw, int l, size_t* smem_out) {
  const size_t smem = cluster_smem<T, E>(kw, l);
  if (smem > 227 * 1024) return false;
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
                         double* out_nrm, int kcap, JacobiCtl* ctl, double* info, int qr_cap) {
  size_t smem = 0;
  if (!cluster_config<T, E>(kw, l, &smem)) {
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
                                   info, qr_cap));
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

template <typename T>
bool split_cluster_fits(int kw, int l) {
  if (std::min(kw, l) > kMaxRows || kw > 1024) return false;
  const int e = e_bucket(l);
  if (e == 0) return false;
  if (sizeof(T) != sizeof(double) && e > 16) return false;  // complex rows beyond 512 spill
  // Residency is checked once per (dtype, E): the answer does not depend on
  // the sizes beyond the shared-memory amount, which is re-checked below.
  size_t smem = 0;
  switch (e) {
    case 4: return cluster_config<T, 4>(kw, l, &smem);
    case 8: return cluster_config<T, 8>(kw, l, &smem);
    case 12: return cluster_config<T, 12>(kw, l, &smem);
    case 16: return cluster_config<T, 16>(kw, l, &smem);
    default: return cluster_config<T, 24>(kw, l, &smem);
  }
}

template <typename T>
int split_cluster_f32(cudaStream_t st, const T* A, int m, int n, bool want_u, double thr_rel,
                      double thr_abs, int max_sweeps, T* out_rows, double* out_nrm, int kcap,
                      JacobiCtl* ctl, double* info, int qr_cap) {
  // W = A^T (kw = n, l = m) when U is wanted, else W = A (kw = m, l = n)
  const int kw = want_u ? n : m;
  const int l = want_u ? m : n;
  const int trans = want_u ? 1 : 0;
  switch (e_bucket(l)) {
#define SM_C(EV)                                                                              \
  case EV:                                                                                    \
    return launch_split_cluster<T, EV>(st, A, n, trans, kw, l, thr_rel, thr_abs, max_sweeps, \
                                       out_rows, out_nrm, kcap, ctl, info, qr_cap)
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

template bool split_cluster_fits<double>(int, int);
template bool split_cluster_fits<cplx>(int, int);
template int split_cluster_f32<double>(cudaStream_t, const double*, int, int, bool, double,
                                       double, int, double*, double*, int, JacobiCtl*, double*,
                                       int);
template int split_cluster_f32<cplx>(cudaStream_t, const cplx*, int, int, bool, double, double,
                                     int, cplx*, double*, int, JacobiCtl*, double*, int);

}  // namespace sm
