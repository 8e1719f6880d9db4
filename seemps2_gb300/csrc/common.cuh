// Shared definitions for the sm_103a kernels of seemps2_gb300.
//
// Scalar types: `double` (float64) and `cplx` (complex128, interleaved re/im,
// the same bytes as numpy/torch complex128).  Every kernel is a template over
// these two types so that real and complex states share one code path.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/seemps_gb300.h"

namespace sm {

struct cplx {
  double re, im;
};

__host__ __device__ inline cplx mk(double r, double i) { return cplx{r, i}; }
__host__ __device__ inline cplx operator+(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ inline cplx operator-(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ inline cplx operator*(cplx a, cplx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__host__ __device__ inline cplx operator*(double s, cplx a) { return {s * a.re, s * a.im}; }
__host__ __device__ inline cplx operator*(cplx a, double s) { return {s * a.re, s * a.im}; }
__host__ __device__ inline cplx& operator+=(cplx& a, cplx b) { a.re += b.re; a.im += b.im; return a; }

// Generic helpers so templates read the same for both types.
template <typename T> struct S;
template <> struct S<double> {
  static constexpr int kDtype = SM_FLOAT64;
  __host__ __device__ static double zero() { return 0.0; }
  __host__ __device__ static double one() { return 1.0; }
  __host__ __device__ static double conj(double a) { return a; }
  __host__ __device__ static double abs2(double a) { return a * a; }
  __host__ __device__ static double real(double a) { return a; }
  __host__ __device__ static double fma(double a, double b, double c) { return ::fma(a, b, c); }
  // c + conj(a) * b
  __host__ __device__ static double cfma(double a, double b, double c) { return ::fma(a, b, c); }
  __host__ __device__ static double scale(double a, double s) { return a * s; }
  __host__ __device__ static double from_real(double a) { return a; }
  __host__ __device__ static double neg(double a) { return -a; }
};
template <> struct S<cplx> {
  static constexpr int kDtype = SM_COMPLEX128;
  __host__ __device__ static cplx zero() { return {0.0, 0.0}; }
  __host__ __device__ static cplx one() { return {1.0, 0.0}; }
  __host__ __device__ static cplx conj(cplx a) { return {a.re, -a.im}; }
  __host__ __device__ static double abs2(cplx a) { return a.re * a.re + a.im * a.im; }
  __host__ __device__ static double real(cplx a) { return a.re; }
  __host__ __device__ static cplx fma(cplx a, cplx b, cplx c) {
    return {::fma(a.re, b.re, ::fma(-a.im, b.im, c.re)), ::fma(a.re, b.im, ::fma(a.im, b.re, c.im))};
  }
  __host__ __device__ static cplx cfma(cplx a, cplx b, cplx c) {
    return {::fma(a.re, b.re, ::fma(a.im, b.im, c.re)), ::fma(a.re, b.im, ::fma(-a.im, b.re, c.im))};
  }
  __host__ __device__ static cplx scale(cplx a, double s) { return {a.re * s, a.im * s}; }
  __host__ __device__ static cplx from_real(double a) { return {a, 0.0}; }
  __host__ __device__ static cplx neg(cplx a) { return {-a.re, -a.im}; }
};

// ---------------------------------------------------------------------------
// Error reporting
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
const char* last_error();

#define SM_CUDA_CHECK(expr)                                                        \
  do {                                                                             \
    cudaError_t _e = (expr);                                                       \
    if (_e != cudaSuccess) {                                                       \
      ::sm::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));         \
      return SM_ERR_CUDA;                                                          \
    }                                                                              \
  } while (0)

#define SM_CHECK(expr)                  \
  do {                                  \
    int _s = (expr);                    \
    if (_s != SM_OK) return _s;         \
  } while (0)

// Status words written by kernels into device memory (bit flags).
enum DevStatus : int {
  DEV_OK = 0,
  DEV_BARRIER_TIMEOUT = 1,
  DEV_NOT_CONVERGED = 2,
  DEV_NONFINITE = 4,
};

// Bounded spin limit for every device-side wait (about a second with backoff).
constexpr long long kSpinLimit = 1LL << 23;

}  // namespace sm
