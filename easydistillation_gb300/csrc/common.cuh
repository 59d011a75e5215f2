// Shared device/host helpers for the GB300 distillation library.
//
// Layouts used by every kernel (V3 = Lx*Ly*Lz, site = x + Lx*(y + Ly*z)):
//   links  : per timeslice [dir 3][row 3][col 3][V3] complex   ("SoA links")
//   vectors: per vector    [colour 3][V3] complex                ("colour planes")
// Complex numbers are stored as (re, im) pairs: double2 for c128, float2 for c64.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/easydist_gb300.h"

namespace ed {

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* what);

#define ED_CHECK_ARG(cond, ...)          \
  do {                                   \
    if (!(cond)) {                       \
      ::ed::set_error(__VA_ARGS__);      \
      return ED_ERR_ARG;                 \
    }                                    \
  } while (0)

#define ED_RETURN_LAUNCH(what)                                   \
  do {                                                           \
    cudaError_t _e = cudaGetLastError();                         \
    if (_e != cudaSuccess) return ::ed::cuda_status(_e, what);   \
  } while (0)

// ---------------------------------------------------------------- complex
template <typename T>
struct cplx {
  T re, im;
};

template <typename T>
__host__ __device__ __forceinline__ cplx<T> mk(T r, T i) {
  cplx<T> c;
  c.re = r;
  c.im = i;
  return c;
}
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) {
  return mk(a.re + b.re, a.im + b.im);
}
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) {
  return mk(a.re - b.re, a.im - b.im);
}
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator*(cplx<T> a, cplx<T> b) {
  return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
// conj(a) * b
template <typename T>
__host__ __device__ __forceinline__ cplx<T> cmul_conj(cplx<T> a, cplx<T> b) {
  return mk(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re);
}
// acc += a * b
template <typename T>
__host__ __device__ __forceinline__ void cfma(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fma(a.re, b.re, acc.re);
  acc.re = fma(-a.im, b.im, acc.re);
  acc.im = fma(a.re, b.im, acc.im);
  acc.im = fma(a.im, b.re, acc.im);
}
// acc += conj(a) * b
template <typename T>
__host__ __device__ __forceinline__ void cfma_conj(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fma(a.re, b.re, acc.re);
  acc.re = fma(a.im, b.im, acc.re);
  acc.im = fma(a.re, b.im, acc.im);
  acc.im = fma(-a.im, b.re, acc.im);
}

template <typename T>
__device__ __forceinline__ cplx<T> ld(const cplx<T>* p);
template <>
__device__ __forceinline__ cplx<double> ld(const cplx<double>* p) {
  double2 v = __ldg(reinterpret_cast<const double2*>(p));
  return mk(v.x, v.y);
}
template <>
__device__ __forceinline__ cplx<float> ld(const cplx<float>* p) {
  float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return mk(v.x, v.y);
}
template <typename T>
__device__ __forceinline__ void st(cplx<T>* p, cplx<T> v) {
  *p = v;
}

// convert between storage precisions
template <typename D, typename S>
__host__ __device__ __forceinline__ cplx<D> cvt(cplx<S> a) {
  return mk((D)a.re, (D)a.im);
}

// ---------------------------------------------------------------- lattice
struct Latt {
  int Lx, Ly, Lz;
  __host__ __device__ int V3() const { return Lx * Ly * Lz; }
};

// Largest spatial volume the entry points accept: kernels number sites and
// colour-plane entries (3 * V3) with 32-bit integers.
constexpr long long MAX_V3 = 1LL << 28;
inline bool lattice_ok(int Lx, int Ly, int Lz) {
  return Lx > 0 && Ly > 0 && Lz > 0 && (long long)Lx * Ly * Lz <= MAX_V3;
}

__host__ __device__ __forceinline__ int wrap_inc(int v, int L) { return v + 1 == L ? 0 : v + 1; }
__host__ __device__ __forceinline__ int wrap_dec(int v, int L) { return v == 0 ? L - 1 : v - 1; }

inline int num_sms() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace ed
