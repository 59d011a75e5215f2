// Minimal stand-in for CuPy's <cupy/complex.cuh> (test infrastructure).
//
// The reference's CUDA stout-smearing kernel (lattice/generator/stout_smear.cu)
// is written for CuPy's RawModule and includes CuPy's complex header, which is
// not installed here.  This header supplies the complex<T> operations that
// kernel uses (construction from one or two reals, real()/imag() getters and
// setters, + - * / and their compound forms, conj) with the textbook formulas,
// so that nvcc can compile the reference kernel unmodified into a cubin that
// the tests and the benchmark launch beside the library's own kernel.
#pragma once

template <typename T>
struct complex {
  T re_, im_;
  __host__ __device__ complex(const T& re = T(0), const T& im = T(0)) : re_(re), im_(im) {}
  __host__ __device__ T real() const { return re_; }
  __host__ __device__ T imag() const { return im_; }
  __host__ __device__ void real(T v) { re_ = v; }
  __host__ __device__ void imag(T v) { im_ = v; }
  __host__ __device__ complex& operator+=(const complex& o) {
    re_ += o.re_;
    im_ += o.im_;
    return *this;
  }
  __host__ __device__ complex& operator-=(const complex& o) {
    re_ -= o.re_;
    im_ -= o.im_;
    return *this;
  }
  __host__ __device__ complex& operator*=(const complex& o) {
    *this = *this * o;
    return *this;
  }
  __host__ __device__ friend complex operator+(const complex& a, const complex& b) {
    return complex(a.re_ + b.re_, a.im_ + b.im_);
  }
  __host__ __device__ friend complex operator-(const complex& a, const complex& b) {
    return complex(a.re_ - b.re_, a.im_ - b.im_);
  }
  __host__ __device__ friend complex operator*(const complex& a, const complex& b) {
    return complex(a.re_ * b.re_ - a.im_ * b.im_, a.re_ * b.im_ + a.im_ * b.re_);
  }
  __host__ __device__ friend complex operator/(const complex& a, const complex& b) {
    const T d = b.re_ * b.re_ + b.im_ * b.im_;
    return complex((a.re_ * b.re_ + a.im_ * b.im_) / d, (a.im_ * b.re_ - a.re_ * b.im_) / d);
  }
};

template <typename T>
__host__ __device__ complex<T> conj(const complex<T>& a) {
  return complex<T>(a.real(), -a.imag());
}
