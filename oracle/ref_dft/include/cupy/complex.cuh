// Minimal complex<T> with the operations the reference's DFT kernel uses
// (construction from (re, im) or a scalar, +=, complex * complex).  Written
// for this project as a stand-in for CuPy's header, which is not installed.
#pragma once

template <typename T>
struct complex {
  T re, im;
  __host__ __device__ complex() : re(0), im(0) {}
  __host__ __device__ complex(T r) : re(r), im(0) {}
  __host__ __device__ complex(T r, T i) : re(r), im(i) {}
  __host__ __device__ complex &operator=(T r) {
    re = r;
    im = 0;
    return *this;
  }
  __host__ __device__ complex &operator+=(const complex &o) {
    re += o.re;
    im += o.im;
    return *this;
  }
};

template <typename T>
__host__ __device__ inline complex<T> operator*(const complex<T> &a, const complex<T> &b) {
  return complex<T>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
