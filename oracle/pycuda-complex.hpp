// Minimal device complex type standing in for pycuda's pycuda-complex.hpp --
// TEST INFRASTRUCTURE ONLY.
//
// The reference's kernel templates (namsa/probe_kernels.cu, namsa/potential_kernels.cu)
// include <pycuda-complex.hpp> and use only: the members _M_re/_M_im, construction
// from (re, im) or from a real, complex *= complex, complex *= real, complex * real,
// complex / real, complex /= real and pycuda::norm (squared magnitude).  This header
// supplies exactly those operations with the textbook formulas, so the rendered
// kernels compile with nvcc for the reference-GPU harness in oracle/refgpu_harness.cu.
#pragma once

namespace pycuda {

template <class T>
struct complex {
  T _M_re, _M_im;
  __host__ __device__ complex(T re = T(), T im = T()) : _M_re(re), _M_im(im) {}
  __host__ __device__ complex& operator*=(const complex& z) {
    const T re = _M_re * z._M_re - _M_im * z._M_im;
    const T im = _M_re * z._M_im + _M_im * z._M_re;
    _M_re = re;
    _M_im = im;
    return *this;
  }
  __host__ __device__ complex& operator*=(T s) {
    _M_re *= s;
    _M_im *= s;
    return *this;
  }
  __host__ __device__ complex& operator/=(T s) {
    _M_re /= s;
    _M_im /= s;
    return *this;
  }
};

template <class T>
__host__ __device__ complex<T> operator*(complex<T> a, T s) {
  a *= s;
  return a;
}

template <class T>
__host__ __device__ complex<T> operator/(complex<T> a, T s) {
  a /= s;
  return a;
}

template <class T>
__host__ __device__ T norm(const complex<T>& z) {
  return z._M_re * z._M_re + z._M_im * z._M_im;
}

}  // namespace pycuda
