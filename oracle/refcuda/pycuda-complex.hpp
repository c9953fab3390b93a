// Minimal stand-in for pycuda's complex header, written for this project.
//
// TEST INFRASTRUCTURE ONLY: used by oracle/ref_build.py to compile the
// reference's own CUDA kernels (svirl/cuda/*.h) into the checker under
// oracle/_ref/.  pycuda (a third-party dependency, `pycuda>=2018.1` in the
// reference's setup.py, unpinned) is absent here; its header supplies a
// `pycuda::complex<T>` with the textbook arithmetic below.  The reference's
// kernels use: construction from (re, im) or from a real, real(), imag(),
// + - * with complex and real operands, division by a real, +=, conj() and
// abs() (svirl/cuda/common.h:28-73, td.h:4-133,295-307, cg.h:305-731).
//
// pycuda compiles the reference inside `extern "C" { ... }` (its
// SourceModule default), so the templates sit in an `extern "C++"` block.
#pragma once

extern "C++" {
namespace pycuda {

// Aligned to its size, like CUDA's float2/double2, so an element is loaded and
// stored as one access.  This matters for the reference's phase-lock kernel
// (svirl/cuda/td.h:295-307): its lock list can name a node several times (the
// reference builds it with np.where(...)[0] of a 2-D grid), so threads of
// different blocks rewrite the same element; with two 8-byte halves one thread
// can read the other's half-written element and store hypot(|psi|, old imag).
template <typename T>
struct alignas(2 * sizeof(T)) complex {
    T re_, im_;  // interleaved (re, im): the layout of the host's complex64/complex128

    __host__ __device__ complex() : re_(T(0)), im_(T(0)) {}
    __host__ __device__ complex(const T &re) : re_(re), im_(T(0)) {}
    __host__ __device__ complex(const T &re, const T &im) : re_(re), im_(im) {}
    template <typename U>
    __host__ __device__ complex(const complex<U> &z) : re_(T(z.real())), im_(T(z.imag())) {}

    __host__ __device__ T real() const { return re_; }
    __host__ __device__ T imag() const { return im_; }

    __host__ __device__ complex &operator+=(const complex &z) { re_ += z.re_; im_ += z.im_; return *this; }
    __host__ __device__ complex &operator-=(const complex &z) { re_ -= z.re_; im_ -= z.im_; return *this; }
    __host__ __device__ complex &operator*=(const complex &z) {
        T r = re_ * z.re_ - im_ * z.im_;
        T i = re_ * z.im_ + im_ * z.re_;
        re_ = r; im_ = i;
        return *this;
    }
    __host__ __device__ complex &operator*=(const T &s) { re_ *= s; im_ *= s; return *this; }
    __host__ __device__ complex &operator/=(const T &s) { re_ /= s; im_ /= s; return *this; }
};

template <typename T>
__host__ __device__ inline complex<T> operator+(const complex<T> &a, const complex<T> &b) {
    return complex<T>(a.real() + b.real(), a.imag() + b.imag());
}
template <typename T>
__host__ __device__ inline complex<T> operator-(const complex<T> &a, const complex<T> &b) {
    return complex<T>(a.real() - b.real(), a.imag() - b.imag());
}
template <typename T>
__host__ __device__ inline complex<T> operator-(const complex<T> &a) {
    return complex<T>(-a.real(), -a.imag());
}
template <typename T>
__host__ __device__ inline complex<T> operator*(const complex<T> &a, const complex<T> &b) {
    return complex<T>(a.real() * b.real() - a.imag() * b.imag(),
                      a.real() * b.imag() + a.imag() * b.real());
}
template <typename T>
__host__ __device__ inline complex<T> operator*(const complex<T> &a, const T &s) {
    return complex<T>(a.real() * s, a.imag() * s);
}
template <typename T>
__host__ __device__ inline complex<T> operator*(const T &s, const complex<T> &a) {
    return complex<T>(s * a.real(), s * a.imag());
}
template <typename T>
__host__ __device__ inline complex<T> operator/(const complex<T> &a, const T &s) {
    return complex<T>(a.real() / s, a.imag() / s);
}
template <typename T>
__host__ __device__ inline complex<T> conj(const complex<T> &a) {
    return complex<T>(a.real(), -a.imag());
}
template <typename T>
__host__ __device__ inline T abs(const complex<T> &a) {
    return hypot(a.real(), a.imag());
}

}  // namespace pycuda
}  // extern "C++"
