// Minimal complex<T> used to compile the reference project's CUDA kernels
// outside CuPy (TEST INFRASTRUCTURE: only oracle/build_ref.py includes it).
//
// The reference kernels include <cupy/complex.cuh> (sources/cuda_kernels/
// common.cu:4) and use a small part of its interface: construction from one or
// two reals or from another complex type, real()/imag(), the arithmetic
// operators between complex values and between a complex and a real of the same
// type, compound assignment, unary minus and conj(). This header supplies
// exactly that, written from the definitions of complex arithmetic:
//   (a+ib)(c+id) = (ac-bd) + i(ad+bc),  s(a+ib) = sa + isb,  (a+ib)/s = a/s + ib/s.
// Mixed real types promote to the wider type, as C++'s usual arithmetic
// conversions do.
#pragma once

#include <type_traits>

template <typename T>
struct alignas(2 * sizeof(T)) complex {
    T re_;
    T im_;

    __host__ __device__ constexpr complex(const T& r = T(), const T& i = T()) : re_(r), im_(i) {}
    template <typename U>
    __host__ __device__ constexpr complex(const complex<U>& o) : re_(T(o.real())), im_(T(o.imag())) {}

    __host__ __device__ constexpr T real() const { return re_; }
    __host__ __device__ constexpr T imag() const { return im_; }
    __host__ __device__ void real(T r) { re_ = r; }
    __host__ __device__ void imag(T i) { im_ = i; }

    __host__ __device__ complex& operator+=(const complex& o) { re_ += o.re_; im_ += o.im_; return *this; }
    __host__ __device__ complex& operator-=(const complex& o) { re_ -= o.re_; im_ -= o.im_; return *this; }
    __host__ __device__ complex& operator*=(const complex& o)
    {
        const T r = re_ * o.re_ - im_ * o.im_;
        const T i = re_ * o.im_ + im_ * o.re_;
        re_ = r;
        im_ = i;
        return *this;
    }
    __host__ __device__ complex& operator+=(const T& s) { re_ += s; return *this; }
    __host__ __device__ complex& operator-=(const T& s) { re_ -= s; return *this; }
    __host__ __device__ complex& operator*=(const T& s) { re_ *= s; im_ *= s; return *this; }
    __host__ __device__ complex& operator/=(const T& s) { re_ /= s; im_ /= s; return *this; }
};

namespace wfs_ref_shim {
template <typename A, typename B>
struct wider { using type = decltype(A() + B()); };
template <typename S>
using real_only = typename std::enable_if<std::is_arithmetic<S>::value, int>::type;
}  // namespace wfs_ref_shim

template <typename A, typename B>
__host__ __device__ inline complex<typename wfs_ref_shim::wider<A, B>::type>
operator+(const complex<A>& a, const complex<B>& b)
{
    using T = typename wfs_ref_shim::wider<A, B>::type;
    return complex<T>(T(a.real()) + T(b.real()), T(a.imag()) + T(b.imag()));
}

template <typename A, typename B>
__host__ __device__ inline complex<typename wfs_ref_shim::wider<A, B>::type>
operator-(const complex<A>& a, const complex<B>& b)
{
    using T = typename wfs_ref_shim::wider<A, B>::type;
    return complex<T>(T(a.real()) - T(b.real()), T(a.imag()) - T(b.imag()));
}

template <typename A, typename B>
__host__ __device__ inline complex<typename wfs_ref_shim::wider<A, B>::type>
operator*(const complex<A>& a, const complex<B>& b)
{
    using T = typename wfs_ref_shim::wider<A, B>::type;
    const T ar = a.real(), ai = a.imag(), br = b.real(), bi = b.imag();
    return complex<T>(ar * br - ai * bi, ar * bi + ai * br);
}

template <typename A, typename B, wfs_ref_shim::real_only<B> = 0>
__host__ __device__ inline complex<typename wfs_ref_shim::wider<A, B>::type>
operator*(const complex<A>& a, const B& s)
{
    using T = typename wfs_ref_shim::wider<A, B>::type;
    return complex<T>(T(a.real()) * T(s), T(a.imag()) * T(s));
}

template <typename A, typename B, wfs_ref_shim::real_only<A> = 0>
__host__ __device__ inline complex<typename wfs_ref_shim::wider<A, B>::type>
operator*(const A& s, const complex<B>& a)
{
    using T = typename wfs_ref_shim::wider<A, B>::type;
    return complex<T>(T(s) * T(a.real()), T(s) * T(a.imag()));
}

template <typename A, typename B, wfs_ref_shim::real_only<B> = 0>
__host__ __device__ inline complex<typename wfs_ref_shim::wider<A, B>::type>
operator/(const complex<A>& a, const B& s)
{
    using T = typename wfs_ref_shim::wider<A, B>::type;
    return complex<T>(T(a.real()) / T(s), T(a.imag()) / T(s));
}

template <typename A, typename B, wfs_ref_shim::real_only<B> = 0>
__host__ __device__ inline complex<typename wfs_ref_shim::wider<A, B>::type>
operator+(const complex<A>& a, const B& s)
{
    using T = typename wfs_ref_shim::wider<A, B>::type;
    return complex<T>(T(a.real()) + T(s), T(a.imag()));
}

template <typename A, typename B, wfs_ref_shim::real_only<B> = 0>
__host__ __device__ inline complex<typename wfs_ref_shim::wider<A, B>::type>
operator-(const complex<A>& a, const B& s)
{
    using T = typename wfs_ref_shim::wider<A, B>::type;
    return complex<T>(T(a.real()) - T(s), T(a.imag()));
}

template <typename T>
__host__ __device__ inline complex<T> operator-(const complex<T>& a)
{
    return complex<T>(-a.real(), -a.imag());
}

template <typename T>
__host__ __device__ inline complex<T> operator+(const complex<T>& a)
{
    return a;
}

template <typename T>
__host__ __device__ inline complex<T> conj(const complex<T>& a)
{
    return complex<T>(a.real(), -a.imag());
}
