// common.cuh — device building blocks shared by the engine's kernels.
//
// * Cx<R>: complex value with 2*sizeof(R) alignment so a load/store is one
//   64-bit (complex64) or 128-bit (complex128) memory transaction.
// * root_of(m, n): exp(2*pi*i*m/n) evaluated at compile time from its
//   Taylor series after an exact octant reduction (plain mathematics; no
//   library math function is involved), so every twiddle inside a
//   register-resident DFT is an immediate constant.
// * dft<N, SIGN>: length-N DFT on an array held in registers, mixed radix
//   2/3/4, decimation in time. SIGN = -1 is numpy's forward transform
//   (exp(-2 pi i k n / N)), SIGN = +1 the inverse (unscaled).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>
#include <utility>

namespace wfs {

template <typename R>
struct alignas(2 * sizeof(R)) Cx {
    R x, y;
};

template <typename R>
__host__ __device__ __forceinline__ Cx<R> mk(R a, R b) { Cx<R> c; c.x = a; c.y = b; return c; }
template <typename R>
__device__ __forceinline__ Cx<R> operator+(Cx<R> a, Cx<R> b) { return mk<R>(a.x + b.x, a.y + b.y); }
template <typename R>
__device__ __forceinline__ Cx<R> operator-(Cx<R> a, Cx<R> b) { return mk<R>(a.x - b.x, a.y - b.y); }
#ifndef WFS_PACKED_F32
#define WFS_PACKED_F32 1
#endif
#if WFS_PACKED_F32
// complex64 add/sub as one packed FP32 pair instruction (sm_100+ __fadd2_rn);
// each component is rounded exactly like the scalar add. Packed multiplies were
// measured slower (the broadcast and swapped operand pairs cost more than the
// saved issue slots), so products stay scalar.
__device__ __forceinline__ Cx<float> operator+(Cx<float> a, Cx<float> b) {
    const float2 r = __fadd2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y));
    return mk<float>(r.x, r.y);
}
__device__ __forceinline__ Cx<float> operator-(Cx<float> a, Cx<float> b) {
    const float2 r = __fadd2_rn(make_float2(a.x, a.y), make_float2(-b.x, -b.y));
    return mk<float>(r.x, r.y);
}
#endif
template <typename R>
__device__ __forceinline__ Cx<R> cmul(Cx<R> a, Cx<R> b) {
    return mk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename R>
__device__ __forceinline__ Cx<R> cmulc(Cx<R> a, Cx<R> b) {  // a * conj(b)
    return mk<R>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename R>
__device__ __forceinline__ Cx<R> scale(Cx<R> a, R s) { return mk<R>(a.x * s, a.y * s); }
// multiply by SIGN * i
template <int SIGN, typename R>
__device__ __forceinline__ Cx<R> mul_si(Cx<R> a) {
    if constexpr (SIGN > 0) return mk<R>(-a.y, a.x);
    else return mk<R>(a.y, -a.x);
}

// ---------------------------------------------------------------------------
// Compile-time roots of unity
// ---------------------------------------------------------------------------
struct Root { double c, s; };

constexpr double kPi = 3.14159265358979323846264338327950288;

__host__ __device__ constexpr double taylor_sin(double x) {  // |x| <= pi/4
    double x2 = x * x, term = x, sum = x;
    for (int k = 1; k < 14; ++k) { term *= -x2 / double((2 * k) * (2 * k + 1)); sum += term; }
    return sum;
}
__host__ __device__ constexpr double taylor_cos(double x) {  // |x| <= pi/4
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 14; ++k) { term *= -x2 / double((2 * k - 1) * (2 * k)); sum += term; }
    return sum;
}
// exp(2 pi i m / n) for integers m, n > 0.
__host__ __device__ constexpr Root root_of(long m, long n) {
    m %= n;
    if (m < 0) m += n;
    long q = (4 * m) / n;          // quadrant
    long r = 4 * m - q * n;        // angle inside quadrant = (pi/2) * r / n
    double ca = 0.0, sa = 0.0;
    if (2 * r <= n) {
        double a = (kPi / 2.0) * double(r) / double(n);
        ca = taylor_cos(a); sa = taylor_sin(a);
    } else {
        double b = (kPi / 2.0) * double(n - r) / double(n);
        ca = taylor_sin(b); sa = taylor_cos(b);
    }
    Root out{ca, sa};
    switch (q & 3) {
        case 0: out = Root{ca, sa}; break;
        case 1: out = Root{-sa, ca}; break;
        case 2: out = Root{-ca, -sa}; break;
        default: out = Root{sa, -ca}; break;
    }
    return out;
}

// ---------------------------------------------------------------------------
// Compile-time loops
// ---------------------------------------------------------------------------
template <int I>
using ic = std::integral_constant<int, I>;

template <typename F, int... Is>
__device__ __forceinline__ void sfor_impl(F&& f, std::integer_sequence<int, Is...>) {
    (f(ic<Is>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void sfor(F&& f) {
    sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// multiply by the compile-time twiddle exp(SIGN * 2 pi i * M / N)
template <int SIGN, int M, int N, typename R>
__device__ __forceinline__ Cx<R> twiddle_const(Cx<R> a) {
    constexpr int m = ((M % N) + N) % N;
    if constexpr (m == 0) {
        return a;
    } else if constexpr (4 * m == N) {            // SIGN * i
        return mul_si<SIGN>(a);
    } else if constexpr (2 * m == N) {            // -1
        return mk<R>(-a.x, -a.y);
    } else if constexpr (4 * m == 3 * N) {        // -SIGN * i
        return mul_si<-SIGN>(a);
    } else {
        constexpr Root w = root_of(long(SIGN) * m, N);
        return cmul(a, mk<R>(R(w.c), R(w.s)));
    }
}

// ---------------------------------------------------------------------------
// Register-resident DFT
// ---------------------------------------------------------------------------
template <int N, int SIGN, typename R>
__device__ __forceinline__ void dft(Cx<R> (&v)[N]);

template <int SIGN, typename R>
__device__ __forceinline__ void dft2(Cx<R>& a, Cx<R>& b) {
    Cx<R> t = a;
    a = t + b;
    b = t - b;
}

template <int N, int SIGN, typename R>
__device__ __forceinline__ void dft(Cx<R> (&v)[N]) {
    if constexpr (N == 1) {
        return;
    } else if constexpr (N == 2) {
        dft2<SIGN>(v[0], v[1]);
    } else if constexpr (N == 3) {
        constexpr R s3 = R(0.86602540378443864676372317075293618);  // sqrt(3)/2
        Cx<R> a = v[0], b = v[1], c = v[2];
        Cx<R> t1 = b + c;
        Cx<R> t2 = mk<R>(a.x - R(0.5) * t1.x, a.y - R(0.5) * t1.y);
        Cx<R> d = b - c;
        // i * SIGN * s3 * d
        Cx<R> t3 = mul_si<SIGN>(mk<R>(s3 * d.x, s3 * d.y));
        v[0] = a + t1;
        v[1] = t2 + t3;
        v[2] = t2 - t3;
    } else if constexpr (N == 4) {
        Cx<R> a = v[0], b = v[1], c = v[2], d = v[3];
        // s3 = SIGN * i * (b - d), formed directly in rotated order from scalar
        // differences so the four outputs are packed adds of aligned pairs
        Cx<R> s0 = a + c, s1 = a - c, s2 = b + d;
        Cx<R> s3 = (SIGN > 0) ? mk<R>(d.y - b.y, b.x - d.x) : mk<R>(b.y - d.y, d.x - b.x);
        v[0] = s0 + s2;
        v[1] = s1 + s3;
        v[2] = s0 - s2;
        v[3] = s1 - s3;
    } else {
        constexpr int F = (N % 4 == 0) ? 4 : ((N % 2 == 0) ? 2 : 3);
        constexpr int M = N / F;
        static_assert(F * M == N, "unsupported DFT length");
        Cx<R> sub[F][M];
        sfor<F>([&](auto J) {
            constexpr int j = decltype(J)::value;
            sfor<M>([&](auto Mi) {
                constexpr int m = decltype(Mi)::value;
                sub[j][m] = v[F * m + j];
            });
            dft<M, SIGN, R>(sub[j]);
            sfor<M>([&](auto K) {
                constexpr int k = decltype(K)::value;
                sub[j][k] = twiddle_const<SIGN, j * k, N>(sub[j][k]);
            });
        });
        sfor<M>([&](auto K) {
            constexpr int k = decltype(K)::value;
            Cx<R> t[F];
            sfor<F>([&](auto J) { t[decltype(J)::value] = sub[decltype(J)::value][k]; });
            dft<F, SIGN, R>(t);
            sfor<F>([&](auto Qi) { v[k + M * decltype(Qi)::value] = t[decltype(Qi)::value]; });
        });
    }
}

__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }

}  // namespace wfs
