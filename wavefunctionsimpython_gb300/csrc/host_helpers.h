// host_helpers.h — host-side pieces shared by the single-grid engine and the batch engine.
#pragma once

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/wfs.h"
#include "kernels.h"

namespace wfs {

// Per-axis envelope g_d(i) and coordinate r_d(i) of the Gaussian packet
// (common.cu:569-586, gaussian_wave_packet.cu:36-40), computed in the
// working precision with the reference's operation order; the device kernel
// multiplies them per voxel.
template <typename R>
inline void gaussian_axes(const int n[3], const double dx[3], const double sigma[3], const double r0[3],
                          std::vector<R>& g, std::vector<R>& r) {
    const int total = n[0] + n[1] + n[2];
    g.assign(total, R(0));
    r.assign(total, R(0));
    const int off[3] = {0, n[0], n[0] + n[1]};
    for (int a = 0; a < 3; ++a) {
        for (int i = 0; i < n[a]; ++i) {
            const int iv = i - n[a] / 2;
            if (sizeof(R) == 8) {
                const double rr = dx[a] * double(iv);
                const double aa = 2.0 * sigma[a];
                const double norm = std::pow(2.0 / M_PI / aa / aa, 0.25);
                const double d = rr - r0[a];
                g[off[a] + i] = R(norm * std::exp(-d * d / aa / aa));
                r[off[a] + i] = R(rr);
            } else {
                volatile float rr = float(dx[a]) * float(iv);
                const float aa = 2.0f * float(sigma[a]);
                volatile float q = 2.0f / float(M_PI);
                q = q / aa;
                q = q / aa;
                const float norm = std::pow(float(q), 0.25f);
                volatile float d = float(rr) - float(r0[a]);
                volatile float ex = -float(d) * float(d);
                ex = ex / aa;
                ex = ex / aa;
                volatile float gg = norm * std::exp(float(ex));
                g[off[a] + i] = R(float(gg));
                r[off[a] + i] = R(float(rr));
            }
        }
    }
}

// Wall parameters for the device (potential_wall.cu:4-83). The normal is
// normalised in double precision and rounded to float32, as the reference does
// on the host (sources/potential.py:180); the wall's frame (up, right, the slit
// rotation) is formed by each thread of wall_kernel in the reference's float32
// device arithmetic.
inline bool wall_frame(const wfs_wall* w, WallDev& wd) {
    const double nn = std::sqrt(w->normal[0] * w->normal[0] + w->normal[1] * w->normal[1] + w->normal[2] * w->normal[2]);
    if (!(nn > 0) || !std::isfinite(nn) || !std::isfinite(w->slit_rotation)) return false;
    wd.U = float(w->potential_hartree);
    wd.cx = float(w->center[0]); wd.cy = float(w->center[1]); wd.cz = float(w->center[2]);
    wd.nx = float(w->normal[0] / nn); wd.ny = float(w->normal[1] / nn); wd.nz = float(w->normal[2] / nn);
    wd.rot = float(w->slit_rotation);
    wd.plateau = float(w->plateau_thickness);
    wd.slope = float(w->slope_thickness);
    wd.slope_exp = float(w->slope_exponent);
    wd.slit_count = w->slit_count < 0 ? 0 : (w->slit_count > 4 ? 4 : w->slit_count);
    wd.slit_spacing = float(w->slit_spacing);
    wd.slit_width = float(w->slit_width);
    return true;
}

// Frame of a sampling plane (probability_current_density.cu:41-49), float32 with
// every product and sum rounded: prefUp = (0,1,0), or (0,0,1) when |n.y| > 0.99;
// right = normalize(n x prefUp); up = normalize(right x n).
inline bool plane_frame(const double normal[3], float n[3], float right[3], float up[3]) {
    const double nn = std::sqrt(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2]);
    if (!(nn > 0)) return false;
    auto mul = [](float a, float b) { volatile float r = a * b; return float(r); };
    auto add = [](float a, float b) { volatile float r = a + b; return float(r); };
    auto sub = [](float a, float b) { volatile float r = a - b; return float(r); };
    for (int i = 0; i < 3; ++i) n[i] = float(normal[i] / nn);
    float pu[3] = {0.f, 1.f, 0.f};
    if (std::fabs(add(add(mul(n[0], pu[0]), mul(n[1], pu[1])), mul(n[2], pu[2]))) > 0.99f) { pu[1] = 0.f; pu[2] = 1.f; }
    auto cross = [&](const float* a, const float* b, float* o) {
        o[0] = sub(mul(a[1], b[2]), mul(a[2], b[1]));
        o[1] = sub(mul(a[2], b[0]), mul(a[0], b[2]));
        o[2] = sub(mul(a[0], b[1]), mul(a[1], b[0]));
    };
    auto normalize = [&](float* a) -> bool {
        const float d = add(add(mul(a[0], a[0]), mul(a[1], a[1])), mul(a[2], a[2]));
        const float l = float(std::sqrt(double(d)));
        if (!(l > 0)) return false;
        for (int i = 0; i < 3; ++i) { volatile float r = a[i] / l; a[i] = r; }
        return true;
    };
    cross(n, pu, right);
    if (!normalize(right)) return false;
    cross(right, n, up);
    return normalize(up);
}

inline AbsorbDev absorbing_dev(const wfs_absorbing* a) {
    AbsorbDev ad;
    for (int i = 0; i < 3; ++i) {
        ad.bottom[i] = float(a->bottom[i]);
        ad.top[i] = float(a->top[i]);
        ad.pp[i] = float(a->potential_pos[i]);
        ad.pn[i] = float(a->potential_neg[i]);
        ad.ep[i] = float(a->exponent_pos[i]);
        ad.en[i] = float(a->exponent_neg[i]);
    }
    ad.offset = float(a->offset);
    return ad;
}

// amp * exp(-i k^2 dt frac / m) for k = 2 pi fftfreq(L, dx), rounded to precision R.
template <typename R>
inline void kinetic_axis(int L, double dx, double dt, double mass, double frac, Cx<R>* out, double amp = 1.0) {
    for (int i = 0; i < L; ++i) {
        const int fi = (i < (L + 1) / 2) ? i : i - L;
        const double k = 2.0 * M_PI * double(fi) / (double(L) * dx);
        const double ang = -k * k * dt * frac / mass;
        out[i] = mk<R>(R(amp * std::cos(ang)), R(amp * std::sin(ang)));
    }
}

// Twiddle table of a length-L axis in both orders two_stage reads (3L entries):
// [0, L) out[m] = exp(-2 pi i m / L); [L, 2L) the (P, Q) plan's rows
// out[L + t*Q + k2] = exp(-2 pi i t k2 / L) (t < P, k2 < Q); [2L, 3L) the transposed
// (Q, P) plan's rows. False for unsupported L.
template <typename R>
inline bool two_stage_roots(int L, Cx<R>* out) {
    int P = 0, Q = 0;
    if (!plan_pq(L, P, Q)) return false;
    auto root = [&](int m) {
        const double a = -2.0 * 3.14159265358979323846 * double(m % L) / double(L);
        return mk<R>(R(std::cos(a)), R(std::sin(a)));
    };
    for (int m = 0; m < L; ++m) out[m] = root(m);
    for (int t = 0; t < P; ++t)
        for (int k = 0; k < Q; ++k) out[L + t * Q + k] = root(t * k);
    for (int t = 0; t < Q; ++t)
        for (int k = 0; k < P; ++k) out[2 * L + t * P + k] = root(t * k);
    return true;
}

// ---------------------------------------------------------------------------
// Mean energy gain of the transforms as built from working-precision constants.
//
// The butterflies multiply by roots of unity rounded to R, and a rounded root is
// not exactly of modulus 1: in complex64, cos(pi/8), sin(pi/8) and sqrt(1/2) all
// round to a slightly shorter root (|w|^2 - 1 = -5.7e-8 and -3.4e-8). Every
// element meets these same constants in every transform, so the norm of a
// complex64 run drifts by a fixed fraction per step (about -3.2e-7 per step at
// 256^3) instead of random-walking. These functions compute the mean gain
// trace(M^H M) / N^2 of each transform from the very constants the kernels use
// (compile-time roots of common.cuh, the uploaded twiddle tables, the rounded
// scale factors), assuming uncorrelated data between stages; the engine folds
// the inverse into its kinetic tables.
// ---------------------------------------------------------------------------
template <typename R>
inline double rounded_norm2(double c, double s) {
    const double cr = double(R(c)), sr = double(R(s));
    return cr * cr + sr * sr;
}
// |w|^2 of exp(2 pi i m / n) as twiddle_const applies it (multiples of n/4 are exact).
template <typename R>
inline double const_root_norm2(long m, long n) {
    m %= n;
    if (m < 0) m += n;
    if (m == 0 || 4 * m == n || 2 * m == n || 4 * m == 3 * n) return 1.0;
    const Root w = root_of(m, n);
    return rounded_norm2<R>(w.c, w.s);
}
// Mean energy gain of dft<N> (unnormalised DFT divided by N), following its
// F x M decomposition in common.cuh.
template <typename R>
inline double dft_gain(int N) {
    if (N <= 2 || N == 4) return 1.0;
    if (N == 3) {
        const double s3 = double(R(0.86602540378443864676372317075293618));
        return (6.0 + 4.0 * s3 * s3) / 9.0;
    }
    const int F = (N % 4 == 0) ? 4 : ((N % 2 == 0) ? 2 : 3);
    const int M = N / F;
    double tw = 0.0;
    for (int j = 0; j < F; ++j)
        for (int k = 0; k < M; ++k) tw += const_root_norm2<R>(long(j) * k, N);
    return dft_gain<R>(M) * (tw / double(F * M)) * dft_gain<R>(F);
}
// Mean energy gain of one two-stage transform of length L, without its scale factor.
template <typename R>
inline double fft_gain(int L) {
    int P = 0, Q = 0;
    if (!plan_pq(L, P, Q)) return 1.0;
    double tw = 0.0;
    for (int t = 0; t < P; ++t)
        for (int k = 0; k < Q; ++k) {
            const double a = -2.0 * 3.14159265358979323846 * double((t * k) % L) / double(L);
            tw += rounded_norm2<R>(std::cos(a), std::sin(a));
        }
    return dft_gain<R>(Q) * (tw / double(P * Q)) * dft_gain<R>(P);
}
// Energy gain of one split step's transforms: the x pass (two x transforms, scale 1/nx
// once) and the y/z work (two y transforms scaled by 1/sqrt(ny) each, two z transforms
// scaled by 1/nz once), identical in the fused plane pass and the per-axis passes.
template <typename R>
inline void split_step_gains(const int n[3], double* g_x, double* g_yz) {
    const double sx = double(R(1.0 / double(n[0])));
    const double sy = double(R(1.0 / std::sqrt(double(n[1]))));
    const double sz = double(R(1.0 / double(n[2])));
    const double gx = fft_gain<R>(n[0]), gy = fft_gain<R>(n[1]), gz = fft_gain<R>(n[2]);
    *g_x = gx * gx * (n[0] * sx) * (n[0] * sx);
    const double gys = gy * n[1] * sy * sy;
    *g_yz = gys * gys * gz * gz * (n[2] * sz) * (n[2] * sz);
}

}  // namespace wfs
