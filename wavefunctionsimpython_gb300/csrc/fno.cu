// fno.cu — kernels of the Fourier-neural-operator surrogate (forward, backward,
// optimiser, loss). Interface and layouts: include/wfs_fno.h.
//
// Network (width C, modes m per axis, grid N^3, batch B), all activations in the
// packed layout [B][channels/2][N^3] complex64:
//   h0  = W0 x + b0                               x = (Re psi, Im psi, V / vscale, 0)
//   h_{l+1} = act(W_l h_l + b_l + S_l(h_l))       l < L; act = GELU except on the last layer
//   out = W_q2 GELU(W_q1 h_L + b_q1) + b_q2 + prior
//
// Spectral layer S (wfs_fno.h): two real channels share one complex FFT
// (Y = F(h_a + i h_b)); the gather separates them with Hermitian symmetry
// (A(k) = (Y(k) + conj Y(-k)) / 2, B(k) = (Y(k) - conj Y(-k)) / 2i) and the
// scatter writes the symmetrised spectrum whose inverse carries Re F^-1(Z_a) in
// its real part and Re F^-1(Z_b) in its imaginary part, which halves the FFT
// work of a real-valued FNO on a complex FFT. Per mode, the channel mixing
// Z = H R is the real product [Hr | Hi] [[Rr, Ri], [-Ri, Rr]] on BF16 tensor cores
// (mma.sync m16n8k16, FP32 accumulation); the adjoint G_H = G_Z R^H uses the
// transposed block matrix. Everything else runs in FP32 with FP64 only in the
// final cross-block sums.
#include <cuda_bf16.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/wfs.h"
#include "../../include/wfs_fno.h"
#include "host_helpers.h"
#include "per_device.h"
#include "kernels.h"

namespace wfs {
namespace {

constexpr int kWgTile = 128;     // sites per weight-gradient tile
constexpr int kWgBlocks = 304;   // weight-gradient CTAs (2 per SM)
constexpr int kWgMaxSlots = 17;  // ceil(64 * 65 / 256) outputs per thread

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * expf(-0.5f * x * x) * 0.39894228040143268f;
}

int grid_for(int64_t n, int cap = 152 * 16) {
    int64_t g = (n + 255) / 256;
    if (g > cap) g = cap;
    return int(g < 1 ? 1 : g);
}

// ---------------------------------------------------------------------------
// Pointwise (1x1) layers
// ---------------------------------------------------------------------------
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) pointwise_kernel(const float2* __restrict__ in, const float* __restrict__ W,
                                                        const float* __restrict__ bias, const float2* add, float2* pre,
                                                        float2* out, float2* copy, int B, int64_t n3, int act) {
    __shared__ float wsh[COUT * CIN + COUT];
    for (int i = threadIdx.x; i < COUT * CIN; i += blockDim.x) wsh[i] = W[i];
    for (int i = threadIdx.x; i < COUT; i += blockDim.x) wsh[COUT * CIN + i] = bias[i];
    __syncthreads();
    constexpr int PI = CIN / 2, PO = COUT / 2;
    const int64_t total = int64_t(B) * n3;
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < total; g += int64_t(gridDim.x) * blockDim.x) {
        const int64_t b = g / n3, p = g - b * n3;
        float x[CIN];
#pragma unroll
        for (int j = 0; j < PI; ++j) {
            const float2 v = in[(b * PI + j) * n3 + p];
            x[2 * j] = v.x;
            x[2 * j + 1] = v.y;
        }
#pragma unroll 2
        for (int q = 0; q < PO; ++q) {
            float s0 = wsh[COUT * CIN + 2 * q], s1 = wsh[COUT * CIN + 2 * q + 1];
#pragma unroll
            for (int j = 0; j < CIN; ++j) {
                s0 = fmaf(wsh[(2 * q) * CIN + j], x[j], s0);
                s1 = fmaf(wsh[(2 * q + 1) * CIN + j], x[j], s1);
            }
            const int64_t oi = (b * PO + q) * n3 + p;
            if (add) {
                const float2 a = add[oi];
                s0 += a.x;
                s1 += a.y;
            }
            if (pre) pre[oi] = make_float2(s0, s1);
            const float2 o = act ? make_float2(gelu(s0), gelu(s1)) : make_float2(s0, s1);
            out[oi] = o;
            if (copy) copy[oi] = o;
        }
    }
}

// gpre = (gout + gout2) * act'(pre); gin = W^T gpre. All loads of a site happen
// before its stores, so gpre may alias gout2 and gin may alias gout.
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) pointwise_backward_kernel(const float2* gout, const float2* gout2,
                                                                 const float2* pre, int act,
                                                                 const float* __restrict__ W, float2* gpre,
                                                                 float2* gin, int B, int64_t n3) {
    __shared__ float wsh[COUT * CIN];
    for (int i = threadIdx.x; i < COUT * CIN; i += blockDim.x) wsh[i] = W[i];
    __syncthreads();
    constexpr int PI = CIN / 2, PO = COUT / 2;
    const int64_t total = int64_t(B) * n3;
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < total; g += int64_t(gridDim.x) * blockDim.x) {
        const int64_t b = g / n3, p = g - b * n3;
        float gp[COUT];
#pragma unroll
        for (int q = 0; q < PO; ++q) {
            const int64_t oi = (b * PO + q) * n3 + p;
            float2 v = gout[oi];
            if (gout2) {
                const float2 w = gout2[oi];
                v.x += w.x;
                v.y += w.y;
            }
            if (act) {
                const float2 z = pre[oi];
                v.x *= gelu_grad(z.x);
                v.y *= gelu_grad(z.y);
            }
            gp[2 * q] = v.x;
            gp[2 * q + 1] = v.y;
        }
#pragma unroll
        for (int q = 0; q < PO; ++q) gpre[(b * PO + q) * n3 + p] = make_float2(gp[2 * q], gp[2 * q + 1]);
        if (gin) {
#pragma unroll 2
            for (int j = 0; j < PI; ++j) {
                float s0 = 0.f, s1 = 0.f;
#pragma unroll
                for (int o = 0; o < COUT; ++o) {
                    s0 = fmaf(wsh[o * CIN + 2 * j], gp[o], s0);
                    s1 = fmaf(wsh[o * CIN + 2 * j + 1], gp[o], s1);
                }
                gin[(b * PI + j) * n3 + p] = make_float2(s0, s1);
            }
        }
    }
}

// Per-CTA partial sums of dW[o][j] = sum g[o] x[j] (j < cin) and db[o] (j = cin),
// q = o * (cin + 1) + j; tiles of kWgTile sites staged in shared memory.
__global__ void __launch_bounds__(256) wgrad_kernel(const float2* __restrict__ g, int cout, const float2* __restrict__ x,
                                                    int cin, int B, int64_t n3, float* __restrict__ partials) {
    extern __shared__ float sh[];
    constexpr int LD = kWgTile + 1;
    float* gs = sh;                  // [cout][LD]
    float* xs = sh + cout * LD;      // [cin + 1][LD], last row = 1 for the bias
    const int nq = cout * (cin + 1);
    const int64_t total = int64_t(B) * n3;
    const int64_t ntiles = (total + kWgTile - 1) / kWgTile;
    for (int s = threadIdx.x; s < kWgTile; s += blockDim.x) xs[cin * LD + s] = 1.f;
    float acc[kWgMaxSlots];
#pragma unroll
    for (int k = 0; k < kWgMaxSlots; ++k) acc[k] = 0.f;
    const int po = cout / 2, pi = cin / 2;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        __syncthreads();
        for (int e = threadIdx.x; e < (po + pi) * kWgTile; e += blockDim.x) {
            const int pair = e / kWgTile, s = e - pair * kWgTile;
            const int64_t site = t * kWgTile + s;
            float2 v = make_float2(0.f, 0.f);
            if (site < total) {
                const int64_t b = site / n3, p = site - b * n3;
                v = pair < po ? g[(b * po + pair) * n3 + p] : x[(b * pi + (pair - po)) * n3 + p];
            }
            float* dst = pair < po ? gs + (2 * pair) * LD : xs + (2 * (pair - po)) * LD;
            dst[s] = v.x;
            dst[LD + s] = v.y;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kWgMaxSlots; ++k) {
            const int q = threadIdx.x + k * blockDim.x;
            if (q < nq) {
                const int o = q / (cin + 1), j = q - o * (cin + 1);
                const float* gr = gs + o * LD;
                const float* xr = xs + j * LD;
                float a = 0.f;
#pragma unroll 8
                for (int s = 0; s < kWgTile; ++s) a = fmaf(gr[s], xr[s], a);
                acc[k] += a;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kWgMaxSlots; ++k) {
        const int q = threadIdx.x + k * blockDim.x;
        if (q < nq) partials[int64_t(blockIdx.x) * nq + q] = acc[k];
    }
}

// dWdb = [dW (cout x cin) | db (cout)] from the per-CTA partials, FP64 sums in CTA order.
__global__ void wgrad_sum_kernel(const float* __restrict__ partials, int nblocks, int cout, int cin,
                                 float* __restrict__ dWdb) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int nq = cout * (cin + 1);
    if (q >= nq) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += double(partials[int64_t(b) * nq + q]);
    const int o = q / (cin + 1), j = q - o * (cin + 1);
    dWdb[j < cin ? o * cin + j : cout * cin + o] = float(s);
}

// ---------------------------------------------------------------------------
// Spectral layer
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t mode_position(int mode, int N, int m) {
    const int iz = mode % m;
    const int iy = (mode / m) % (2 * m);
    const int ix = mode / (2 * m * m);
    const int kx = ix < m ? ix : N - 2 * m + ix;
    const int ky = iy < m ? iy : N - 2 * m + iy;
    return (int64_t(kx) * N + ky) * N + iz;
}
// index of a kept mode, -1 when (kx, ky, kz) is not kept
__device__ __forceinline__ int mode_of(int kx, int ky, int kz, int N, int m) {
    const int ix = kx < m ? kx : (kx >= N - m ? kx - N + 2 * m : -1);
    const int iy = ky < m ? ky : (ky >= N - m ? ky - N + 2 * m : -1);
    if (ix < 0 || iy < 0 || kz >= m) return -1;
    return (ix * 2 * m + iy) * m + kz;
}

__global__ void gather_kernel(const float2* __restrict__ spec, float2* __restrict__ Hm, int B, int C, int N, int m) {
    const int P = C / 2;
    const int nm = 4 * m * m * m;
    const int64_t n3 = int64_t(N) * N * N;
    const int64_t total = int64_t(nm) * B * P;
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < total; g += int64_t(gridDim.x) * blockDim.x) {
        const int j = int(g % P);
        const int b = int((g / P) % B);
        const int mode = int(g / (int64_t(P) * B));
        const int64_t pos = mode_position(mode, N, m);
        const int kz = int(pos % N), ky = int((pos / N) % N), kx = int(pos / (int64_t(N) * N));
        const int64_t neg = (int64_t((N - kx) % N) * N + (N - ky) % N) * N + (N - kz) % N;
        const float2* f = spec + (int64_t(b) * P + j) * n3;
        const float2 y1 = f[pos], y2 = f[neg];  // Y(k), Y(-k)
        // A = (Y(k) + conj Y(-k)) / 2, B = (Y(k) - conj Y(-k)) / 2i
        const float2 a = make_float2(0.5f * (y1.x + y2.x), 0.5f * (y1.y - y2.y));
        const float2 d = make_float2(y1.x - y2.x, y1.y + y2.y);
        const float2 bb = make_float2(0.5f * d.y, -0.5f * d.x);
        float2* dst = Hm + (int64_t(mode) * B + b) * C + 2 * j;
        dst[0] = a;
        dst[1] = bb;
    }
}

// Pull form over the kept modes and their mirrors (no write conflicts):
// Y(k) = (Za(k) + conj Za(-k)) / 2 + i (Zb(k) + conj Zb(-k)) / 2, Z = 0 off the kept set.
// The kept x (and y) set [0, m) u [N-m, N) is not closed under negation (the mirror of
// N-m is m), so the written x and y indices are [0, m] u [N-m, N) when 2m < N (2m + 1
// values; all N when 2m = N) and the z indices [0, m) u (N-m, N).
__host__ __device__ __forceinline__ int mirror_span(int N, int m) { return 2 * m < N ? 2 * m + 1 : 2 * m; }
__device__ __forceinline__ int mirror_index(int i, int N, int m) {
    return (2 * m < N && i > m) ? N - 2 * m - 1 + i : i;
}
__global__ void scatter_kernel(const float2* __restrict__ Zm, float2* __restrict__ spec, int B, int C, int N, int m) {
    const int P = C / 2;
    const int nz = 2 * m - 1;
    const int nxy = mirror_span(N, m);
    const int64_t npos = int64_t(nxy) * nxy * nz;
    const int64_t n3 = int64_t(N) * N * N;
    const int64_t total = npos * B * P;
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < total; g += int64_t(gridDim.x) * blockDim.x) {
        const int j = int(g % P);
        const int b = int((g / P) % B);
        const int64_t ip = g / (int64_t(P) * B);
        const int iz = int(ip % nz), iy = int((ip / nz) % nxy), ix = int(ip / (int64_t(nz) * nxy));
        const int kx = mirror_index(ix, N, m);
        const int ky = mirror_index(iy, N, m);
        const int kz = iz < m ? iz : N - m + 1 + (iz - m);
        const int mp = mode_of(kx, ky, kz, N, m);
        const int mn = mode_of((N - kx) % N, (N - ky) % N, (N - kz) % N, N, m);
        float2 za = make_float2(0.f, 0.f), zb = za, wa = za, wb = za;
        if (mp >= 0) {
            const float2* z = Zm + (int64_t(mp) * B + b) * C + 2 * j;
            za = z[0];
            zb = z[1];
        }
        if (mn >= 0) {
            const float2* z = Zm + (int64_t(mn) * B + b) * C + 2 * j;
            wa = z[0];
            wb = z[1];
        }
        const float2 sa = make_float2(0.5f * (za.x + wa.x), 0.5f * (za.y - wa.y));  // sym(Za)(k)
        const float2 sb = make_float2(0.5f * (zb.x + wb.x), 0.5f * (zb.y - wb.y));  // sym(Zb)(k)
        spec[(int64_t(b) * P + j) * n3 + (int64_t(kx) * N + ky) * N + kz] = make_float2(sa.x - sb.y, sa.y + sb.x);
    }
}

// W[mode][n][k] = M[k][n], M = [[Rr, Ri], [-Ri, Rr]] (2C x 2C); WT[mode][n][k] = M[n][k].
__global__ void pack_weights_kernel(const float* __restrict__ R, __nv_bfloat16* __restrict__ W,
                                    __nv_bfloat16* __restrict__ WT, int C, int nmodes) {
    const int K2 = 2 * C;
    const int64_t total = int64_t(nmodes) * K2 * K2;
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < total; g += int64_t(gridDim.x) * blockDim.x) {
        const int k = int(g % K2);
        const int n = int((g / K2) % K2);
        const int mode = int(g / (int64_t(K2) * K2));
        auto mval = [&](int r, int c) -> float {
            const float* rr = R + ((int64_t(mode) * C + (r % C)) * C + (c % C)) * 2;
            const bool top = r < C, left = c < C;
            if (top == left) return rr[0];
            return top ? rr[1] : -rr[1];
        };
        W[g] = __float2bfloat16_rn(mval(k, n));
        WT[g] = __float2bfloat16_rn(mval(n, k));
    }
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// Y[mode][b][:] = [Xr | Xi][mode][b][:] . M(mode); one warp per (mode, 16 samples).
template <int C>
__global__ void __launch_bounds__(256) mix_kernel(const float2* __restrict__ X, const __nv_bfloat16* __restrict__ Wsel,
                                                  float2* __restrict__ Y, int B, int nmodes) {
    constexpr int K2 = 2 * C;
    const int warp = int((blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    const int chunks = (B + 15) / 16;
    if (warp >= nmodes * chunks) return;
    const int mode = warp / chunks, b0 = (warp % chunks) * 16;
    const int g = lane >> 2, t4 = lane & 3;
    const float2* Xm = X + int64_t(mode) * B * C;
    const __nv_bfloat16* Wm = Wsel + int64_t(mode) * K2 * K2;
    auto aval = [&](int r, int j) -> float {  // A[r][j]: j < C real part, else imaginary part
        const int br = b0 + r;
        if (br >= B) return 0.f;
        const float2 v = Xm[int64_t(br) * C + (j < C ? j : j - C)];
        return j < C ? v.x : v.y;
    };
    float acc[K2 / 8][4];
#pragma unroll
    for (int nt = 0; nt < K2 / 8; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
#pragma unroll
    for (int kt = 0; kt < K2 / 16; ++kt) {
        const int kc = kt * 16 + t4 * 2;
        const uint32_t a0 = pack_bf16x2(aval(g, kc), aval(g, kc + 1));
        const uint32_t a1 = pack_bf16x2(aval(g + 8, kc), aval(g + 8, kc + 1));
        const uint32_t a2 = pack_bf16x2(aval(g, kc + 8), aval(g, kc + 9));
        const uint32_t a3 = pack_bf16x2(aval(g + 8, kc + 8), aval(g + 8, kc + 9));
#pragma unroll
        for (int nt = 0; nt < K2 / 8; ++nt) {
            const __nv_bfloat16* wr = Wm + int64_t(nt * 8 + g) * K2 + kc;
            const uint32_t w0 = *reinterpret_cast<const uint32_t*>(wr);
            const uint32_t w1 = *reinterpret_cast<const uint32_t*>(wr + 8);
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                "{%0,%1,%2,%3};\n"
                : "+f"(acc[nt][0]), "+f"(acc[nt][1]), "+f"(acc[nt][2]), "+f"(acc[nt][3])
                : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(w0), "r"(w1));
        }
    }
    float* Ym = reinterpret_cast<float*>(Y + int64_t(mode) * B * C);
#pragma unroll
    for (int nt = 0; nt < K2 / 8; ++nt) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int br = b0 + g + (q >= 2 ? 8 : 0);
            const int c = nt * 8 + t4 * 2 + (q & 1);
            if (br < B) Ym[(int64_t(br) * C + (c < C ? c : c - C)) * 2 + (c < C ? 0 : 1)] = acc[nt][q];
        }
    }
}

__global__ void spectral_wgrad_kernel(const float2* __restrict__ H, const float2* __restrict__ G, float* __restrict__ dR,
                                      int B, int C, int nmodes) {
    const int64_t total = int64_t(nmodes) * C * C;
    for (int64_t gi = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; gi < total; gi += int64_t(gridDim.x) * blockDim.x) {
        const int o = int(gi % C);
        const int i = int((gi / C) % C);
        const int64_t mode = gi / (int64_t(C) * C);
        float re = 0.f, im = 0.f;
        for (int b = 0; b < B; ++b) {
            const float2 h = H[(mode * B + b) * C + i];
            const float2 gz = G[(mode * B + b) * C + o];
            re = fmaf(h.x, gz.x, fmaf(h.y, gz.y, re));
            im = fmaf(h.x, gz.y, fmaf(-h.y, gz.x, im));
        }
        dR[gi * 2] = re;
        dR[gi * 2 + 1] = im;
    }
}

// ---------------------------------------------------------------------------
// Optimiser, loss, acceptance norms
// ---------------------------------------------------------------------------
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, int64_t n, float lr, float b1, float b2, float eps, float wd,
                            float bc1, float bc2) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.f - b1) * gi;
        const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = v;
        const float mh = a / bc1, vh = v / bc2;
        p[i] -= lr * (mh / (sqrtf(vh) + eps) + wd * p[i]);
    }
}

// One CTA per (sample, slice): partial sums of |p - t|^2 and |t|^2 (FP64 across warps).
constexpr int kLossSlices = 32;
__global__ void __launch_bounds__(256) loss_partial_kernel(const float* __restrict__ pred, const float* __restrict__ target,
                                                           int64_t per_sample, double* __restrict__ part) {
    const int b = blockIdx.x / kLossSlices, sl = blockIdx.x % kLossSlices;
    const int64_t chunk = (per_sample + kLossSlices - 1) / kLossSlices;
    const int64_t lo = sl * chunk, hi = lo + chunk < per_sample ? lo + chunk : per_sample;
    const float* p = pred + int64_t(b) * per_sample;
    const float* t = target + int64_t(b) * per_sample;
    float d2 = 0.f, t2 = 0.f;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const float d = p[i] - t[i];
        d2 = fmaf(d, d, d2);
        t2 = fmaf(t[i], t[i], t2);
    }
    for (int off = 16; off > 0; off >>= 1) {
        d2 += __shfl_down_sync(0xffffffffu, d2, off);
        t2 += __shfl_down_sync(0xffffffffu, t2, off);
    }
    __shared__ double sd[8], st[8];
    if ((threadIdx.x & 31) == 0) {
        sd[threadIdx.x >> 5] = d2;
        st[threadIdx.x >> 5] = t2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, c = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) {
            a += sd[w];
            c += st[w];
        }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = c;
    }
}
__global__ void loss_finish_kernel(const double* __restrict__ part, int B, float grad_scale,
                                   float* __restrict__ sample_err, float* __restrict__ loss,
                                   float* __restrict__ scale_out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double total = 0.0;
    for (int b = 0; b < B; ++b) {
        double a = 0.0, c = 0.0;
        for (int s = 0; s < kLossSlices; ++s) {
            a += part[2 * (b * kLossSlices + s)];
            c += part[2 * (b * kLossSlices + s) + 1];
        }
        if (c <= 0.0) c = 1.0;
        sample_err[b] = float(a / c);
        scale_out[b] = float(double(grad_scale) * 2.0 / (double(B) * c));
        total += a / c;
    }
    *loss = float(total / B);
}
__global__ void loss_grad_kernel(const float* __restrict__ pred, const float* __restrict__ target, int64_t per_sample,
                                 int B, const float* __restrict__ scale, float* __restrict__ grad) {
    const int64_t total = int64_t(B) * per_sample;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x)
        grad[i] = scale[i / per_sample] * (pred[i] - target[i]);
}

__global__ void __launch_bounds__(256) sample_norms_kernel(const float2* __restrict__ a, const float2* __restrict__ c,
                                                           int64_t per_sample, double* __restrict__ part) {
    const int b = blockIdx.x / kLossSlices, sl = blockIdx.x % kLossSlices;
    const int64_t chunk = (per_sample + kLossSlices - 1) / kLossSlices;
    const int64_t lo = sl * chunk, hi = lo + chunk < per_sample ? lo + chunk : per_sample;
    float s2 = 0.f, d2 = 0.f;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const float2 u = a[int64_t(b) * per_sample + i];
        s2 = fmaf(u.x, u.x, fmaf(u.y, u.y, s2));
        if (c) {
            const float2 v = c[int64_t(b) * per_sample + i];
            const float dx = u.x - v.x, dy = u.y - v.y;
            d2 = fmaf(dx, dx, fmaf(dy, dy, d2));
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        s2 += __shfl_down_sync(0xffffffffu, s2, off);
        d2 += __shfl_down_sync(0xffffffffu, d2, off);
    }
    __shared__ double ss[8], sd[8];
    if ((threadIdx.x & 31) == 0) {
        ss[threadIdx.x >> 5] = s2;
        sd[threadIdx.x >> 5] = d2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) {
            x += ss[w];
            y += sd[w];
        }
        part[2 * blockIdx.x] = x;
        part[2 * blockIdx.x + 1] = y;
    }
}
__global__ void sample_norms_finish_kernel(const double* __restrict__ part, int B, double* __restrict__ a2,
                                           double* __restrict__ d2) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    double x = 0.0, y = 0.0;
    for (int s = 0; s < kLossSlices; ++s) {
        x += part[2 * (b * kLossSlices + s)];
        y += part[2 * (b * kLossSlices + s) + 1];
    }
    a2[b] = x;
    if (d2) d2[b] = y;
}

// x[b][0] = psi_b / s_b, x[b][1] = V_b * vscale, s_b = sqrt(a2_b / n3) (1 when a2 is NULL)
__global__ void make_input_kernel(const float2* __restrict__ psi, const float2* __restrict__ V, float vscale,
                                  const double* __restrict__ a2, float2* __restrict__ x, int B, int64_t n3) {
    const int64_t total = int64_t(B) * n3;
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < total; g += int64_t(gridDim.x) * blockDim.x) {
        const int64_t b = g / n3, p = g - b * n3;
        const float inv = a2 ? float(1.0 / sqrt(a2[b] / double(n3))) : 1.f;
        const float2 u = psi[g];
        const float2 v = V[g];
        x[(b * 2) * n3 + p] = make_float2(u.x * inv, u.y * inv);
        x[(b * 2 + 1) * n3 + p] = make_float2(v.x * vscale, v.y * vscale);
    }
}
// a_b *= s_b (invert = 0) or a_b /= s_b (invert = 1), s_b = sqrt(a2_b / n3)
__global__ void scale_samples_kernel(float2* __restrict__ a, const double* __restrict__ a2, int invert, int B,
                                     int64_t n3) {
    const int64_t total = int64_t(B) * n3;
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < total; g += int64_t(gridDim.x) * blockDim.x) {
        const double s = sqrt(a2[g / n3] / double(n3));
        const float f = float(invert ? 1.0 / s : s);
        const float2 u = a[g];
        a[g] = make_float2(u.x * f, u.y * f);
    }
}

// ---------------------------------------------------------------------------
// Host side: per-device twiddle tables and scratch
// ---------------------------------------------------------------------------
std::mutex g_fno_mu;
std::map<std::pair<int, int>, Cx<float>*> g_twiddles;   // (device, N) -> table
std::map<int, std::pair<void*, size_t>> g_scratch;       // device -> small scratch

const Cx<float>* twiddles_for(int N) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_fno_mu);
    auto it = g_twiddles.find({dev, N});
    if (it != g_twiddles.end()) return it->second;
    std::vector<Cx<float>> t(3 * size_t(N));
    if (!two_stage_roots<float>(N, t.data())) return nullptr;
    Cx<float>* d = nullptr;
    if (cudaMalloc(&d, t.size() * sizeof(Cx<float>)) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, t.data(), t.size() * sizeof(Cx<float>), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    g_twiddles[{dev, N}] = d;
    return d;
}

// Small per-device scratch used by the loss and norm reductions; calls that use
// it must be ordered on one stream.
void* scratch_for(size_t bytes) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_fno_mu);
    auto& s = g_scratch[dev];
    if (s.second >= bytes) return s.first;
    if (s.first) {
        cudaDeviceSynchronize();
        cudaFree(s.first);
    }
    s = {nullptr, 0};
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    s = {p, bytes};
    return p;
}

int status_of(cudaError_t e) { return e == cudaSuccess ? WFS_OK : WFS_ERR_CUDA; }

bool supported_width(int c) { return c == 2 || c == 4 || c == 8 || c == 16 || c == 32 || c == 64; }

template <int CIN, int COUT>
cudaError_t run_pointwise(const void* in, const float* W, const float* bias, const void* add, void* pre, void* out,
                          void* copy, int B, int64_t n3, int act, cudaStream_t s) {
    pointwise_kernel<CIN, COUT><<<grid_for(int64_t(B) * n3), 256, 0, s>>>(
        (const float2*)in, W, bias, (const float2*)add, (float2*)pre, (float2*)out, (float2*)copy, B, n3, act);
    return cudaGetLastError();
}
template <int CIN, int COUT>
cudaError_t run_pointwise_backward(const void* gout, const void* gout2, const void* pre, int act, const float* W,
                                   void* gpre, void* gin, int B, int64_t n3, cudaStream_t s) {
    pointwise_backward_kernel<CIN, COUT><<<grid_for(int64_t(B) * n3), 256, 0, s>>>(
        (const float2*)gout, (const float2*)gout2, (const float2*)pre, act, W, (float2*)gpre, (float2*)gin, B, n3);
    return cudaGetLastError();
}

// (cin, cout) pairs the network uses: lift 4 -> C, layers C -> C, projection C -> 2C
// and 2C -> 2, for C in {4, 8, 16, 32}.
#define WFS_FNO_PAIRS(M) \
    M(4, 4) M(4, 8) M(4, 16) M(4, 32) M(8, 8) M(16, 16) M(32, 32) M(8, 16) M(16, 32) M(32, 64) \
    M(8, 2) M(16, 2) M(32, 2) M(64, 2)

}  // namespace
}  // namespace wfs

using namespace wfs;

extern "C" {

int wfs_fno_pointwise(const void* in, int32_t cin, const float* W, const float* bias, const void* add, void* pre,
                      void* out, void* copy, int32_t cout, int32_t B, int64_t n3, int32_t act, void* stream) {
    if (!in || !W || !bias || !out || B < 1 || n3 < 1) return WFS_ERR_ARG;
    if (!supported_width(cin) || !supported_width(cout)) return WFS_ERR_UNSUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
#define WFS_PW(CI, CO) \
    if (cin == CI && cout == CO) return status_of(run_pointwise<CI, CO>(in, W, bias, add, pre, out, copy, B, n3, act, s));
    WFS_FNO_PAIRS(WFS_PW)
#undef WFS_PW
    return WFS_ERR_UNSUPPORTED;
}

int wfs_fno_pointwise_backward(const void* gout, const void* gout2, const void* pre, int32_t act, const float* W,
                               void* gpre, void* gin, int32_t cin, int32_t cout, int32_t B, int64_t n3,
                               void* stream) {
    if (!gout || !W || !gpre || B < 1 || n3 < 1 || (act && !pre)) return WFS_ERR_ARG;
    if (!supported_width(cin) || !supported_width(cout)) return WFS_ERR_UNSUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
#define WFS_PWB(CI, CO)                                                                                        \
    if (cin == CI && cout == CO)                                                                               \
        return status_of(run_pointwise_backward<CI, CO>(gout, gout2, pre, act, W, gpre, gin, B, n3, s));
    WFS_FNO_PAIRS(WFS_PWB)
#undef WFS_PWB
    return WFS_ERR_UNSUPPORTED;
}

int64_t wfs_fno_wgrad_scratch(int32_t cin, int32_t cout) { return int64_t(kWgBlocks) * cout * (cin + 1); }

int wfs_fno_weight_grad(const void* g, int32_t cout, const void* x, int32_t cin, int32_t B, int64_t n3,
                        float* partials, float* dWdb, void* stream) {
    if (!g || !x || !partials || !dWdb || B < 1 || n3 < 1) return WFS_ERR_ARG;
    if (!supported_width(cin) || !supported_width(cout)) return WFS_ERR_UNSUPPORTED;
    if (cout * (cin + 1) > kWgMaxSlots * 256) return WFS_ERR_UNSUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t ntiles = (int64_t(B) * n3 + kWgTile - 1) / kWgTile;
    const int nblocks = int(ntiles < kWgBlocks ? ntiles : kWgBlocks);
    const size_t smem = size_t(cout + cin + 1) * (kWgTile + 1) * sizeof(float);
    static PerDevice attr;
    const int dev = current_device();
    if (!attr.get(dev)) {
        if (cudaFuncSetAttribute(wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 80 * 1024) != cudaSuccess)
            return WFS_ERR_CUDA;
        attr.put(dev, 1);
    }
    wgrad_kernel<<<nblocks, 256, smem, s>>>((const float2*)g, cout, (const float2*)x, cin, B, n3, partials);
    const int nq = cout * (cin + 1);
    wgrad_sum_kernel<<<(nq + 255) / 256, 256, 0, s>>>(partials, nblocks, cout, cin, dWdb);
    return status_of(cudaGetLastError());
}

int wfs_fno_fft3(void* data, int64_t nfields, int32_t N, int32_t dir, void* stream) {
    if (!data || nfields < 1 || (dir != -1 && dir != 1)) return WFS_ERR_ARG;
    if (!fft_length_supported(N, false)) return WFS_ERR_UNSUPPORTED;
    const int64_t n2 = int64_t(N) * N, n3 = n2 * N;
    if (nfields * n3 >= (int64_t(1) << 31)) return WFS_ERR_UNSUPPORTED;
    const Cx<float>* tw = twiddles_for(N);
    if (!tw) return WFS_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    PassArgs<float> a;
    std::memset(&a, 0, sizeof(a));
    a.data = reinterpret_cast<Cx<float>*>(data);
    a.tw = tw;
    a.dir = dir;
    a.scale = float(1.0 / std::sqrt(double(N)));
    // x pencils: one outer slab per field, N^2 contiguous columns
    a.outer_stride = n3;
    a.row_stride = n2;
    a.ncols = int32_t(n2);
    cudaError_t e = launch_fft_strided<float>(N, OP_PLAIN, a, nfields, s);
    if (e != cudaSuccess) return WFS_ERR_CUDA;
    // y pencils: one outer slab per (field, x), N contiguous columns
    a.outer_stride = n2;
    a.row_stride = N;
    a.ncols = N;
    e = launch_fft_strided<float>(N, OP_PLAIN, a, nfields * N, s);
    if (e != cudaSuccess) return WFS_ERR_CUDA;
    // z rows
    a.nrows = nfields * n2;
    e = launch_fft_contig<float>(N, OP_PLAIN, a, s, nullptr);
    return status_of(e);
}

int wfs_fno_gather(const void* spec, void* Hm, int32_t B, int32_t C, int32_t N, int32_t m, void* stream) {
    if (!spec || !Hm || B < 1 || C < 2 || (C & 1) || m < 1 || 2 * m > N) return WFS_ERR_ARG;
    const int64_t total = int64_t(4) * m * m * m * B * (C / 2);
    gather_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>((const float2*)spec, (float2*)Hm, B, C, N, m);
    return status_of(cudaGetLastError());
}

int wfs_fno_scatter(const void* Zm, void* spec, int32_t B, int32_t C, int32_t N, int32_t m, void* stream) {
    if (!Zm || !spec || B < 1 || C < 2 || (C & 1) || m < 1 || 2 * m > N) return WFS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n3 = int64_t(N) * N * N;
    if (cudaMemsetAsync(spec, 0, size_t(B) * (C / 2) * n3 * sizeof(float2), s) != cudaSuccess) return WFS_ERR_CUDA;
    const int nxy = mirror_span(N, m);
    const int64_t total = int64_t(nxy) * nxy * (2 * m - 1) * B * (C / 2);
    scatter_kernel<<<grid_for(total), 256, 0, s>>>((const float2*)Zm, (float2*)spec, B, C, N, m);
    return status_of(cudaGetLastError());
}

int wfs_fno_pack_weights(const float* R, void* W, void* WT, int32_t C, int32_t nmodes, void* stream) {
    if (!R || !W || !WT || C < 1 || nmodes < 1) return WFS_ERR_ARG;
    const int64_t total = int64_t(nmodes) * 4 * C * C;
    pack_weights_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(R, (__nv_bfloat16*)W, (__nv_bfloat16*)WT, C,
                                                                            nmodes);
    return status_of(cudaGetLastError());
}

int wfs_fno_mix(const void* X, const void* Wsel, void* Y, int32_t B, int32_t C, int32_t nmodes, void* stream) {
    if (!X || !Wsel || !Y || B < 1 || nmodes < 1) return WFS_ERR_ARG;
    const int64_t warps = int64_t(nmodes) * ((B + 15) / 16);
    const int64_t blocks64 = (warps * 32 + 255) / 256;
    if (blocks64 >= (int64_t(1) << 31)) return WFS_ERR_UNSUPPORTED;
    const int blocks = int(blocks64);
    cudaStream_t s = (cudaStream_t)stream;
    const float2* x = (const float2*)X;
    const __nv_bfloat16* w = (const __nv_bfloat16*)Wsel;
    float2* y = (float2*)Y;
    switch (C) {
        case 8: mix_kernel<8><<<blocks, 256, 0, s>>>(x, w, y, B, nmodes); break;
        case 16: mix_kernel<16><<<blocks, 256, 0, s>>>(x, w, y, B, nmodes); break;
        case 32: mix_kernel<32><<<blocks, 256, 0, s>>>(x, w, y, B, nmodes); break;
        default: return WFS_ERR_UNSUPPORTED;
    }
    return status_of(cudaGetLastError());
}

int wfs_fno_spectral_weight_grad(const void* H, const void* G, float* dR, int32_t B, int32_t C, int32_t nmodes,
                                 void* stream) {
    if (!H || !G || !dR || B < 1 || C < 1 || nmodes < 1) return WFS_ERR_ARG;
    const int64_t total = int64_t(nmodes) * C * C;
    spectral_wgrad_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>((const float2*)H, (const float2*)G, dR, B,
                                                                              C, nmodes);
    return status_of(cudaGetLastError());
}

int wfs_fno_adam(float* p, const float* g, float* m1, float* m2, int64_t n, float lr, float beta1, float beta2,
                 float eps, float weight_decay, int32_t step, void* stream) {
    if (!p || !g || !m1 || !m2 || n < 1 || step < 1) return WFS_ERR_ARG;
    const float bc1 = float(1.0 - std::pow(double(beta1), step));
    const float bc2 = float(1.0 - std::pow(double(beta2), step));
    adam_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(p, g, m1, m2, n, lr, beta1, beta2, eps, weight_decay,
                                                                bc1, bc2);
    return status_of(cudaGetLastError());
}

int wfs_fno_loss(const float* pred, const float* target, int64_t per_sample, int32_t B, float grad_scale,
                 float* sample_err, float* grad, float* loss, void* stream) {
    if (!pred || !target || !sample_err || !loss || per_sample < 1 || B < 1 || !(grad_scale > 0.f))
        return WFS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t part_bytes = ((size_t(B) * kLossSlices * 2 * sizeof(double) + 255) / 256) * 256;
    char* scr = (char*)scratch_for(part_bytes + size_t(B) * sizeof(float));
    if (!scr) return WFS_ERR_CUDA;
    double* part = (double*)scr;
    float* scale = (float*)(scr + part_bytes);
    loss_partial_kernel<<<B * kLossSlices, 256, 0, s>>>(pred, target, per_sample, part);
    loss_finish_kernel<<<1, 32, 0, s>>>(part, B, grad_scale, sample_err, loss, scale);
    if (grad) loss_grad_kernel<<<grid_for(int64_t(B) * per_sample), 256, 0, s>>>(pred, target, per_sample, B, scale, grad);
    return status_of(cudaGetLastError());
}

int wfs_fno_sample_norms(const void* a, const void* c, int64_t per_sample, int32_t B, double* a2, double* d2,
                         void* stream) {
    if (!a || !a2 || per_sample < 1 || B < 1 || (c && !d2)) return WFS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    double* part = (double*)scratch_for(((size_t(B) * kLossSlices * 2 * sizeof(double) + 255) / 256) * 256 +
                                        size_t(B) * sizeof(float));
    if (!part) return WFS_ERR_CUDA;
    sample_norms_kernel<<<B * kLossSlices, 256, 0, s>>>((const float2*)a, (const float2*)c, per_sample, part);
    sample_norms_finish_kernel<<<(B + 127) / 128, 128, 0, s>>>(part, B, a2, d2);
    return status_of(cudaGetLastError());
}

int wfs_fno_make_input(const void* psi, const void* V, float vscale, const double* a2, void* x, int32_t B, int64_t n3,
                       void* stream) {
    if (!psi || !V || !x || B < 1 || n3 < 1) return WFS_ERR_ARG;
    make_input_kernel<<<grid_for(int64_t(B) * n3), 256, 0, (cudaStream_t)stream>>>(
        (const float2*)psi, (const float2*)V, vscale, a2, (float2*)x, B, n3);
    return status_of(cudaGetLastError());
}

int wfs_fno_scale_samples(void* a, const double* a2, int32_t invert, int32_t B, int64_t n3, void* stream) {
    if (!a || !a2 || B < 1 || n3 < 1) return WFS_ERR_ARG;
    scale_samples_kernel<<<grid_for(int64_t(B) * n3), 256, 0, (cudaStream_t)stream>>>((float2*)a, a2, invert, B, n3);
    return status_of(cudaGetLastError());
}

}  // extern "C"
