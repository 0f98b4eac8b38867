// fno_fast.cu — inference forward pass of the FNO surrogate on the kept modes only.
//
// The training forward (fno.cu) transforms every hidden field with full 64^3 FFTs and
// keeps FP32 activations: about 9 KB of HBM traffic per grid site and sample. A jump's
// correction is small against the prior it is added to (about 1e-2 of psi), so an
// inference pass can run every product on BF16 tensor cores with FP32 accumulation
// and keep its intermediates in BF16 without moving the jump's error. This file does
// that, and transforms only what the spectral layers use:
//
//   z-row kernel   one CTA per 4 z-rows (256 sites, all 32 channels): the inverse
//                  z-DFT of the layer's spectral branch (12 kept kz -> 64 z) and the
//                  pointwise 1x1 layer accumulate into one product, then bias, GELU,
//                  the BF16 store of h, and the forward z-DFT of h (64 z -> 12 kz) with
//                  the activations transposed in registers (movmatrix). The lift and
//                  the last layer with both projections are variants of the same kernel.
//   y kernels      per (sample, channel, 8 x-columns): the 64 -> 24 kept-ky DFT and back.
//   x+mix kernel   per kept (ky, kz) and 16 samples: the 64 -> 24 kept-kx DFT, the
//                  per-mode complex channel mixing Z = H R, and the 24 -> 64 inverse.
//
// Every product is mma.sync m16n8k16 (BF16 operands, FP32 accumulation); the DFT
// matrices are BF16 constants. Traffic per site and sample for four layers is about
// 1.3 KB plus the mixing weights (56 MB per layer per 16 samples).
//
// Layouts (bf16x2 words: two channels, or the real and imaginary part of one value):
//   H   [B][16][64^3]              channel pairs (2j, 2j+1), as the packed layout
//   SZ  [B][32][64 x][64 y][12 kz] z-spectra of each real channel
//   SY  [24 ky][12 kz][B][32][64 x] y-spectra, x fastest (the x+mix kernel's rows)
// The kept modes follow include/wfs_fno.h: kx, ky in [0, 12) u [52, 64), kz in [0, 12);
// mode = (ix * 24 + iy) * 12 + iz. Geometry is fixed: N = 64, width 32, 12 modes.
#include <cuda_bf16.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/wfs.h"
#include "../../include/wfs_fno.h"

namespace wfs {
namespace {

constexpr int FN = 64;                 // grid points per axis
constexpr int FC = 32;                 // hidden channels
constexpr int FM = 12;                 // kept kz
constexpr int FK = 24;                 // kept kx and ky
constexpr int64_t FN3 = int64_t(FN) * FN * FN;
constexpr int ZSLAB = FN * FM;         // words of one (b, c, x) z-spectrum slab
constexpr int NPK = FK * FM;           // kept (ky, kz) pairs
constexpr int FWD_LD = 68;             // forward DFT matrix row stride in smem (words)
constexpr int INV_LD = 28;             // inverse DFT matrix row stride in smem (words)
constexpr int HS_B = 36;               // x+mix: words per sample row of the mode buffer
constexpr int HS_K = 584;              // x+mix: words per kept kx of the mode buffer

// BF16 constants of the kept-mode DFTs, per device (see fast_tables).
struct FastTables {
    uint16_t* tz;    // [64 z][32 j]   j = 2 kz + (0: cos, 1: -sin) / 8, j >= 24 zero
    uint16_t* tzt;   // [32 j][64 z]   transpose of tz
    uint16_t* fwd;   // [48 j][128 k]  forward 64 -> 24 DFT, k = 2 n + s, j = 2 k' + s'
    uint16_t* inv;   // [128 j][48 k]  inverse 24 -> 64 DFT, k = 2 k' + s, j = 2 n + s'
};

std::mutex g_fast_mu;
std::map<int, FastTables> g_fast;

// round-to-nearest-even float -> bfloat16 bits (host)
uint16_t bf16_bits(double v) {
    float f = float(v);
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return uint16_t(u >> 16);
}

int kept_freq(int i) { return i < FM ? i : i + (FN - FK); }

const FastTables* fast_tables() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_fast_mu);
    auto it = g_fast.find(dev);
    if (it != g_fast.end()) return &it->second;
    const double two_pi = 6.283185307179586476925286766559, s = 1.0 / std::sqrt(double(FN));
    std::vector<uint16_t> tz(64 * 32, 0), tzt(32 * 64, 0), fwd(48 * 128), inv(128 * 48);
    for (int z = 0; z < FN; ++z)
        for (int kz = 0; kz < FM; ++kz) {
            const double th = two_pi * double((kz * z) % FN) / FN;
            const uint16_t c = bf16_bits(std::cos(th) * s), sn = bf16_bits(-std::sin(th) * s);
            tz[z * 32 + 2 * kz] = c;
            tz[z * 32 + 2 * kz + 1] = sn;
            tzt[(2 * kz) * 64 + z] = c;
            tzt[(2 * kz + 1) * 64 + z] = sn;
        }
    for (int n = 0; n < FN; ++n)
        for (int kk = 0; kk < FK; ++kk) {
            const double th = two_pi * double((kept_freq(kk) * n) % FN) / FN;
            const double c = std::cos(th) * s, sn = std::sin(th) * s;
            // forward: out(k') = sum_n in(n) e^{-i th}: re = a c + b sn, im = b c - a sn
            fwd[(2 * kk) * 128 + 2 * n] = bf16_bits(c);
            fwd[(2 * kk) * 128 + 2 * n + 1] = bf16_bits(sn);
            fwd[(2 * kk + 1) * 128 + 2 * n] = bf16_bits(-sn);
            fwd[(2 * kk + 1) * 128 + 2 * n + 1] = bf16_bits(c);
            // inverse: out(n) = sum_k' in(k') e^{+i th}: re = a c - b sn, im = b c + a sn
            inv[(2 * n) * 48 + 2 * kk] = bf16_bits(c);
            inv[(2 * n) * 48 + 2 * kk + 1] = bf16_bits(-sn);
            inv[(2 * n + 1) * 48 + 2 * kk] = bf16_bits(sn);
            inv[(2 * n + 1) * 48 + 2 * kk + 1] = bf16_bits(c);
        }
    const size_t words = tz.size() + tzt.size() + fwd.size() + inv.size();
    uint16_t* d = nullptr;
    if (cudaMalloc(&d, words * sizeof(uint16_t)) != cudaSuccess) return nullptr;
    std::vector<uint16_t> all;
    all.reserve(words);
    for (auto* v : {&tz, &tzt, &fwd, &inv}) all.insert(all.end(), v->begin(), v->end());
    if (cudaMemcpy(d, all.data(), words * sizeof(uint16_t), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    FastTables t;
    t.tz = d;
    t.tzt = t.tz + tz.size();
    t.fwd = t.tzt + tzt.size();
    t.inv = t.fwd + fwd.size();
    return &(g_fast[dev] = t);
}

// ---------------------------------------------------------------------------
// Fragments of mma.m16n8k16 (row.col): lane = 4 g + t4.
//   A (16 x 16): a0 = A[g][2t4..], a1 = A[g+8][2t4..], a2 = A[g][2t4+8..], a3 = A[g+8][2t4+8..]
//   B (16 x 8):  b0 = B[2t4..][g],  b1 = B[2t4+8..][g]   (lower k in the low half)
//   D (16 x 8):  d0,d1 = D[g][2t4], D[g][2t4+1]; d2,d3 = D[g+8][2t4], D[g+8][2t4+1]
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mma(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t pk(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
// 8x8 b16 transpose across the warp: lane 4r + c holds row r, columns 2c and 2c+1
__device__ __forceinline__ uint32_t trans8(uint32_t x) {
    uint32_t y;
    asm volatile("movmatrix.sync.aligned.m8n8.trans.b16 %0, %1;\n" : "=r"(y) : "r"(x));
    return y;
}
__device__ __forceinline__ uint32_t w32(const uint16_t* p, int i) {  // two bf16 at an even index
    return *reinterpret_cast<const uint32_t*>(p + i);
}
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

struct ZrowArgs {
    const float2* x;        // lift: network input [B][2][n3] complex64 (4 channels)
    const uint32_t* h;      // layer / last: H of the previous layer
    uint32_t* sz;           // SZ: read (layer, last) and written (lift, layer), in place
    const uint16_t* W;      // pointwise weights bf16 [32][16] (lift, zero padded) or [32][32]
    const float* bias;      // [32]
    const uint16_t* Wq1;    // last: [64][32]
    const float* bq1;       // last: [64]
    const uint16_t* Wq2;    // last: [8][64], rows 2..7 zero
    const float* bq2;       // last: [2]
    const float2* prior;    // last: [B][n3] complex64
    uint32_t* h_out;        // lift / layer: H of this layer
    float2* out;            // last: prior + network, [B][n3] complex64
    const uint16_t* tz;
    const uint16_t* tzt;
    int B;
};

enum { ZROW_LIFT = 0, ZROW_LAYER = 1, ZROW_LAST = 2 };

// One CTA: sample b, column x, rows y0..y0+3 (y0 = 4 * (blockIdx % 16)). Warp w owns
// row y0 + w/2 and sites z in [32 (w&1), 32 (w&1) + 32): two 16-site m-tiles.
template <int MODE>
__global__ void __launch_bounds__(256) fno_zrow_kernel(const ZrowArgs a) {
    __shared__ float2 red[4][FC][FM];      // partial forward z-spectra of the second half-rows
    __shared__ uint32_t szbuf[FC][4 * FM]; // the CTA's finished z-spectra, per channel
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t4 = lane & 3;
    const int yg = blockIdx.x % 16, xcol = (blockIdx.x / 16) % FN, b = blockIdx.x / (16 * FN);
    const int r = warp >> 1, half = warp & 1, y = 4 * yg + r, z0 = 32 * half;
    const int64_t row = (int64_t(xcol) * FN + y) * FN;   // site index of z = 0
    float d[2][4][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) d[mt][nt][q] = 0.f;

    if constexpr (MODE == ZROW_LIFT) {
        // h0 = W0 x + b0: channels (Re psi, Im psi) in pair 0, (Re V s, Im V s) in pair 1
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const int64_t s0 = row + z0 + 16 * mt + g;
            uint32_t A[4] = {0u, 0u, 0u, 0u};
            if (t4 < 2) {
                const float2* xb = a.x + (int64_t(b) * 2 + t4) * FN3;
                const float2 v0 = xb[s0], v1 = xb[s0 + 8];
                A[0] = pk(v0.x, v0.y);
                A[1] = pk(v1.x, v1.y);
            }
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
                mma(d[mt][nt], A, w32(a.W, (nt * 8 + g) * 16 + 2 * t4), w32(a.W, (nt * 8 + g) * 16 + 8 + 2 * t4));
        }
    } else {
        // pointwise term W h
        const uint32_t* hb = a.h + int64_t(b) * (FC / 2) * FN3;
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            uint32_t Bw[4][2];
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                Bw[nt][0] = w32(a.W, (nt * 8 + g) * 32 + 16 * ks + 2 * t4);
                Bw[nt][1] = w32(a.W, (nt * 8 + g) * 32 + 16 * ks + 8 + 2 * t4);
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int64_t s0 = row + z0 + 16 * mt + g;
                const uint32_t* p0 = hb + int64_t(8 * ks + t4) * FN3;
                const uint32_t* p1 = p0 + 4 * FN3;
                const uint32_t A[4] = {p0[s0], p0[s0 + 8], p1[s0], p1[s0 + 8]};
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) mma(d[mt][nt], A, Bw[nt][0], Bw[nt][1]);
            }
        }
        // spectral term: s_c(z) = sum_j T[z][j] W_c[j], W_c = (re, im) of the 12 kept kz
        const uint32_t* szb = a.sz + ((int64_t(b) * FC * FN + xcol) * FN + y) * FM;   // channel 0
        const int64_t cstride = int64_t(FN) * FN * FM;
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            uint32_t At[2][4];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int zr = z0 + 16 * mt + g;
                At[mt][0] = w32(a.tz, zr * 32 + 16 * ks + 2 * t4);
                At[mt][1] = w32(a.tz, (zr + 8) * 32 + 16 * ks + 2 * t4);
                At[mt][2] = w32(a.tz, zr * 32 + 16 * ks + 8 + 2 * t4);
                At[mt][3] = w32(a.tz, (zr + 8) * 32 + 16 * ks + 8 + 2 * t4);
            }
            const int kz0 = 8 * ks + t4, kz1 = kz0 + 4;
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const uint32_t* sc = szb + int64_t(nt * 8 + g) * cstride;
                const uint32_t b0 = kz0 < FM ? sc[kz0] : 0u;
                const uint32_t b1 = kz1 < FM ? sc[kz1] : 0u;
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) mma(d[mt][nt], At[mt], b0, b1);
            }
        }
    }

    // bias (and GELU for hidden layers)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const float c0 = a.bias[nt * 8 + 2 * t4], c1 = a.bias[nt * 8 + 2 * t4 + 1];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            d[mt][nt][0] += c0;
            d[mt][nt][1] += c1;
            d[mt][nt][2] += c0;
            d[mt][nt][3] += c1;
            if constexpr (MODE == ZROW_LAYER) {
#pragma unroll
                for (int q = 0; q < 4; ++q) d[mt][nt][q] = gelu(d[mt][nt][q]);
            }
        }
    }

    if constexpr (MODE == ZROW_LAST) {
        // out = Wq2 GELU(Wq1 h + bq1) + bq2 + prior, chained through the fragments
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            uint32_t A1[2][4];
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {
                A1[ks][0] = pk(d[mt][2 * ks][0], d[mt][2 * ks][1]);
                A1[ks][1] = pk(d[mt][2 * ks][2], d[mt][2 * ks][3]);
                A1[ks][2] = pk(d[mt][2 * ks + 1][0], d[mt][2 * ks + 1][1]);
                A1[ks][3] = pk(d[mt][2 * ks + 1][2], d[mt][2 * ks + 1][3]);
            }
            float q[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
                for (int i = 0; i < 4; ++i) q[nt][i] = 0.f;
#pragma unroll
                for (int ks = 0; ks < 2; ++ks)
                    mma(q[nt], A1[ks], w32(a.Wq1, (nt * 8 + g) * 32 + 16 * ks + 2 * t4),
                        w32(a.Wq1, (nt * 8 + g) * 32 + 16 * ks + 8 + 2 * t4));
                const float c0 = a.bq1[nt * 8 + 2 * t4], c1 = a.bq1[nt * 8 + 2 * t4 + 1];
                q[nt][0] = gelu(q[nt][0] + c0);
                q[nt][1] = gelu(q[nt][1] + c1);
                q[nt][2] = gelu(q[nt][2] + c0);
                q[nt][3] = gelu(q[nt][3] + c1);
            }
            float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                const uint32_t A2[4] = {pk(q[2 * ks][0], q[2 * ks][1]), pk(q[2 * ks][2], q[2 * ks][3]),
                                        pk(q[2 * ks + 1][0], q[2 * ks + 1][1]),
                                        pk(q[2 * ks + 1][2], q[2 * ks + 1][3])};
                mma(o, A2, w32(a.Wq2, g * 64 + 16 * ks + 2 * t4), w32(a.Wq2, g * 64 + 16 * ks + 8 + 2 * t4));
            }
            if (t4 == 0) {
                const int64_t s0 = int64_t(b) * FN3 + row + z0 + 16 * mt + g;
                const float2 p0 = a.prior[s0], p1 = a.prior[s0 + 8];
                a.out[s0] = make_float2(o[0] + a.bq2[0] + p0.x, o[1] + a.bq2[1] + p0.y);
                a.out[s0 + 8] = make_float2(o[2] + a.bq2[0] + p1.x, o[3] + a.bq2[1] + p1.y);
            }
        }
        return;
    } else {
        // store h (BF16 channel pairs) and keep the packed fragments for the z-DFT
        uint32_t P[2][4][2];
        uint32_t* hb = a.h_out + int64_t(b) * (FC / 2) * FN3;
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const int64_t s0 = row + z0 + 16 * mt + g;
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                P[mt][nt][0] = pk(d[mt][nt][0], d[mt][nt][1]);
                P[mt][nt][1] = pk(d[mt][nt][2], d[mt][nt][3]);
                uint32_t* hp = hb + int64_t(nt * 4 + t4) * FN3;
                hp[s0] = P[mt][nt][0];
                hp[s0 + 8] = P[mt][nt][1];
            }
        }
        // forward z-DFT of this half-row: Y[c][j] = sum_z h[z][c] T[z][j]; the A operand
        // (channels x sites) is the transpose of the fragments above
        float e[2][3][4];
#pragma unroll
        for (int qq = 0; qq < 2; ++qq)
#pragma unroll
            for (int nt = 0; nt < 3; ++nt)
#pragma unroll
                for (int i = 0; i < 4; ++i) e[qq][nt][i] = 0.f;
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) {
            uint32_t A[2][4];
#pragma unroll
            for (int qq = 0; qq < 2; ++qq) {
                A[qq][0] = trans8(P[kk][2 * qq][0]);
                A[qq][1] = trans8(P[kk][2 * qq + 1][0]);
                A[qq][2] = trans8(P[kk][2 * qq][1]);
                A[qq][3] = trans8(P[kk][2 * qq + 1][1]);
            }
            const int zz = z0 + 16 * kk + 2 * t4;
#pragma unroll
            for (int nt = 0; nt < 3; ++nt) {
                const int j = nt * 8 + g;
                const uint32_t b0 = w32(a.tzt, j * 64 + zz), b1 = w32(a.tzt, j * 64 + zz + 8);
#pragma unroll
                for (int qq = 0; qq < 2; ++qq) mma(e[qq][nt], A[qq], b0, b1);
            }
        }
        // e[qq][nt]: channel 16 qq + g (+8 in e[2], e[3]), (re, im) of kz = 4 nt + t4
        if (half == 1) {
#pragma unroll
            for (int qq = 0; qq < 2; ++qq)
#pragma unroll
                for (int nt = 0; nt < 3; ++nt) {
                    red[r][16 * qq + g][4 * nt + t4] = make_float2(e[qq][nt][0], e[qq][nt][1]);
                    red[r][16 * qq + g + 8][4 * nt + t4] = make_float2(e[qq][nt][2], e[qq][nt][3]);
                }
        }
        __syncthreads();
        if (half == 0) {
#pragma unroll
            for (int qq = 0; qq < 2; ++qq)
#pragma unroll
                for (int nt = 0; nt < 3; ++nt) {
                    const int kz = 4 * nt + t4, c0 = 16 * qq + g;
                    const float2 u = red[r][c0][kz], v = red[r][c0 + 8][kz];
                    szbuf[c0][r * FM + kz] = pk(e[qq][nt][0] + u.x, e[qq][nt][1] + u.y);
                    szbuf[c0 + 8][r * FM + kz] = pk(e[qq][nt][2] + v.x, e[qq][nt][3] + v.y);
                }
        }
        __syncthreads();
        // the four rows of a channel are contiguous in SZ
        uint32_t* dst = a.sz + ((int64_t(b) * FC * FN + xcol) * FN + 4 * yg) * FM;
        for (int i = threadIdx.x; i < FC * 4 * FM; i += 256) {
            const int c = i / (4 * FM), k = i % (4 * FM);
            dst[int64_t(c) * FN * FN * FM + k] = szbuf[c][k];
        }
    }
}

// y DFT 64 -> 24 kept ky, per (b, c, 8 x-columns); warp w owns column x0 + w:
// out^T[kz][j] = sum_k A[kz][k] F[k][j], k = 2 y + s (the complex value in(y, kz)).
__global__ void __launch_bounds__(256) fno_ydft_fwd_kernel(const uint32_t* __restrict__ sz, uint32_t* __restrict__ sy,
                                                           const uint16_t* __restrict__ fwd, int B) {
    __shared__ uint32_t slab[8][ZSLAB];
    __shared__ uint32_t fs[48 * FWD_LD];
    __shared__ uint32_t obuf[NPK * 8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t4 = lane & 3;
    const int xg = blockIdx.x % 8, c = (blockIdx.x / 8) % FC, b = blockIdx.x / (8 * FC);
    const int x0 = 8 * xg;
    const uint4* src = reinterpret_cast<const uint4*>(sz + ((int64_t(b) * FC + c) * FN + x0) * ZSLAB);
    uint4* sl = reinterpret_cast<uint4*>(&slab[0][0]);
    for (int i = threadIdx.x; i < 8 * ZSLAB / 4; i += 256) sl[i] = src[i];
    const uint32_t* f32 = reinterpret_cast<const uint32_t*>(fwd);
    for (int i = threadIdx.x; i < 48 * 64; i += 256) fs[(i / 64) * FWD_LD + i % 64] = f32[i];
    __syncthreads();
    float d[6][4];
#pragma unroll
    for (int nt = 0; nt < 6; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) d[nt][q] = 0.f;
    const uint32_t* s = slab[warp];
    const bool lo = g < FM, hi = g + 8 < FM;
#pragma unroll
    for (int ks = 0; ks < 8; ++ks) {
        const int yy = 8 * ks + t4;
        const uint32_t A[4] = {lo ? s[yy * FM + g] : 0u, hi ? s[yy * FM + g + 8] : 0u,
                               lo ? s[(yy + 4) * FM + g] : 0u, hi ? s[(yy + 4) * FM + g + 8] : 0u};
#pragma unroll
        for (int nt = 0; nt < 6; ++nt) {
            const uint32_t* fr = fs + (nt * 8 + g) * FWD_LD + 8 * ks + t4;
            mma(d[nt], A, fr[0], fr[4]);
        }
    }
#pragma unroll
    for (int nt = 0; nt < 6; ++nt) {
        const int ky = 4 * nt + t4;
        if (lo) obuf[(ky * FM + g) * 8 + warp] = pk(d[nt][0], d[nt][1]);
        if (hi) obuf[(ky * FM + g + 8) * 8 + warp] = pk(d[nt][2], d[nt][3]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NPK * 8; i += 256) {
        const int p = i / 8, xi = i % 8;
        sy[((int64_t(p) * B + b) * FC + c) * FN + x0 + xi] = obuf[i];
    }
}

// y DFT 24 kept ky -> 64, per (b, c, 8 x-columns): out^T[kz][j] = sum_k A[kz][k] G[k][j],
// k = 2 ky' + s, j = 2 y + s'.
__global__ void __launch_bounds__(256) fno_ydft_inv_kernel(const uint32_t* __restrict__ sy, uint32_t* __restrict__ sz,
                                                           const uint16_t* __restrict__ inv, int B) {
    constexpr int IN_LD = NPK + 4;
    __shared__ uint32_t in[8 * IN_LD];
    __shared__ uint32_t gs[128 * INV_LD];
    __shared__ uint32_t obuf[8][ZSLAB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t4 = lane & 3;
    const int xg = blockIdx.x % 8, c = (blockIdx.x / 8) % FC, b = blockIdx.x / (8 * FC);
    const int x0 = 8 * xg;
    for (int i = threadIdx.x; i < NPK * 8; i += 256) {
        const int p = i / 8, xi = i % 8;
        in[xi * IN_LD + p] = sy[((int64_t(p) * B + b) * FC + c) * FN + x0 + xi];
    }
    const uint32_t* g32 = reinterpret_cast<const uint32_t*>(inv);
    for (int i = threadIdx.x; i < 128 * 24; i += 256) gs[(i / 24) * INV_LD + i % 24] = g32[i];
    __syncthreads();
    float d[16][4];
#pragma unroll
    for (int nt = 0; nt < 16; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) d[nt][q] = 0.f;
    const uint32_t* s = in + warp * IN_LD;
    const bool lo = g < FM, hi = g + 8 < FM;
#pragma unroll
    for (int ks = 0; ks < 3; ++ks) {
        const int ky = 8 * ks + t4;
        const uint32_t A[4] = {lo ? s[ky * FM + g] : 0u, hi ? s[ky * FM + g + 8] : 0u,
                               lo ? s[(ky + 4) * FM + g] : 0u, hi ? s[(ky + 4) * FM + g + 8] : 0u};
#pragma unroll
        for (int nt = 0; nt < 16; ++nt) {
            const uint32_t* gr = gs + (nt * 8 + g) * INV_LD + 8 * ks + t4;
            mma(d[nt], A, gr[0], gr[4]);
        }
    }
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
        const int yy = 4 * nt + t4;
        if (lo) obuf[warp][yy * FM + g] = pk(d[nt][0], d[nt][1]);
        if (hi) obuf[warp][yy * FM + g + 8] = pk(d[nt][2], d[nt][3]);
    }
    __syncthreads();
    uint4* dst = reinterpret_cast<uint4*>(sz + ((int64_t(b) * FC + c) * FN + x0) * ZSLAB);
    const uint4* ob = reinterpret_cast<const uint4*>(&obuf[0][0]);
    for (int i = threadIdx.x; i < 8 * ZSLAB / 4; i += 256) dst[i] = ob[i];
}

// x DFT of one kept (ky, kz) for 16 samples, the channel mixing of its 24 modes, and
// the inverse x DFT, in place on SY. Rows are (sample, channel), 64 x values each.
struct XmixSmem {
    uint32_t fs[48 * FWD_LD];
    uint32_t gs[128 * INV_LD];
    uint32_t hs[FK * HS_K];   // [kx'][sample][channel], padded strides
};

__global__ void __launch_bounds__(256) fno_xmix_kernel(uint32_t* __restrict__ sy, const uint16_t* __restrict__ wmix,
                                                       const uint16_t* __restrict__ fwd,
                                                       const uint16_t* __restrict__ inv, int B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    XmixSmem& sm = *reinterpret_cast<XmixSmem*>(smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t4 = lane & 3;
    const int p = blockIdx.x % NPK, b0 = 16 * (blockIdx.x / NPK);
    const int nb = B - b0 < 16 ? B - b0 : 16;
    uint32_t* base = sy + (int64_t(p) * B + b0) * FC * FN;   // row (sample, channel), x
    const uint32_t* f32 = reinterpret_cast<const uint32_t*>(fwd);
    for (int i = threadIdx.x; i < 48 * 64; i += 256) sm.fs[(i / 64) * FWD_LD + i % 64] = f32[i];
    const uint32_t* g32 = reinterpret_cast<const uint32_t*>(inv);
    for (int i = threadIdx.x; i < 128 * 24; i += 256) sm.gs[(i / 24) * INV_LD + i % 24] = g32[i];
    __syncthreads();

    // forward x DFT: H[row][j] = sum_k in[row][k] F[k][j]; 32 m-tiles of 16 rows, 4 per warp
    for (int i = 0; i < 4; ++i) {
        const int mt = warp + 8 * i;
        const int r0 = 16 * mt + g, r1 = r0 + 8;
        const bool v0 = r0 / FC < nb, v1 = r1 / FC < nb;
        float d[6][4];
#pragma unroll
        for (int nt = 0; nt < 6; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) d[nt][q] = 0.f;
#pragma unroll
        for (int ks = 0; ks < 8; ++ks) {
            const int xx = 8 * ks + t4;
            const uint32_t A[4] = {v0 ? base[r0 * FN + xx] : 0u, v1 ? base[r1 * FN + xx] : 0u,
                                   v0 ? base[r0 * FN + xx + 4] : 0u, v1 ? base[r1 * FN + xx + 4] : 0u};
#pragma unroll
            for (int nt = 0; nt < 6; ++nt) {
                const uint32_t* fr = sm.fs + (nt * 8 + g) * FWD_LD + 8 * ks + t4;
                mma(d[nt], A, fr[0], fr[4]);
            }
        }
#pragma unroll
        for (int nt = 0; nt < 6; ++nt) {
            const int kx = 4 * nt + t4;
            sm.hs[kx * HS_K + (r0 / FC) * HS_B + r0 % FC] = pk(d[nt][0], d[nt][1]);
            sm.hs[kx * HS_K + (r1 / FC) * HS_B + r1 % FC] = pk(d[nt][2], d[nt][3]);
        }
    }
    __syncthreads();

    // mixing, one kept kx per pass: Z[b][n] = sum_k H[b][k] M'[k][n], k = 2 i + s, n = 2 o + s'
    for (int i = 0; i < 3; ++i) {
        const int kx = warp + 8 * i;
        const uint16_t* wm = wmix + (int64_t(kx) * NPK + p) * (2 * FC) * (2 * FC);
        uint32_t* hk = sm.hs + kx * HS_K;
        uint32_t A[4][4];
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            A[ks][0] = hk[g * HS_B + 8 * ks + t4];
            A[ks][1] = hk[(g + 8) * HS_B + 8 * ks + t4];
            A[ks][2] = hk[g * HS_B + 8 * ks + 4 + t4];
            A[ks][3] = hk[(g + 8) * HS_B + 8 * ks + 4 + t4];
        }
        __syncwarp();
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            float z[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
                mma(z, A[ks], w32(wm, (nt * 8 + g) * 64 + 16 * ks + 2 * t4),
                    w32(wm, (nt * 8 + g) * 64 + 16 * ks + 8 + 2 * t4));
            const int o = 4 * nt + t4;
            hk[g * HS_B + o] = pk(z[0], z[1]);
            hk[(g + 8) * HS_B + o] = pk(z[2], z[3]);
        }
    }
    __syncthreads();

    // inverse x DFT: out[row][j] = sum_k Z[row][k] G[k][j], k = 2 kx' + s, j = 2 x + s'
    for (int i = 0; i < 4; ++i) {
        const int mt = warp + 8 * i;
        const int r0 = 16 * mt + g, r1 = r0 + 8;
        const int h0 = (r0 / FC) * HS_B + r0 % FC, h1 = (r1 / FC) * HS_B + r1 % FC;
        float d[16][4];
#pragma unroll
        for (int nt = 0; nt < 16; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) d[nt][q] = 0.f;
#pragma unroll
        for (int ks = 0; ks < 3; ++ks) {
            const int kx = 8 * ks + t4;
            const uint32_t A[4] = {sm.hs[kx * HS_K + h0], sm.hs[kx * HS_K + h1], sm.hs[(kx + 4) * HS_K + h0],
                                   sm.hs[(kx + 4) * HS_K + h1]};
#pragma unroll
            for (int nt = 0; nt < 16; ++nt) {
                const uint32_t* gr = sm.gs + (nt * 8 + g) * INV_LD + 8 * ks + t4;
                mma(d[nt], A, gr[0], gr[4]);
            }
        }
        const bool v0 = r0 / FC < nb, v1 = r1 / FC < nb;
#pragma unroll
        for (int nt = 0; nt < 16; ++nt) {
            const int xx = 4 * nt + t4;
            if (v0) base[r0 * FN + xx] = pk(d[nt][0], d[nt][1]);
            if (v1) base[r1 * FN + xx] = pk(d[nt][2], d[nt][3]);
        }
    }
}

// Wi[mode][n][k] = M'[k][n] with k = 2 i + s, n = 2 o + s' (interleaved real/imaginary):
// M'[2i][2o] = Rr, M'[2i+1][2o] = -Ri, M'[2i][2o+1] = Ri, M'[2i+1][2o+1] = Rr.
__global__ void pack_mix_interleaved_kernel(const float* __restrict__ R, __nv_bfloat16* __restrict__ Wi, int C,
                                            int nmodes) {
    const int K2 = 2 * C;
    const int64_t total = int64_t(nmodes) * K2 * K2;
    for (int64_t gi = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; gi < total;
         gi += int64_t(gridDim.x) * blockDim.x) {
        const int k = int(gi % K2), n = int((gi / K2) % K2);
        const int64_t mode = gi / (int64_t(K2) * K2);
        const int i = k >> 1, s = k & 1, o = n >> 1, so = n & 1;
        const float* rr = R + ((mode * C + i) * C + o) * 2;
        const float v = (s == so) ? rr[0] : (s == 1 ? -rr[1] : rr[1]);
        Wi[gi] = __float2bfloat16_rn(v);
    }
}

// dst[r][c] = src[r][c] as bf16 for r < rows, c < cols, zero elsewhere (rows_pad x cols_pad)
__global__ void to_bf16_kernel(const float* __restrict__ src, int rows, int cols, __nv_bfloat16* __restrict__ dst,
                               int rows_pad, int cols_pad) {
    const int n = rows_pad * cols_pad;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int r = i / cols_pad, c = i % cols_pad;
        dst[i] = __float2bfloat16_rn(r < rows && c < cols ? src[r * cols + c] : 0.f);
    }
}

int st(cudaError_t e) { return e == cudaSuccess ? WFS_OK : WFS_ERR_CUDA; }

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

int launch_zrow(int mode, ZrowArgs& a, cudaStream_t s) {
    const FastTables* t = fast_tables();
    if (!t) return WFS_ERR_CUDA;
    a.tz = t->tz;
    a.tzt = t->tzt;
    const unsigned grid = unsigned(a.B) * FN * 16;
    if (mode == ZROW_LIFT) fno_zrow_kernel<ZROW_LIFT><<<grid, 256, 0, s>>>(a);
    else if (mode == ZROW_LAYER) fno_zrow_kernel<ZROW_LAYER><<<grid, 256, 0, s>>>(a);
    else fno_zrow_kernel<ZROW_LAST><<<grid, 256, 0, s>>>(a);
    return st(cudaGetLastError());
}

}  // namespace
}  // namespace wfs

using namespace wfs;

extern "C" {

int wfs_fno_fast_lift(const void* x, const void* W0p, const float* b0, void* h, void* sz, int32_t B, void* stream) {
    if (!x || !W0p || !b0 || !h || !sz || B < 1 || !aligned16(sz)) return WFS_ERR_ARG;
    ZrowArgs a;
    std::memset(&a, 0, sizeof(a));
    a.x = static_cast<const float2*>(x);
    a.W = static_cast<const uint16_t*>(W0p);
    a.bias = b0;
    a.h_out = static_cast<uint32_t*>(h);
    a.sz = static_cast<uint32_t*>(sz);
    a.B = B;
    return launch_zrow(ZROW_LIFT, a, static_cast<cudaStream_t>(stream));
}

int wfs_fno_fast_layer(const void* h_in, void* sz, const void* W, const float* bias, void* h_out, int32_t B,
                       void* stream) {
    if (!h_in || !sz || !W || !bias || !h_out || h_in == h_out || B < 1 || !aligned16(sz)) return WFS_ERR_ARG;
    ZrowArgs a;
    std::memset(&a, 0, sizeof(a));
    a.h = static_cast<const uint32_t*>(h_in);
    a.sz = static_cast<uint32_t*>(sz);
    a.W = static_cast<const uint16_t*>(W);
    a.bias = bias;
    a.h_out = static_cast<uint32_t*>(h_out);
    a.B = B;
    return launch_zrow(ZROW_LAYER, a, static_cast<cudaStream_t>(stream));
}

int wfs_fno_fast_last(const void* h_in, const void* sz, const void* W, const float* bias, const void* Wq1,
                      const float* bq1, const void* Wq2p, const float* bq2, const void* prior, void* out, int32_t B,
                      void* stream) {
    if (!h_in || !sz || !W || !bias || !Wq1 || !bq1 || !Wq2p || !bq2 || !prior || !out || B < 1) return WFS_ERR_ARG;
    ZrowArgs a;
    std::memset(&a, 0, sizeof(a));
    a.h = static_cast<const uint32_t*>(h_in);
    a.sz = const_cast<uint32_t*>(static_cast<const uint32_t*>(sz));
    a.W = static_cast<const uint16_t*>(W);
    a.bias = bias;
    a.Wq1 = static_cast<const uint16_t*>(Wq1);
    a.bq1 = bq1;
    a.Wq2 = static_cast<const uint16_t*>(Wq2p);
    a.bq2 = bq2;
    a.prior = static_cast<const float2*>(prior);
    a.out = static_cast<float2*>(out);
    a.B = B;
    return launch_zrow(ZROW_LAST, a, static_cast<cudaStream_t>(stream));
}

int wfs_fno_fast_ydft(const void* src, void* dst, int32_t dir, int32_t B, void* stream) {
    if (!src || !dst || src == dst || B < 1 || (dir != -1 && dir != 1) || !aligned16(src) || !aligned16(dst))
        return WFS_ERR_ARG;
    const FastTables* t = fast_tables();
    if (!t) return WFS_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned grid = unsigned(B) * FC * 8;
    if (dir < 0)
        fno_ydft_fwd_kernel<<<grid, 256, 0, s>>>(static_cast<const uint32_t*>(src), static_cast<uint32_t*>(dst),
                                                 t->fwd, B);
    else
        fno_ydft_inv_kernel<<<grid, 256, 0, s>>>(static_cast<const uint32_t*>(src), static_cast<uint32_t*>(dst),
                                                 t->inv, B);
    return st(cudaGetLastError());
}

int wfs_fno_fast_xmix(void* sy, const void* Wi, int32_t B, void* stream) {
    if (!sy || !Wi || B < 1) return WFS_ERR_ARG;
    const FastTables* t = fast_tables();
    if (!t) return WFS_ERR_CUDA;
    static std::mutex mu;
    static std::map<int, bool> attr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return WFS_ERR_CUDA;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!attr[dev]) {
            if (cudaFuncSetAttribute(fno_xmix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(sizeof(XmixSmem))) != cudaSuccess)
                return WFS_ERR_CUDA;
            attr[dev] = true;
        }
    }
    const unsigned grid = unsigned(NPK) * unsigned((B + 15) / 16);
    fno_xmix_kernel<<<grid, 256, sizeof(XmixSmem), static_cast<cudaStream_t>(stream)>>>(
        static_cast<uint32_t*>(sy), static_cast<const uint16_t*>(Wi), t->fwd, t->inv, B);
    return st(cudaGetLastError());
}

int wfs_fno_pack_mix_interleaved(const float* R, void* Wi, int32_t C, int32_t nmodes, void* stream) {
    if (!R || !Wi || C < 1 || nmodes < 1) return WFS_ERR_ARG;
    const int64_t total = int64_t(nmodes) * 4 * C * C;
    const int grid = int(total / 256 + 1 < 152 * 16 ? total / 256 + 1 : 152 * 16);
    pack_mix_interleaved_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        R, static_cast<__nv_bfloat16*>(Wi), C, nmodes);
    return st(cudaGetLastError());
}

int wfs_fno_to_bf16(const float* src, int32_t rows, int32_t cols, void* dst, int32_t rows_pad, int32_t cols_pad,
                    void* stream) {
    if (!src || !dst || rows < 1 || cols < 1 || rows_pad < rows || cols_pad < cols) return WFS_ERR_ARG;
    const int n = rows_pad * cols_pad;
    to_bf16_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        src, rows, cols, static_cast<__nv_bfloat16*>(dst), rows_pad, cols_pad);
    return st(cudaGetLastError());
}

}  // extern "C"
