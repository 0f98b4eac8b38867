// fno_fast.cu — inference forward pass of the FNO surrogate on the kept modes only.
//
// The training forward (fno.cu) transforms every hidden field with full 64^3 FFTs and
// keeps FP32 activations: about 9 KB of HBM traffic per grid site and sample. A jump's
// correction is small against the prior it is added to (about 1e-2 of psi), so an
// inference pass can run every product on BF16 tensor cores with FP32 accumulation
// and keep its intermediates in BF16 without moving the jump's error. This file does
// that, and transforms only what the spectral layers use:
//
//   plane kernel   one CTA per (sample, x) plane: the inverse y and z DFTs of the
//                  layer's spectral branch, the pointwise 1x1 layer, bias and GELU, the
//                  BF16 store of h, and the forward z and y DFTs of the new h onto the
//                  kept (ky, kz), all on chip; h streams through shared memory by cp.async
//                  two row groups ahead. The lift (with the input normalisation) and the
//                  last layer with both projections are variants of the same kernel.
//   x+mix kernel   per kept (ky, kz) and 16 samples: the 64 -> 24 kept-kx DFT, the
//                  per-mode complex channel mixing Z = H R, and the 24 -> 64 inverse.
//
// The spectral mixing, the network's only dense contraction, runs on tcgen05.mma with
// FP32 accumulators in tensor memory; the DFTs and the pointwise layers are mma.sync
// m16n8k16 products (BF16 operands, FP32 accumulation) on BF16 constant matrices. Per
// layer a site moves its h in and out (128 B) and its share of the kept spectra four
// times (about 36 B), plus the mixing weights (56 MB per layer per 16 samples).
//
// Layouts (bf16x2 words: two channels, or the real and imaginary part of one value):
//   H   [B][16][64^3]                   channel pairs (2j, 2j+1), as the packed layout
//   SY  [B][64 x][24 ky][12 kz][32 c]   y- and z-spectra of each real channel, kept modes
// The kept modes follow include/wfs_fno.h: kx, ky in [0, 12) u [52, 64), kz in [0, 12);
// mode = (ix * 24 + iy) * 12 + iz. Geometry is fixed: N = 64, width 32, 12 modes.
#include <cuda_bf16.h>
#include <stdint.h>

#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/wfs.h"
#include "../../include/wfs_fno.h"
#include "bulk_copy.cuh"

namespace wfs {
namespace {

constexpr int FN = 64;                 // grid points per axis
constexpr int FC = 32;                 // hidden channels
constexpr int FM = 12;                 // kept kz
constexpr int FK = 24;                 // kept kx and ky
constexpr int64_t FN3 = int64_t(FN) * FN * FN;
constexpr int NPK = FK * FM;           // kept (ky, kz) pairs
constexpr int HS_B = 36;               // x+mix: words per sample row of the mode buffer
constexpr int HS_K = 584;              // x+mix: words per kept kx of the mode buffer

// BF16 constants of the kept-mode DFTs as per-lane mma fragments (one 16- or 8-byte load
// per fragment), per device. They are cut from four tables built on the host:
//   tz  [64 z][32 j]   j = 2 kz + (0: cos, 1: -sin), scaled by 1/8; j >= 24 zero
//   tzt [32 j][64 z]   the transpose of tz
//   fwd [48 j][128 k]  forward 64 -> 24 DFT, k = 2 n + s, j = 2 k' + s'
//   inv [128 j][48 k]  inverse 24 -> 64 DFT, k = 2 k' + s, j = 2 n + s'
struct FastTables {
    uint4* inv_a;    // [group 8][ks 3][lane]       inverse y DFT, rows re/im of the group's y
    uint4* fwd_a;    // [group 8][mt 3][lane]       forward y DFT, rows re/im of 8 ky', cols the group
    uint4* tz_a;     // [half 2][mt 2][ks 2][lane]  inverse z DFT over a warp's 32 sites
    uint2* tzt_b;    // [half 2][kk 2][nt 3][lane]  forward z DFT over a warp's 32 sites
    uint2* xf_b;     // [ks 8][nt 6][lane]          forward x DFT (B = fwd^T)
    uint2* xi_b;     // [ks 3][nt 16][lane]         inverse x DFT (B = inv^T)
};

std::mutex g_fast_mu;
std::map<int, FastTables> g_fast;
// limit of the mixing kernel's waits for its tensor-core commits (wfs_fno_set_wait_limit)
std::atomic<uint64_t> g_fno_wait_ns{1000000000ull};

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
    // fragments: A tile rows R[0..15] x cols K0..K0+15 of a [.][ld] table; B tile of a
    // table stored [n][k] (k contiguous), n = N0 + g, k = K0..K0+15
    auto word = [](const std::vector<uint16_t>& t, int ld, int row, int col) {
        return uint32_t(t[size_t(row) * ld + col]) | (uint32_t(t[size_t(row) * ld + col + 1]) << 16);
    };
    std::vector<uint32_t> frags;
    auto a_tile = [&](const std::vector<uint16_t>& t, int ld, const int* R, int K0) {
        for (int lane = 0; lane < 32; ++lane) {
            const int g = lane >> 2, t4 = lane & 3;
            frags.push_back(word(t, ld, R[g], K0 + 2 * t4));
            frags.push_back(word(t, ld, R[g + 8], K0 + 2 * t4));
            frags.push_back(word(t, ld, R[g], K0 + 8 + 2 * t4));
            frags.push_back(word(t, ld, R[g + 8], K0 + 8 + 2 * t4));
        }
    };
    auto b_tile = [&](const std::vector<uint16_t>& t, int ld, int N0, int K0) {
        for (int lane = 0; lane < 32; ++lane) {
            const int g = lane >> 2, t4 = lane & 3;
            frags.push_back(word(t, ld, N0 + g, K0 + 2 * t4));
            frags.push_back(word(t, ld, N0 + g, K0 + 8 + 2 * t4));
        }
    };
    int R[16];
    const size_t off_inv = frags.size();
    for (int grp = 0; grp < FN / 8; ++grp)
        for (int ks = 0; ks < 3; ++ks) {
            for (int i = 0; i < 8; ++i) R[i] = 2 * (8 * grp + i), R[i + 8] = 2 * (8 * grp + i) + 1;
            a_tile(inv, 48, R, 16 * ks);
        }
    const size_t off_fwd = frags.size();
    for (int grp = 0; grp < FN / 8; ++grp)
        for (int mt = 0; mt < 3; ++mt) {
            for (int i = 0; i < 8; ++i) R[i] = 2 * (8 * mt + i), R[i + 8] = 2 * (8 * mt + i) + 1;
            a_tile(fwd, 128, R, 16 * grp);
        }
    const size_t off_tz = frags.size();
    for (int half = 0; half < 2; ++half)
        for (int mt = 0; mt < 2; ++mt)
            for (int ks = 0; ks < 2; ++ks) {
                for (int i = 0; i < 16; ++i) R[i] = 32 * half + 16 * mt + i;
                a_tile(tz, 32, R, 16 * ks);
            }
    const size_t off_tzt = frags.size();
    for (int half = 0; half < 2; ++half)
        for (int kk = 0; kk < 2; ++kk)
            for (int nt = 0; nt < 3; ++nt) b_tile(tzt, 64, 8 * nt, 32 * half + 16 * kk);
    const size_t off_xf = frags.size();
    for (int ks = 0; ks < 8; ++ks)
        for (int nt = 0; nt < 6; ++nt) b_tile(fwd, 128, 8 * nt, 16 * ks);
    const size_t off_xi = frags.size();
    for (int ks = 0; ks < 3; ++ks)
        for (int nt = 0; nt < 16; ++nt) b_tile(inv, 48, 8 * nt, 16 * ks);
    uint32_t* fr = nullptr;
    if (cudaMalloc(&fr, frags.size() * sizeof(uint32_t)) != cudaSuccess) return nullptr;
    if (cudaMemcpy(fr, frags.data(), frags.size() * sizeof(uint32_t), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(fr);
        return nullptr;
    }
    FastTables t;
    t.inv_a = reinterpret_cast<uint4*>(fr + off_inv);
    t.fwd_a = reinterpret_cast<uint4*>(fr + off_fwd);
    t.tz_a = reinterpret_cast<uint4*>(fr + off_tz);
    t.tzt_b = reinterpret_cast<uint2*>(fr + off_tzt);
    t.xf_b = reinterpret_cast<uint2*>(fr + off_xf);
    t.xi_b = reinterpret_cast<uint2*>(fr + off_xi);
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
// GELU in its tanh form, x/2 (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))) (Hendrycks and
// Gimpel), on the hardware tanh: within 5e-4 of the erf form the network is trained with,
// below the BF16 rounding of every stored activation.
__device__ __forceinline__ float gelu(float x) {
    const float in = x * fmaf(0.0356774081f, x * x, 0.7978845608f);
    float t;
    asm("tanh.approx.f32 %0, %1;\n" : "=f"(t) : "f"(in));
    const float hx = 0.5f * x;
    return fmaf(hx, t, hx);
}
// 16-column blocks of BF16 weights in fragment order: dst column 4 t + e holds source
// column 2 t + e (e < 2) or 8 + 2 t + e - 2, so a lane's two B-fragment words (k = 2 t4,
// 2 t4 + 1 and 8 + 2 t4, 9 + 2 t4) are one 8-byte load.
__host__ __device__ __forceinline__ int frag_src_col(int d) {
    const int blk = d & ~15, t = (d & 15) >> 2, e = d & 3;
    return blk + (e < 2 ? 2 * t + e : 8 + 2 * t + e - 2);
}
__device__ __forceinline__ uint2 wfrag(const uint16_t* W, int ld, int n, int ks, int t4) {
    return *reinterpret_cast<const uint2*>(W + n * ld + 16 * ks + 4 * t4);
}

// ---------------------------------------------------------------------------
// Plane kernel: one CTA (16 warps) per (sample b, column x) owns the yz-plane of 64 z-rows
// and walks it in 8 groups of 8 rows. Per group, between two block barriers:
//   A. per warp (row r = w/2, sites z in [32 (w&1), +32)): the pointwise product W h and
//      the inverse z-DFT T . zs of the layer's spectral branch accumulate into one set of
//      fragments; bias, GELU, the BF16 store of the new h; the forward z-DFT of the new h
//      over the warp's 32 sites, as FP32 partial sums in red[half]
//   B. the forward y DFT of this group (the two half-rows' partials summed as they are
//      read) accumulates into the plane's new y-spectra (registers), and the inverse y DFT
//      of the next group's rows fills zs from the plane's y-spectra in shared memory
// The group's h arrives in shared memory by cp.async two groups ahead. After the last
// group the new y-spectra are stored over SY[b][x] (read whole at the start: in place).
// The lift reads psi and V instead of h and has no spectral branch; the last layer
// stops after the projections of step A.
// ---------------------------------------------------------------------------
constexpr int PT = 512;                 // threads per plane CTA
constexpr int GROWS = 8;                // z-rows per group
constexpr int NGROUP = FN / GROWS;
constexpr int SY_KS = FM * FC + 8;      // words per ky' of the plane's y-spectra in smem
constexpr int ZS_KZ = FC + 8;           // words per kz of a row's z-spectra
constexpr int ZS_Y = FM * ZS_KZ + 8;    // words per row of the group's z-spectra
constexpr int HS_P = GROWS * FN + 8;    // words per channel pair of the staged h
constexpr int SYW = NPK * FC;           // words of one plane's y-spectra in global memory
constexpr int RD_KZ = 2 * FC + 8;       // words per kz of a row's FP32 partial z-spectra (float2 per channel)
constexpr int RD_Y = FM * RD_KZ + 8;    // words per row of the partial z-spectra

struct PlaneSmem {
    uint32_t sy[FK * SY_KS];
    uint32_t zs[GROWS * ZS_Y];
    float red[2][GROWS * RD_Y];         // [half][row][kz][channel][re, im]
    uint32_t hs[2][(FC / 2) * HS_P];
};

struct PlaneArgs {
    const float2* psi;      // lift: field 0 (psi), sample stride psi_stride (complex values)
    const float2* V;        // lift: field 1 (V), sample stride v_stride
    int64_t psi_stride, v_stride;
    float vscale;           // lift: V is scaled by vscale
    const double* a2;       // lift: psi / s_b, last: prior + s_b net, s_b = sqrt(a2[b] / n3) (NULL: 1)
    const uint32_t* h;      // layer / last: H of the previous layer
    uint32_t* sy;           // SY: read (layer, last), written (lift, layer)
    const uint16_t* W;      // bf16 [32][16] (lift) or [32][32]
    const float* bias;
    const uint16_t* Wq1;    // last: [64][32]
    const float* bq1;
    const uint16_t* Wq2;    // last: [8][64], rows 2..7 zero
    const float* bq2;
    const float2* prior;    // last: [B][n3]
    uint32_t* h_out;        // lift / layer
    float2* out;            // last: [B][n3]
    double* out_norm;       // last, optional: += sum |out|^2 per sample
    const uint4* inv_a;
    const uint4* fwd_a;
    const uint4* tz_a;
    const uint2* tzt_b;
};

enum { PLANE_LIFT = 0, PLANE_LAYER = 1, PLANE_LAST = 2 };

__device__ __forceinline__ void cp16(void* smem, const void* gmem) {
    const unsigned s = unsigned(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

template <int MODE>
__global__ void __launch_bounds__(PT, 1) fno_plane_kernel(const PlaneArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PlaneSmem& sm = *reinterpret_cast<PlaneSmem*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t4 = lane & 3;
    const int xcol = blockIdx.x % FN, b = blockIdx.x / FN;
    const int r = warp >> 1, half = warp & 1, z0 = 32 * half;
    const int64_t plane0 = int64_t(xcol) * FN * FN;                  // site of (x, 0, 0)
    uint32_t* syg = a.sy + (int64_t(b) * FN + xcol) * SYW;           // SY[b][x]
    float s_b = 1.0f;
    if ((MODE == PLANE_LIFT || MODE == PLANE_LAST) && a.a2) s_b = float(sqrt(a.a2[b] / double(FN3)));

    // staging of one group's input: h (16 pairs x 512 sites) or psi and V (2 x 512 values)
    auto stage = [&](int grp) {
        if (grp < NGROUP) {
            const int64_t s0 = plane0 + int64_t(grp) * GROWS * FN;
            uint32_t* dst = sm.hs[grp & 1];
            if constexpr (MODE == PLANE_LIFT) {
                // 2 fields x 512 complex values = 2 x 256 chunks of 16 B
                const int f = tid >> 8, ch = tid & 255;
                const float2* src = f == 0 ? a.psi + int64_t(b) * a.psi_stride : a.V + int64_t(b) * a.v_stride;
                cp16(dst + f * HS_P * 2 + ch * 4, src + s0 + ch * 2);
            } else {
                const uint32_t* hb = a.h + int64_t(b) * (FC / 2) * FN3;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int k = tid + PT * i, pr = k >> 7, ch = k & 127;
                    cp16(dst + pr * HS_P + ch * 4, hb + int64_t(pr) * FN3 + s0 + ch * 4);
                }
            }
        }
        cp_commit();
    };
    if constexpr (MODE != PLANE_LIFT) {
        for (int k = tid; k < SYW / 4; k += PT) {
            const int p = (k * 4) / FC, c = (k * 4) % FC;   // p = ky' * 12 + kz
            cp16(sm.sy + (p / FM) * SY_KS + (p % FM) * FC + c, syg + k * 4);
        }
    }
    stage(0);
    stage(1);

    float acc[3][3][4];   // new y-spectra: m-tile (8 ky': re rows, im rows) x this warp's 3 n-tiles
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;

    // inverse y DFT of group grp: zs[row][kz][c] = sum_ky' G[y][ky'] SY[ky'][kz][c] (interleaved
    // rows: re of y0+g in rows 0-7, im in rows 8-15); warp w owns n-tiles 3w..3w+2 of (kz, c)
    auto inverse_y = [&](int grp) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int nt = 3 * warp + j, kz = nt >> 2, c = (nt & 3) * 8 + g;
            float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int ks = 0; ks < 3; ++ks) {
                const uint4 f = a.inv_a[(grp * 3 + ks) * 32 + lane];
                const uint32_t A[4] = {f.x, f.y, f.z, f.w};
                const int ky = 8 * ks + t4;
                mma(d, A, sm.sy[ky * SY_KS + kz * FC + c], sm.sy[(ky + 4) * SY_KS + kz * FC + c]);
            }
            const int cc = (nt & 3) * 8 + 2 * t4;
            sm.zs[g * ZS_Y + kz * ZS_KZ + cc] = pk(d[0], d[2]);
            sm.zs[g * ZS_Y + kz * ZS_KZ + cc + 1] = pk(d[1], d[3]);
        }
    };
    if constexpr (MODE != PLANE_LIFT) {
        cp_wait1();
        __syncthreads();   // sy and group 0's h have landed
        inverse_y(0);
    } else {
        cp_wait1();
    }

    for (int grp = 0; grp < NGROUP; ++grp) {
        const int y0 = grp * GROWS;
        const uint32_t* hs = sm.hs[grp & 1];
        __syncthreads();   // this group's h and zs are ready; red is free

        // A. pointwise + inverse z-DFT for this warp's 32 sites
        const int rowsite = r * FN + z0;   // local site of the warp's first z
        float d[2][4][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                for (int q = 0; q < 4; ++q) d[mt][nt][q] = 0.f;
        if constexpr (MODE == PLANE_LIFT) {
            // channels (Re psi / s, Im psi / s) in pair 0, (Re V vs, Im V vs) in pair 1
            const float sc = t4 == 0 ? 1.0f / s_b : a.vscale;
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                uint32_t A[4] = {0u, 0u, 0u, 0u};
                if (t4 < 2) {
                    const uint32_t* f = hs + t4 * HS_P * 2;   // field t4, two words per value
                    const int s0 = rowsite + 16 * mt + g;
                    A[0] = pk(__uint_as_float(f[2 * s0]) * sc, __uint_as_float(f[2 * s0 + 1]) * sc);
                    A[1] = pk(__uint_as_float(f[2 * s0 + 16]) * sc, __uint_as_float(f[2 * s0 + 17]) * sc);
                }
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const uint2 w = wfrag(a.W, 16, nt * 8 + g, 0, t4);
                    mma(d[mt][nt], A, w.x, w.y);
                }
            }
        } else {
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {
                uint2 Bw[4];
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) Bw[nt] = wfrag(a.W, 32, nt * 8 + g, ks, t4);
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) {
                    const int s0 = rowsite + 16 * mt + g;
                    const uint32_t* p0 = hs + (8 * ks + t4) * HS_P;
                    const uint32_t* p1 = p0 + 4 * HS_P;
                    const uint32_t A[4] = {p0[s0], p0[s0 + 8], p1[s0], p1[s0 + 8]};
#pragma unroll
                    for (int nt = 0; nt < 4; ++nt) mma(d[mt][nt], A, Bw[nt].x, Bw[nt].y);
                }
            }
            const uint32_t* zr = sm.zs + r * ZS_Y;
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {
                uint32_t At[2][4];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) {
                    const uint4 f = a.tz_a[((half * 2 + mt) * 2 + ks) * 32 + lane];
                    At[mt][0] = f.x;
                    At[mt][1] = f.y;
                    At[mt][2] = f.z;
                    At[mt][3] = f.w;
                }
                const int kz0 = 8 * ks + t4, kz1 = kz0 + 4;
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const int c = nt * 8 + g;
                    const uint32_t b0 = kz0 < FM ? zr[kz0 * ZS_KZ + c] : 0u;
                    const uint32_t b1 = kz1 < FM ? zr[kz1 * ZS_KZ + c] : 0u;
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt) mma(d[mt][nt], At[mt], b0, b1);
                }
            }
        }
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const float c0 = a.bias[nt * 8 + 2 * t4], c1 = a.bias[nt * 8 + 2 * t4 + 1];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                d[mt][nt][0] += c0;
                d[mt][nt][1] += c1;
                d[mt][nt][2] += c0;
                d[mt][nt][3] += c1;
                if constexpr (MODE == PLANE_LAYER) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) d[mt][nt][q] = gelu(d[mt][nt][q]);
                }
            }
        }

        const int64_t gsite = plane0 + int64_t(y0 + r) * FN + z0;   // global site of the warp's first z
        if constexpr (MODE == PLANE_LAST) {
            // out = prior + s_b (Wq2 GELU(Wq1 h + bq1) + bq2), chained through the fragments
            float nsum = 0.f;
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
                    for (int ks = 0; ks < 2; ++ks) {
                        const uint2 w = wfrag(a.Wq1, 32, nt * 8 + g, ks, t4);
                        mma(q[nt], A1[ks], w.x, w.y);
                    }
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
                    const uint2 w = wfrag(a.Wq2, 64, g, ks, t4);
                    mma(o, A2, w.x, w.y);
                }
                if (t4 == 0) {
                    const int64_t s0 = int64_t(b) * FN3 + gsite + 16 * mt + g;
                    const float2 p0 = a.prior[s0], p1 = a.prior[s0 + 8];
                    const float2 v0 = make_float2(fmaf(s_b, o[0] + a.bq2[0], p0.x), fmaf(s_b, o[1] + a.bq2[1], p0.y));
                    const float2 v1 = make_float2(fmaf(s_b, o[2] + a.bq2[0], p1.x), fmaf(s_b, o[3] + a.bq2[1], p1.y));
                    a.out[s0] = v0;
                    a.out[s0 + 8] = v1;
                    nsum += v0.x * v0.x + v0.y * v0.y + v1.x * v1.x + v1.y * v1.y;
                }
            }
            if (a.out_norm) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) nsum += __shfl_xor_sync(0xffffffffu, nsum, o);
                if (lane == 0) atomicAdd(a.out_norm + b, double(nsum));
            }
        } else {
            // store h (BF16 channel pairs) and keep the packed fragments for the z-DFT
            uint32_t P[2][4][2];
            uint32_t* hb = a.h_out + int64_t(b) * (FC / 2) * FN3;
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int64_t s0 = gsite + 16 * mt + g;
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    P[mt][nt][0] = pk(d[mt][nt][0], d[mt][nt][1]);
                    P[mt][nt][1] = pk(d[mt][nt][2], d[mt][nt][3]);
                    uint32_t* hp = hb + int64_t(nt * 4 + t4) * FN3;
                    hp[s0] = P[mt][nt][0];
                    hp[s0 + 8] = P[mt][nt][1];
                }
            }
            // forward z-DFT over the warp's 32 sites: Y[c][j] = sum_z h[z][c] T[z][j]; the A
            // operand (channels x sites) is the transpose of the fragments above
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
#pragma unroll
                for (int nt = 0; nt < 3; ++nt) {
                    const uint2 bz = a.tzt_b[((half * 2 + kk) * 3 + nt) * 32 + lane];
#pragma unroll
                    for (int qq = 0; qq < 2; ++qq) mma(e[qq][nt], A[qq], bz.x, bz.y);
                }
            }
            // e[qq][nt]: channel 16 qq + g (+8 in e[2], e[3]), (re, im) of kz = 4 nt + t4
            float* rd = sm.red[half] + r * RD_Y;
#pragma unroll
            for (int qq = 0; qq < 2; ++qq)
#pragma unroll
                for (int nt = 0; nt < 3; ++nt) {
                    float* p = rd + (4 * nt + t4) * RD_KZ + 2 * (16 * qq + g);
                    *reinterpret_cast<float2*>(p) = make_float2(e[qq][nt][0], e[qq][nt][1]);
                    *reinterpret_cast<float2*>(p + 16) = make_float2(e[qq][nt][2], e[qq][nt][3]);
                }
        }
        __syncthreads();   // red ready; this group's h buffer and zs are free
        stage(grp + 2);
        if constexpr (MODE != PLANE_LAST) {
            // B. forward y DFT over the group's rows: acc[ky'][n] += sum_y F[y][ky'] Y[y][n]
            //    (interleaved rows: re of ky' = 8 mt + g in rows 0-7, im in rows 8-15), with
            //    Y the sum of the two half-rows' partials
            uint32_t Bf[3][2];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int nt = 3 * warp + j, kz = nt >> 2, c = (nt & 3) * 8 + g;
#pragma unroll
                for (int h2 = 0; h2 < 2; ++h2) {
                    const int off = (t4 + 4 * h2) * RD_Y + kz * RD_KZ + 2 * c;
                    const float2 u = *reinterpret_cast<const float2*>(sm.red[0] + off);
                    const float2 v = *reinterpret_cast<const float2*>(sm.red[1] + off);
                    Bf[j][h2] = pk(u.x + v.x, u.y + v.y);
                }
            }
#pragma unroll
            for (int mt = 0; mt < 3; ++mt) {
                const uint4 f = a.fwd_a[(grp * 3 + mt) * 32 + lane];
                const uint32_t A[4] = {f.x, f.y, f.z, f.w};
#pragma unroll
                for (int j = 0; j < 3; ++j) mma(acc[mt][j], A, Bf[j][0], Bf[j][1]);
            }
        }
        if constexpr (MODE != PLANE_LIFT) {
            if (grp + 1 < NGROUP) inverse_y(grp + 1);
        }
        cp_wait1();   // the next group's h has landed (visible after the next barrier)
    }

    if constexpr (MODE != PLANE_LAST) {
        // the plane's new y-spectra: (re, im) of ky' = 8 mt + g at n and n+1
#pragma unroll
        for (int mt = 0; mt < 3; ++mt)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int nt = 3 * warp + j, kz = nt >> 2, c = (nt & 3) * 8 + 2 * t4;
                const int ky = 8 * mt + g;
                uint2 v = make_uint2(pk(acc[mt][j][0], acc[mt][j][2]), pk(acc[mt][j][1], acc[mt][j][3]));
                *reinterpret_cast<uint2*>(syg + (ky * FM + kz) * FC + c) = v;
            }
    }
}

// x DFT of one kept (ky, kz) for 16 samples, the channel mixing of its 24 modes on the
// fifth-generation tensor cores, and the inverse x DFT, in place on SY. Rows are (sample,
// channel), 64 x values each; a row's values lie SYW words apart (SY is [b][x][(ky', kz)][c]).
//
// Mixing, per pair of kept kx (modes m1, m2): D[128][16] = A[128][128] x B[128][16] with
//   A = [[W1, 0], [0, W2]] (W = the mode's 64 x 64 BF16 block, output feature x input
//   component, columns in fragment order), B = [H1^T; H2^T] (input components x samples),
// one tcgen05.mma chain of 8 K=16 steps, FP32 accumulation in tensor memory (16 columns
// per pair, lane = output feature). Operands sit in shared memory in the no-swizzle
// K-major layout: 8-row x 16-byte core matrices, K-adjacent ones 128 B apart (leading
// byte offset), 8-row groups 1024 B apart (stride byte offset). The zero blocks of A are
// one 8 KB zero region between W1 and W2: for the first four K steps the descriptor
// starts at W1 (rows 64-127 then read the zeros), for the last four at the zeros (rows
// 0-63) followed by W2. One thread issues the MMAs and commits them to an mbarrier per
// operand buffer; the buffers alternate so that staging the next pair overlaps the
// current pair's MMAs. Waits are bounded (wfs_fno_set_wait_limit): a wait that gives up
// marks the CTA's results NaN (the jump then fails its acceptance test and is rerun
// exactly), drains the MMAs still in flight (bounded again), frees the tensor memory and
// returns.
constexpr int XM_TMEM_COLS = 256;       // 12 pairs x 16 columns, rounded to a power of two
constexpr int XM_A_BYTES = 3 * 8192;    // W1 | zeros | W2
constexpr int XM_B_BYTES = 2 * 2048;    // H1^T | H2^T

struct XmixSmem {
    unsigned char a[2][XM_A_BYTES];     // 1024-byte aligned operand buffers first
    unsigned char bop[2][XM_B_BYTES];
    uint32_t hs[FK * HS_K];             // [kx'][sample][channel], padded strides
    unsigned long long bar[3];          // commits per operand buffer; [2]: all MMAs of the CTA
    uint32_t tmem_base;
    int failed;
};

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    // start address >> 4 | leading byte offset 128 >> 4 | stride byte offset 1024 >> 4 | version 1
    return uint64_t((saddr & 0x3FFFFu) >> 4) | (uint64_t(128 >> 4) << 16) | (uint64_t(1024 >> 4) << 32) |
           (uint64_t(1) << 46);
}
// kind::f16 instruction descriptor: F32 accumulator, BF16 A and B, both K-major, N = 16, M = 128
constexpr uint32_t kMixIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(kMixIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                 : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }

__global__ void __launch_bounds__(256, 2) fno_xmix_kernel(uint32_t* __restrict__ sy, const uint16_t* __restrict__ wmix,
                                                       const uint2* __restrict__ xf_b,
                                                       const uint2* __restrict__ xi_b, int B, uint64_t wait_ns) {
    extern __shared__ __align__(1024) unsigned char smem_xm[];   // no static shared memory: starts at 0
    XmixSmem& sm = *reinterpret_cast<XmixSmem*>(smem_xm);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t4 = lane & 3;
    const int p = blockIdx.x % NPK, b0 = 16 * (blockIdx.x / NPK);
    const int nb = B - b0 < 16 ? B - b0 : 16;
    uint32_t* base = sy + p * FC;
    auto at = [&](int row, int xx) { return (int64_t(b0 + row / FC) * FN + xx) * SYW + row % FC; };

    // tensor memory (warp 0), the two commit barriers, zero regions of A
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         smem_addr(&sm.tmem_base)),
                     "r"(XM_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(smem_addr(&sm.bar[0]), 1);
        mbar_init(smem_addr(&sm.bar[1]), 1);
        mbar_init(smem_addr(&sm.bar[2]), 1);
        mbar_init_fence();
        sm.failed = 0;
    }
    for (int i = tid; i < 8192 / 16; i += 256) {
        reinterpret_cast<uint4*>(sm.a[0] + 8192)[i] = make_uint4(0u, 0u, 0u, 0u);
        reinterpret_cast<uint4*>(sm.a[1] + 8192)[i] = make_uint4(0u, 0u, 0u, 0u);
    }

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
#pragma unroll 4
        for (int ks = 0; ks < 8; ++ks) {
            const int xx = 8 * ks + t4;
            const uint32_t A[4] = {v0 ? base[at(r0, xx)] : 0u, v1 ? base[at(r1, xx)] : 0u,
                                   v0 ? base[at(r0, xx + 4)] : 0u, v1 ? base[at(r1, xx + 4)] : 0u};
#pragma unroll
            for (int nt = 0; nt < 6; ++nt) {
                const uint2 f = xf_b[(ks * 6 + nt) * 32 + lane];
                mma(d[nt], A, f.x, f.y);
            }
        }
#pragma unroll
        for (int nt = 0; nt < 6; ++nt) {
            const int kx = 4 * nt + t4;
            sm.hs[kx * HS_K + (r0 / FC) * HS_B + r0 % FC] = pk(d[nt][0], d[nt][1]);
            sm.hs[kx * HS_K + (r1 / FC) * HS_B + r1 % FC] = pk(d[nt][2], d[nt][3]);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sm.tmem_base;

    // mixing on the tensor cores, one pair of kept kx per step; the weights of pair j + 1
    // are copied while pair j is staged and multiplied
    constexpr int NPAIR = FK / 2;
    bool ok = true;
    auto stage_weights = [&](int j) {   // modes (2j, 2j+1): 2 x 64 rows x 8 chunks of 16 bytes
        if (j < NPAIR) {
            const int u = j & 1;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int c = tid + 256 * i, half = c >> 9, rem = c & 511, n = rem >> 3, kc = rem & 7;
                const int kx = 2 * j + half;
                const uint16_t* src = wmix + ((int64_t(kx) * NPK + p) * 64 + n) * 64 + kc * 8;
                cp16(sm.a[u] + half * 16384 + (n >> 3) * 1024 + kc * 128 + (n & 7) * 16, src);
            }
        }
        cp_commit();
    };
    stage_weights(0);
    for (int j = 0; j < NPAIR; ++j) {
        const int u = j & 1;
        // buffer 1 - u was read by the MMAs of pair j - 1: wait for them before refilling it
        if (j >= 1 && !mbar_wait_bounded(smem_addr(&sm.bar[1 - u]), uint32_t(((j - 1) >> 1) & 1), wait_ns))
            ok = false;
        stage_weights(j + 1);
        // activations: H^T of both modes, 16 samples x 8 chunks of 16 bytes each, in the
        // weights' column order (fragment order within each 16-column block)
        {
            const int half = tid >> 7, rem = tid & 127, bb = rem >> 3, kc = rem & 7;
            const uint32_t* hk = sm.hs + (2 * j + half) * HS_K + bb * HS_B + 8 * (kc >> 1);
            const uint4 v = (kc & 1) ? make_uint4(hk[2], hk[6], hk[3], hk[7]) : make_uint4(hk[0], hk[4], hk[1], hk[5]);
            *reinterpret_cast<uint4*>(sm.bop[u] + half * 2048 + (bb >> 3) * 1024 + kc * 128 + (bb & 7) * 16) = v;
        }
        cp_wait1();   // pair j's weights have landed (pair j + 1's may still be in flight)
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = smem_addr(sm.a[u]), bq = smem_addr(sm.bop[u]);
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
                const uint32_t aa = kk < 4 ? a0 + kk * 256 : a0 + 8192 + (kk - 4) * 256;
                const uint32_t ba = kk < 4 ? bq + kk * 256 : bq + 2048 + (kk - 4) * 256;
                umma_bf16(tmem + uint32_t(16 * j), umma_desc(aa), umma_desc(ba), kk > 0 ? 1u : 0u);
            }
            umma_commit(smem_addr(&sm.bar[u]));
        }
    }
    // one more commit, on its own barrier, covers every MMA of the CTA; after a wait that gave
    // up, the MMAs still in flight are drained (bounded by the default limit) before the
    // tensor memory is read or freed
    if (tid == 0) umma_commit(smem_addr(&sm.bar[2]));
    const bool done = mbar_wait_bounded(smem_addr(&sm.bar[2]), 0u, wait_ns);
    if (!ok || !done) atomicOr(&sm.failed, 1);
    if (!done) mbar_wait_bounded(smem_addr(&sm.bar[2]), 0u, kWaitLimitNs);
    tc_fence_after();
    // read D back: warp w reads lanes 32 (w % 4) .. +31 (output features) of pairs
    // 6 (w / 4) .. +5; lane 2o holds the real part of output o, lane 2o+1 the imaginary part
    {
        const int q4 = warp & 3, r = 32 * q4 + lane, half = r >> 6, n = r & 63;
#pragma unroll 1
        for (int jj = 0; jj < NPAIR / 2; ++jj) {
            const int j = (warp >> 2) * (NPAIR / 2) + jj;
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(tmem + (uint32_t(32 * q4) << 16) + uint32_t(16 * j)));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            uint32_t* hk = sm.hs + (2 * j + half) * HS_K + (n >> 1);
#pragma unroll
            for (int bb = 0; bb < 16; ++bb) {
                const float re = __uint_as_float(v[bb]);
                const float im = __shfl_down_sync(0xffffffffu, re, 1);
                if (!(n & 1)) hk[bb * HS_B] = pk(re, im);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(XM_TMEM_COLS)
                     : "memory");
    }
    const bool failed = sm.failed != 0;

    // inverse x DFT: out[row][j] = sum_k Z[row][k] G[k][j], k = 2 kx' + s, j = 2 x + s'; each
    // m-tile in two halves of 8 n-tiles (32 x values) so that fragments and sums fit in registers
    const uint32_t nanw = 0x7FC07FC0u;
    for (int i = 0; i < 8; ++i) {
        const int mt = warp + 8 * (i >> 1), nh = i & 1;
        const int r0 = 16 * mt + g, r1 = r0 + 8;
        const int h0 = (r0 / FC) * HS_B + r0 % FC, h1 = (r1 / FC) * HS_B + r1 % FC;
        float d[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) d[nt][q] = 0.f;
#pragma unroll
        for (int ks = 0; ks < 3; ++ks) {
            const int kx = 8 * ks + t4;
            const uint32_t A[4] = {sm.hs[kx * HS_K + h0], sm.hs[kx * HS_K + h1], sm.hs[(kx + 4) * HS_K + h0],
                                   sm.hs[(kx + 4) * HS_K + h1]};
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const uint2 f = xi_b[(ks * 16 + 8 * nh + nt) * 32 + lane];
                mma(d[nt], A, f.x, f.y);
            }
        }
        const bool v0 = r0 / FC < nb, v1 = r1 / FC < nb;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int xx = 4 * (8 * nh + nt) + t4;
            if (v0) base[at(r0, xx)] = failed ? nanw : pk(d[nt][0], d[nt][1]);
            if (v1) base[at(r1, xx)] = failed ? nanw : pk(d[nt][2], d[nt][3]);
        }
    }
}

// Wi[mode][n][d] = M'[k][n], k = frag_src_col(d), with k = 2 i + s, n = 2 o + s'
// (interleaved real/imaginary): M'[2i][2o] = Rr, M'[2i+1][2o] = -Ri, M'[2i][2o+1] = Ri,
// M'[2i+1][2o+1] = Rr.
__global__ void pack_mix_interleaved_kernel(const float* __restrict__ R, __nv_bfloat16* __restrict__ Wi, int C,
                                            int nmodes) {
    const int K2 = 2 * C;
    const int64_t total = int64_t(nmodes) * K2 * K2;
    for (int64_t gi = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; gi < total;
         gi += int64_t(gridDim.x) * blockDim.x) {
        const int k = frag_src_col(int(gi % K2)), n = int((gi / K2) % K2);
        const int64_t mode = gi / (int64_t(K2) * K2);
        const int i = k >> 1, s = k & 1, o = n >> 1, so = n & 1;
        const float* rr = R + ((mode * C + i) * C + o) * 2;
        const float v = (s == so) ? rr[0] : (s == 1 ? -rr[1] : rr[1]);
        Wi[gi] = __float2bfloat16_rn(v);
    }
}

// dst[r][c] = src[r][c'] as bf16 for r < rows, c' < cols, zero elsewhere (rows_pad x
// cols_pad); c' = c, or frag_src_col(c) in fragment order
__global__ void to_bf16_kernel(const float* __restrict__ src, int rows, int cols, __nv_bfloat16* __restrict__ dst,
                               int rows_pad, int cols_pad, int frag) {
    const int n = rows_pad * cols_pad;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int r = i / cols_pad, c = frag ? frag_src_col(i % cols_pad) : i % cols_pad;
        dst[i] = __float2bfloat16_rn(r < rows && c < cols ? src[r * cols + c] : 0.f);
    }
}

int st(cudaError_t e) { return e == cudaSuccess ? WFS_OK : WFS_ERR_CUDA; }

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

template <int MODE>
int launch_plane(PlaneArgs& a, int B, cudaStream_t s) {
    const FastTables* t = fast_tables();
    if (!t) return WFS_ERR_CUDA;
    a.inv_a = t->inv_a;
    a.fwd_a = t->fwd_a;
    a.tz_a = t->tz_a;
    a.tzt_b = t->tzt_b;
    static std::mutex mu;
    static std::map<int, bool> attr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return WFS_ERR_CUDA;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!attr[dev]) {
            if (cudaFuncSetAttribute(fno_plane_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(sizeof(PlaneSmem))) != cudaSuccess)
                return WFS_ERR_CUDA;
            attr[dev] = true;
        }
    }
    fno_plane_kernel<MODE><<<unsigned(B) * FN, PT, sizeof(PlaneSmem), s>>>(a);
    return st(cudaGetLastError());
}

}  // namespace
}  // namespace wfs

using namespace wfs;

extern "C" {

int wfs_fno_fast_lift(const void* psi, int64_t psi_stride, const void* V, int64_t v_stride, float vscale,
                      const double* a2, const void* W0p, const float* b0, void* h, void* sy, int32_t B,
                      void* stream) {
    if (!psi || !V || !W0p || !b0 || !h || !sy || B < 1 || !aligned16(psi) || !aligned16(V) || !aligned16(h) ||
        !aligned16(sy) || (psi_stride & 1) || (v_stride & 1))
        return WFS_ERR_ARG;
    PlaneArgs a;
    std::memset(&a, 0, sizeof(a));
    a.psi = static_cast<const float2*>(psi);
    a.V = static_cast<const float2*>(V);
    a.psi_stride = psi_stride;
    a.v_stride = v_stride;
    a.vscale = vscale;
    a.a2 = a2;
    a.W = static_cast<const uint16_t*>(W0p);
    a.bias = b0;
    a.h_out = static_cast<uint32_t*>(h);
    a.sy = static_cast<uint32_t*>(sy);
    return launch_plane<PLANE_LIFT>(a, B, static_cast<cudaStream_t>(stream));
}

int wfs_fno_fast_layer(const void* h_in, void* sy, const void* W, const float* bias, void* h_out, int32_t B,
                       void* stream) {
    if (!h_in || !sy || !W || !bias || !h_out || h_in == h_out || B < 1 || !aligned16(h_in) || !aligned16(sy))
        return WFS_ERR_ARG;
    PlaneArgs a;
    std::memset(&a, 0, sizeof(a));
    a.h = static_cast<const uint32_t*>(h_in);
    a.sy = static_cast<uint32_t*>(sy);
    a.W = static_cast<const uint16_t*>(W);
    a.bias = bias;
    a.h_out = static_cast<uint32_t*>(h_out);
    return launch_plane<PLANE_LAYER>(a, B, static_cast<cudaStream_t>(stream));
}

int wfs_fno_fast_last(const void* h_in, const void* sy, const void* W, const float* bias, const void* Wq1,
                      const float* bq1, const void* Wq2p, const float* bq2, const void* prior, const double* a2,
                      void* out, double* out_norm, int32_t B, void* stream) {
    if (!h_in || !sy || !W || !bias || !Wq1 || !bq1 || !Wq2p || !bq2 || !prior || !out || B < 1 ||
        !aligned16(h_in) || !aligned16(sy))
        return WFS_ERR_ARG;
    PlaneArgs a;
    std::memset(&a, 0, sizeof(a));
    a.h = static_cast<const uint32_t*>(h_in);
    a.sy = const_cast<uint32_t*>(static_cast<const uint32_t*>(sy));
    a.W = static_cast<const uint16_t*>(W);
    a.bias = bias;
    a.Wq1 = static_cast<const uint16_t*>(Wq1);
    a.bq1 = bq1;
    a.Wq2 = static_cast<const uint16_t*>(Wq2p);
    a.bq2 = bq2;
    a.prior = static_cast<const float2*>(prior);
    a.a2 = a2;
    a.out = static_cast<float2*>(out);
    a.out_norm = out_norm;
    return launch_plane<PLANE_LAST>(a, B, static_cast<cudaStream_t>(stream));
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
        static_cast<uint32_t*>(sy), static_cast<const uint16_t*>(Wi), t->xf_b, t->xi_b, B,
        g_fno_wait_ns.load(std::memory_order_relaxed));
    return st(cudaGetLastError());
}

int wfs_fno_set_wait_limit(double seconds) {
    if (!(seconds >= 0.0) || seconds > 60.0) return WFS_ERR_ARG;
    g_fno_wait_ns.store(uint64_t(seconds * 1e9), std::memory_order_relaxed);
    return WFS_OK;
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
                    int32_t frag_order, void* stream) {
    if (!src || !dst || rows < 1 || cols < 1 || rows_pad < rows || cols_pad < cols || (frag_order && (cols_pad & 15)))
        return WFS_ERR_ARG;
    const int n = rows_pad * cols_pad;
    to_bf16_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        src, rows, cols, static_cast<__nv_bfloat16*>(dst), rows_pad, cols_pad, frag_order ? 1 : 0);
    return st(cudaGetLastError());
}

}  // extern "C"
