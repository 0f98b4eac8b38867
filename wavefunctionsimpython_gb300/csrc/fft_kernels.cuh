// fft_kernels.cuh — pencil FFT passes for the split-operator propagator.
//
// A pencil of length L = P*Q is transformed by T = max(P, Q) threads in two
// register-resident stages with a single shared-memory transpose between
// them (the "four-step" factorisation):
//   stage 1: thread n1 < P holds x[n1 + P*n2] (n2 < Q), does a Q-point DFT,
//            multiplies by w_L^(n1*k2)          -> A[n1][k2]
//   stage 2: thread k2 < Q gathers A[.][k2], does a P-point DFT
//            -> holds X[k2 + Q*k1] (k1 < P).
// The inverse with the transposed plan (Q, P) maps that distribution back to
// the first one, so a fused forward -> diagonal -> inverse pass stores to the
// same addresses it loaded from and no extra reordering pass exists.
//
// Strided passes (x and y axes) give each CTA W contiguous columns of the
// pencil family, so every global access of a warp is a run of W contiguous
// elements (128 B for complex64 at W = 16). The contiguous pass (z axis)
// gives each CTA W whole rows.
#pragma once

#include "kernels.h"

namespace wfs {

// Two-stage transform. in: thread t < P1 holds x[t + P1*i] in a_in[Q1].
// out: thread t < Q1 holds X[t + Q1*k] in a_out[P1]. SIGN -1 forward, +1 inverse.
// sidx(k2, n1) is the shared-memory slot of A[n1][k2] for this thread's pencil.
template <int P1, int Q1, int SIGN, typename R, typename SI>
__device__ __forceinline__ void two_stage(Cx<R> (&a_in)[Q1], Cx<R> (&a_out)[P1], Cx<R>* sm,
                                          const Cx<R>* __restrict__ tw, int t, SI sidx) {
    if (t < P1) {
        dft<Q1, SIGN, R>(a_in);
#pragma unroll
        for (int k2 = 1; k2 < Q1; ++k2) {
            Cx<R> w = tw[t * k2];
            a_in[k2] = (SIGN < 0) ? cmul(a_in[k2], w) : cmulc(a_in[k2], w);
        }
#pragma unroll
        for (int k2 = 0; k2 < Q1; ++k2) sm[sidx(k2, t)] = a_in[k2];
    }
    __syncthreads();
    if (t < Q1) {
#pragma unroll
        for (int n1 = 0; n1 < P1; ++n1) a_out[n1] = sm[sidx(t, n1)];
        dft<P1, SIGN, R>(a_out);
    }
}

template <typename R>
__device__ __forceinline__ R simpson_w(int v, int b, int cnt) {
    int j = v - b;
    if (j < 0 || j >= cnt) return R(0);
    if (j == 0 || j == cnt - 1) return R(1);
    return (j & 1) ? R(4) : R(2);
}

// Block-wide sum of acc[0..nq) written to partials[blockIdx.x * nq + q].
// Warp sums use the working precision R (a 32-term tree); the sums of the warps
// and, later, of the blocks are FP64. FP64 work is a few adds per block.
template <int NQ, typename R>
__device__ __forceinline__ void block_reduce_store(R (&acc)[NQ], int nq, double* scratch, double* out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        R v = acc[q];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0 && q < nq) scratch[q * 32 + warp] = double(v);
    }
    __syncthreads();
    if (threadIdx.x < nq) {
        double s = 0.0;
        for (int w = 0; w < nwarp; ++w) s += scratch[threadIdx.x * 32 + w];
        out[(int64_t)blockIdx.x * nq + threadIdx.x] = s;
    }
}

// Observation sums. A thread sums the few elements of one (x, y) row it holds
// (RowAcc: Simpson z-weight * |psi|^2 per box, and the location moments in z),
// folds the row in with the row's x/y weights (obs_row_flush), and the block
// reduction adds threads in a 32-term tree; all of that is in the working
// precision. Only warp-to-block and block-to-grid sums are FP64, since GB300's
// FP64 rate is a small fraction of its FP32 rate.
template <typename R>
struct RowAcc {
    R box[kMaxBox];
    R s0, sz, szz;
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int b = 0; b < kMaxBox; ++b) box[b] = R(0);
        s0 = sz = szz = R(0);
    }
};

template <typename R>
__device__ __forceinline__ void obs_row_element(const ObsArgs& o, RowAcc<R>& ra, int z, Cx<R> v) {
    const R p = v.x * v.x + v.y * v.y;
#pragma unroll
    for (int b = 0; b < kMaxBox; ++b)
        if (b < o.nbox) ra.box[b] += simpson_w<R>(z, o.box[b].b[2], o.box[b].c[2]) * p;
    if (o.has_loc) {
        const R w = simpson_w<R>(z, o.loc.b[2], o.loc.c[2]) * p;
        const R rz = R(o.dx[2]) * R(z - o.n[2] / 2);
        ra.s0 += w;
        ra.sz += w * rz;
        ra.szz += w * rz * rz;
    }
}

template <typename R>
__device__ __forceinline__ void obs_row_flush(const ObsArgs& o, R (&acc)[kMaxBox + kLocQ], const RowAcc<R>& ra,
                                              const R (&wxy)[kMaxBox], R lxy, R rx, R ry) {
#pragma unroll
    for (int b = 0; b < kMaxBox; ++b)
        if (b < o.nbox) acc[b] += wxy[b] * ra.box[b];
    if (o.has_loc && lxy != R(0)) {
        const R ls0 = lxy * ra.s0;
        acc[kMaxBox + 0] += ls0;
        acc[kMaxBox + 1] += rx * ls0;
        acc[kMaxBox + 2] += ry * ls0;
        acc[kMaxBox + 3] += lxy * ra.sz;
        acc[kMaxBox + 4] += rx * rx * ls0;
        acc[kMaxBox + 5] += ry * ry * ls0;
        acc[kMaxBox + 6] += lxy * ra.szz;
    }
}

template <typename R>
__device__ __forceinline__ void obs_row_factors(const ObsArgs& o, int x, int y, R (&wxy)[kMaxBox], R& lxy,
                                                R& rx, R& ry) {
#pragma unroll
    for (int b = 0; b < kMaxBox; ++b) {
        wxy[b] = (b < o.nbox) ? simpson_w<R>(x, o.box[b].b[0], o.box[b].c[0]) *
                                    simpson_w<R>(y, o.box[b].b[1], o.box[b].c[1])
                              : R(0);
    }
    if (o.has_loc) {
        lxy = simpson_w<R>(x, o.loc.b[0], o.loc.c[0]) * simpson_w<R>(y, o.loc.b[1], o.loc.c[1]);
    } else {
        lxy = R(0);
    }
    rx = R(o.dx[0]) * R(x - o.n[0] / 2);
    ry = R(o.dx[1]) * R(y - o.n[1] / 2);
}

// Compacts the fixed accumulator layout to [nbox probs][loc sums] and stores per-CTA partials.
template <typename R>
__device__ __forceinline__ void obs_store(const ObsArgs& o, R (&acc)[kMaxBox + kLocQ], double* scratch) {
    R packed[kMaxBox + kLocQ];
#pragma unroll
    for (int q = 0; q < kMaxBox + kLocQ; ++q) packed[q] = R(0);
#pragma unroll
    for (int b = 0; b < kMaxBox; ++b)
        if (b < o.nbox) packed[b] = acc[b];
#pragma unroll
    for (int q = 0; q < kLocQ; ++q) {
        // place location sums right after the boxes
#pragma unroll
        for (int b = 0; b <= kMaxBox; ++b)
            if (b == o.nbox && o.has_loc) packed[b + q] = acc[kMaxBox + q];
    }
    block_reduce_store<kMaxBox + kLocQ>(packed, o.nq, scratch, o.partials);
}

// ---------------------------------------------------------------------------
// Strided pass (x or y axis)
// ---------------------------------------------------------------------------
template <typename R, int P, int Q, int W, int OP>
__global__ void __launch_bounds__(cmax(P, Q) * W, WFS_MINB_PASS) fft_strided_kernel(const PassArgs<R> a) {
    constexpr int L = P * Q;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cx<R>* sm = reinterpret_cast<Cx<R>*>(smem_raw);
    const int tid = threadIdx.x, c = tid % W, t = tid / W;
    const int tile = blockIdx.x % a.tiles;
    const int64_t outer = blockIdx.x / a.tiles;
    const int col = tile * W + c;
    const bool active = col < a.ncols;
    Cx<R>* base = a.data + outer * a.outer_stride + col;
    // 32-bit element offsets from one 64-bit base (the host guarantees L * row_stride < 2^31);
    // 64-bit per-row addresses kept live from load to store cost 32 registers
    const int rs = int(a.row_stride);

    Cx<R> a1[Q], a2[P];
    if (t < P) {
#pragma unroll
        for (int i = 0; i < Q; ++i) a1[i] = active ? base[(t + P * i) * rs] : mk<R>(R(0), R(0));
    }
    auto sidx_f = [&](int k2, int n1) { return (k2 * P + n1) * W + c; };
    auto sidx_i = [&](int k2, int n1) { return (k2 * Q + n1) * W + c; };

    if constexpr (OP == OP_PLAIN) {
        if (a.dir < 0) two_stage<P, Q, -1, R>(a1, a2, sm, a.tw, t, sidx_f);
        else two_stage<P, Q, +1, R>(a1, a2, sm, a.tw, t, sidx_f);
        if (active && t < Q) {
#pragma unroll
            for (int k = 0; k < P; ++k) base[(t + Q * k) * rs] = scale(a2[k], a.scale);
        }
    } else {  // OP_KIN: forward, diagonal kinetic factor, inverse
        two_stage<P, Q, -1, R>(a1, a2, sm, a.tw, t, sidx_f);
        if (t < Q) {
            Cx<R> cf = mk<R>(R(0), R(0));
            if (active) cf = scale(cmul(a.k_c1[col / a.c2n], a.k_c2[col % a.c2n]), a.scale);
#pragma unroll
            for (int k = 0; k < P; ++k) a2[k] = cmul(a2[k], cmul(a.k_row[t + Q * k], cf));
        }
        __syncthreads();
        two_stage<Q, P, +1, R>(a2, a1, sm, a.tw, t, sidx_i);
        if (active && t < P) {
#pragma unroll
            for (int i = 0; i < Q; ++i) base[(t + P * i) * rs] = a1[i];
        }
    }
}

// ---------------------------------------------------------------------------
// Contiguous pass (z axis)
// ---------------------------------------------------------------------------
template <typename R, int P, int Q, int W, int OP>
__global__ void __launch_bounds__(cmax(P, Q) * W, WFS_MINB_PASS) fft_contig_kernel(const PassArgs<R> a) {
    constexpr int L = P * Q, T = cmax(P, Q);
    constexpr int RS = cmax(Q * (P + 1), P * (Q + 1));
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cx<R>* sm = reinterpret_cast<Cx<R>*>(smem_raw);
    const int tid = threadIdx.x, t = tid % T, r = tid / T;
    const int64_t row = (int64_t)blockIdx.x * W + r;
    const bool active = row < a.nrows;
    Cx<R>* rp = a.data + row * L;

    Cx<R> a1[Q], a2[P];
    if (t < P) {
#pragma unroll
        for (int i = 0; i < Q; ++i) a1[i] = active ? rp[t + P * i] : mk<R>(R(0), R(0));
    }
    auto sidx_f = [&](int k2, int n1) { return r * RS + k2 * (P + 1) + n1; };
    auto sidx_i = [&](int k2, int n1) { return r * RS + k2 * (Q + 1) + n1; };

    if constexpr (OP == OP_PLAIN) {
        if (a.dir < 0) two_stage<P, Q, -1, R>(a1, a2, sm, a.tw, t, sidx_f);
        else two_stage<P, Q, +1, R>(a1, a2, sm, a.tw, t, sidx_f);
        if (active && t < Q) {
#pragma unroll
            for (int k = 0; k < P; ++k) rp[t + Q * k] = scale(a2[k], a.scale);
        }
    } else if constexpr (OP == OP_VPH) {  // inverse, potential phase, forward
        two_stage<P, Q, +1, R>(a1, a2, sm, a.tw, t, sidx_f);
        if (t < Q) {
            const Cx<R>* ep = a.ephase + row * L;
#pragma unroll
            for (int k = 0; k < P; ++k) {
                Cx<R> e = active ? ep[t + Q * k] : mk<R>(R(0), R(0));
                a2[k] = cmul(a2[k], scale(e, a.scale));
            }
        }
        __syncthreads();
        two_stage<Q, P, -1, R>(a2, a1, sm, a.tw, t, sidx_i);
        if (active && t < P) {
#pragma unroll
            for (int i = 0; i < Q; ++i) rp[t + P * i] = a1[i];
        }
    } else {  // OP_OBS: inverse transform in registers, observe, no store
        two_stage<P, Q, +1, R>(a1, a2, sm, a.tw, t, sidx_f);
        R acc[kMaxBox + kLocQ];
#pragma unroll
        for (int q = 0; q < kMaxBox + kLocQ; ++q) acc[q] = R(0);
        if (active && t < Q) {
            const ObsArgs& o = a.obs;
            const int x = int(row / o.n[1]), y = int(row % o.n[1]);
            R wxy[kMaxBox], lxy, rx, ry;
            obs_row_factors<R>(o, x, y, wxy, lxy, rx, ry);
            RowAcc<R> ra;
            ra.zero();
#pragma unroll
            for (int k = 0; k < P; ++k) obs_row_element<R>(o, ra, t + Q * k, scale(a2[k], a.scale));
            obs_row_flush<R>(o, acc, ra, wxy, lxy, rx, ry);
        }
        __syncthreads();
        obs_store(a.obs, acc, reinterpret_cast<double*>(smem_raw));
    }
}

// ---------------------------------------------------------------------------
// Host-side plan table and dispatch
// ---------------------------------------------------------------------------
template <int L>
struct PlanOf;
#define WFS_PLAN(L_, P_, Q_) template <> struct PlanOf<L_> { static constexpr int P = P_, Q = Q_; };
WFS_PLAN(2, 2, 1)
WFS_PLAN(3, 3, 1)
WFS_PLAN(4, 2, 2)
WFS_PLAN(6, 3, 2)
WFS_PLAN(8, 4, 2)
WFS_PLAN(12, 4, 3)
WFS_PLAN(16, 4, 4)
WFS_PLAN(24, 6, 4)
WFS_PLAN(32, 8, 4)
WFS_PLAN(48, 8, 6)
WFS_PLAN(64, 8, 8)
WFS_PLAN(96, 12, 8)
WFS_PLAN(128, 16, 8)
WFS_PLAN(192, 16, 12)
WFS_PLAN(256, 16, 16)
WFS_PLAN(384, 24, 16)
WFS_PLAN(512, 32, 16)
WFS_PLAN(768, 32, 24)
WFS_PLAN(1024, 32, 32)
#undef WFS_PLAN

template <typename R, int T>
struct StridedW {
    static constexpr int value = sizeof(R) == 4 ? (T <= 8 ? 32 : 16) : (T <= 8 ? 16 : 8);
};
template <typename R, int T>
struct ContigW {
    static constexpr int value = (256 / T) > 0 ? (256 / T) : 1;
};

template <typename R, int L, int OP>
cudaError_t run_strided(const PassArgs<R>& a0, int64_t outer_count, cudaStream_t s) {
    constexpr int P = PlanOf<L>::P, Q = PlanOf<L>::Q, T = cmax(P, Q);
    constexpr int W = StridedW<R, T>::value;
    PassArgs<R> a = a0;
    a.tiles = (a.ncols + W - 1) / W;
    const size_t smem = size_t(L) * W * sizeof(Cx<R>);
    auto kern = fft_strided_kernel<R, P, Q, W, OP>;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int64_t grid = outer_count * a.tiles;
    kern<<<dim3(unsigned(grid)), dim3(T * W), smem, s>>>(a);
    return cudaGetLastError();
}

template <typename R, int L, int OP>
cudaError_t run_contig(const PassArgs<R>& a, cudaStream_t s, int* grid_out) {
    constexpr int P = PlanOf<L>::P, Q = PlanOf<L>::Q, T = cmax(P, Q);
    constexpr int W = ContigW<R, T>::value;
    constexpr int RS = cmax(Q * (P + 1), P * (Q + 1));
    size_t smem = size_t(W) * RS * sizeof(Cx<R>);
    if (OP == OP_OBS) smem = smem > (kMaxBox + kLocQ) * 32 * sizeof(double) ? smem : (kMaxBox + kLocQ) * 32 * sizeof(double);
    auto kern = fft_contig_kernel<R, P, Q, W, OP>;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int64_t grid = (a.nrows + W - 1) / W;
    if (grid_out) *grid_out = int(grid);
    kern<<<dim3(unsigned(grid)), dim3(T * W), smem, s>>>(a);
    return cudaGetLastError();
}

#define WFS_FOR_EACH_L(M) M(2) M(3) M(4) M(6) M(8) M(12) M(16) M(24) M(32) M(48) M(64) M(96) M(128) M(192) M(256) M(384) M(512) M(768) M(1024)

template <typename R>
cudaError_t dispatch_strided(int L, int op, const PassArgs<R>& a, int64_t outer_count, cudaStream_t s) {
#define WFS_CASE(L_)                                                                   \
    case L_:                                                                           \
        return op == OP_KIN ? run_strided<R, L_, OP_KIN>(a, outer_count, s)            \
                            : run_strided<R, L_, OP_PLAIN>(a, outer_count, s);
    switch (L) {
        WFS_FOR_EACH_L(WFS_CASE)
        default:
            return cudaErrorInvalidValue;
    }
#undef WFS_CASE
}

template <typename R>
cudaError_t dispatch_contig(int L, int op, const PassArgs<R>& a, cudaStream_t s, int* grid_out) {
#define WFS_CASE(L_)                                                         \
    case L_:                                                                 \
        if (op == OP_VPH) return run_contig<R, L_, OP_VPH>(a, s, grid_out);  \
        if (op == OP_OBS) return run_contig<R, L_, OP_OBS>(a, s, grid_out);  \
        return run_contig<R, L_, OP_PLAIN>(a, s, grid_out);
    switch (L) {
        WFS_FOR_EACH_L(WFS_CASE)
        default:
            return cudaErrorInvalidValue;
    }
#undef WFS_CASE
}

}  // namespace wfs
