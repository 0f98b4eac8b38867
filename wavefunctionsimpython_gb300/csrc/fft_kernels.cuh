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

#include "per_device.h"

#include <cmath>
#include <cstdlib>

#include "bulk_copy.cuh"
#include "kernels.h"

namespace wfs {

// Two-stage transform. in: thread t < P1 holds x[t + P1*i] in a_in[Q1].
// out: thread t < Q1 holds X[t + Q1*k] in a_out[P1]. SIGN -1 forward, +1 inverse.
// sidx(k2, n1) is the shared-memory slot of A[n1][k2] for this thread's pencil.
// Twiddles w = exp(-2 pi i t k2 / L) come from the axis table (two_stage_roots) in one
// of two orders, whichever suits how the kernel maps pencils onto a warp:
//   TW_ANGLE: tw[t*k2] (tw = the table itself); a warp that spans many t (rows of
//             a contiguous axis) finds the small angles of each k2 in a few lines;
//   TW_ROW:   tw[t*Q1 + k2] (tw = the plan's row block); a warp that spans one or
//             two t (strided axes) reads its contiguous row, two twiddles per 16 bytes.
//   TW_ROW_SMEM: TW_ROW with the rows in shared memory (plain loads instead of __ldg).
constexpr int TW_ANGLE = 0, TW_ROW = 1, TW_ROW_SMEM = 2;
// Row block of the plan (P1, Q1) in an axis table whose own plan is (P, Q).
template <int P1, int Q1, int P, int Q, typename R>
__device__ __forceinline__ const Cx<R>* tw_rows(const Cx<R>* tw) {
    return tw + (P1 == P ? 1 : 2) * (P * Q);
}
template <int P1, int Q1, int SIGN, int TWL, typename R, typename SI>
__device__ __forceinline__ void two_stage(Cx<R> (&a_in)[Q1], Cx<R> (&a_out)[P1], Cx<R>* sm,
                                          const Cx<R>* __restrict__ tw, int t, SI sidx) {
    if (t < P1) {
        dft<Q1, SIGN, R>(a_in);
        auto apply = [&](int k2, Cx<R> w) { a_in[k2] = (SIGN < 0) ? cmul(a_in[k2], w) : cmulc(a_in[k2], w); };
        if constexpr ((TWL == TW_ROW || TWL == TW_ROW_SMEM) && sizeof(Cx<R>) == 8 && Q1 % 2 == 0) {
            const Cx<R>* row = tw + t * Q1;
#pragma unroll
            for (int j = 0; j < Q1 / 2; ++j) {
                const float4 w2 = (TWL == TW_ROW) ? __ldg(reinterpret_cast<const float4*>(row) + j)
                                                  : reinterpret_cast<const float4*>(row)[j];
                if (j > 0) apply(2 * j, mk<R>(w2.x, w2.y));
                apply(2 * j + 1, mk<R>(w2.z, w2.w));
            }
        } else if constexpr (TWL == TW_ROW || TWL == TW_ROW_SMEM) {
            const Cx<R>* row = tw + t * Q1;
#pragma unroll
            for (int k2 = 1; k2 < Q1; ++k2) apply(k2, row[k2]);
        } else {
#pragma unroll
            for (int k2 = 1; k2 < Q1; ++k2) apply(k2, tw[t * k2]);
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

// Observation sums (volume probabilities with Simpson weights, location moments).
// Complex128 sums run in FP64 throughout. Complex64 sums are accumulated by each
// thread and across the warp as compensated float-float pairs (hi, lo): every add is an
// error-free transformation (TwoSum) whose rounding error is carried in lo, so the pair
// holds the sum to about 2^-46 relative, as accurate as an FP64 accumulation of the
// float32 terms, at FP32 instruction rates (GB300's FP64 rate is about 1/60 of its FP32
// rate; FP64 adds per element would cost the observation pass more than its HBM
// traffic). Each warp's pair is converted to FP64 once; CTA and grid sums are FP64 in
// a fixed order. Partials are laid out [CTA][nbox box probabilities, then the 7
// location sums]. Location sums carry exact integer offsets from the grid centre
// (v - N/2); the host multiplies by the spacing in FP64.
template <typename R>
struct CSum;
template <>
struct CSum<double> {
    double hi = 0.0;
    __device__ __forceinline__ void add(double v) { hi += v; }
    __device__ __forceinline__ void merge(const CSum& o) { hi += o.hi; }
    __device__ __forceinline__ CSum scaled(double k) const { CSum r; r.hi = hi * k; return r; }
    __device__ __forceinline__ CSum shfl_xor(int m) const {
        CSum r;
        r.hi = __shfl_xor_sync(0xffffffffu, hi, m);
        return r;
    }
    __device__ __forceinline__ double value() const { return hi; }
};
template <>
struct CSum<float> {
    float hi = 0.0f, lo = 0.0f;
    // TwoSum (Knuth): s + e equals hi + v exactly
    __device__ __forceinline__ void add(float v) {
        const float s = __fadd_rn(hi, v);
        const float vv = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, vv)), __fsub_rn(v, vv));
        hi = s;
        lo = __fadd_rn(lo, e);
    }
    __device__ __forceinline__ void merge(const CSum& o) {
        add(o.hi);
        lo = __fadd_rn(lo, o.lo);
    }
    // times k, the product of hi kept exact by its FMA residual (TwoProd)
    __device__ __forceinline__ CSum scaled(float k) const {
        CSum r;
        r.hi = __fmul_rn(hi, k);
        r.lo = __fmaf_rn(lo, k, __fmaf_rn(hi, k, -r.hi));
        return r;
    }
    __device__ __forceinline__ CSum shfl_xor(int m) const {
        CSum r;
        r.hi = __shfl_xor_sync(0xffffffffu, hi, m);
        r.lo = __shfl_xor_sync(0xffffffffu, lo, m);
        return r;
    }
    __device__ __forceinline__ double value() const { return double(hi) + double(lo); }
};

// |v|^2 with one rounding fewer than x*x + y*y
__device__ __forceinline__ float abs2(Cx<float> v) { return __fmaf_rn(v.x, v.x, __fmul_rn(v.y, v.y)); }
__device__ __forceinline__ double abs2(Cx<double> v) { return v.x * v.x + v.y * v.y; }

// Sums v over the warp and stores the sum, as FP64, at scratch[q * 32 + warp]; every
// lane of the warp must call it.
template <typename R>
__device__ __forceinline__ void warp_sum_to(CSum<R> v, double* scratch, int q) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v.merge(v.shfl_xor(m));
    if ((threadIdx.x & 31) == 0) scratch[q * 32 + (threadIdx.x >> 5)] = v.value();
}

// A thread's share of the location sums of one (x, y) row from its sums over z of
// w = Simpson weight * |psi|^2: s0 = sum w, s1 = sum w kz, s2 = sum w kz^2, with
// kz = z - nz/2; lxy is the row's Simpson weight (a power of two), kx, ky its offsets.
// Warp-sums S, S kx, S ky, s1 lxy, S kx^2, S ky^2, s2 lxy into slots q0 .. q0 + 6.
template <typename R>
__device__ __forceinline__ void loc_sums_to(const CSum<R>& s0, const CSum<R>& s1, const CSum<R>& s2, R lxy, R kx,
                                            R ky, double* scratch, int q0) {
    const CSum<R> S = s0.scaled(lxy);
    warp_sum_to<R>(S, scratch, q0);
    warp_sum_to<R>(S.scaled(kx), scratch, q0 + 1);
    warp_sum_to<R>(S.scaled(ky), scratch, q0 + 2);
    warp_sum_to<R>(s1.scaled(lxy), scratch, q0 + 3);
    warp_sum_to<R>(S.scaled(kx * kx), scratch, q0 + 4);
    warp_sum_to<R>(S.scaled(ky * ky), scratch, q0 + 5);
    warp_sum_to<R>(s2.scaled(lxy), scratch, q0 + 6);
}
// FP64 sums over the warps of quantities [0, nq) into out[blockIdx.x * nq + q]
// (after a block barrier that follows the warp_sum_to calls).
__device__ __forceinline__ void block_partials(const double* scratch, int nq, double* out) {
    const int nwarp = (blockDim.x + 31) >> 5;
    if (int(threadIdx.x) < nq) {
        double s = 0.0;
        for (int w = 0; w < nwarp; ++w) s += scratch[threadIdx.x * 32 + w];
        out[(int64_t)blockIdx.x * nq + threadIdx.x] = s;
    }
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
        if (a.dir < 0) two_stage<P, Q, -1, TW_ROW>(a1, a2, sm, tw_rows<P, Q, P, Q>(a.tw), t, sidx_f);
        else two_stage<P, Q, +1, TW_ROW>(a1, a2, sm, tw_rows<P, Q, P, Q>(a.tw), t, sidx_f);
        if (active && t < Q) {
#pragma unroll
            for (int k = 0; k < P; ++k) base[(t + Q * k) * rs] = scale(a2[k], a.scale);
        }
    } else {  // OP_KIN: forward, diagonal kinetic factor, inverse
        two_stage<P, Q, -1, TW_ROW>(a1, a2, sm, tw_rows<P, Q, P, Q>(a.tw), t, sidx_f);
        if (t < Q) {
            Cx<R> cf = mk<R>(R(0), R(0));
            if (active) cf = scale(cmul(a.k_c1[col / a.c2n], a.k_c2[col % a.c2n]), a.scale);
#pragma unroll
            for (int k = 0; k < P; ++k) a2[k] = cmul(a2[k], cmul(a.k_row[t + Q * k], cf));
        }
        __syncthreads();
        two_stage<Q, P, +1, TW_ROW>(a2, a1, sm, tw_rows<Q, P, P, Q>(a.tw), t, sidx_i);
        if (active && t < P) {
#pragma unroll
            for (int i = 0; i < Q; ++i) base[(t + P * i) * rs] = a1[i];
        }
    }
}

// ---------------------------------------------------------------------------
// Pipelined strided pass: persistent CTAs walk the (outer, tile) items with a
// stride of gridDim.x; while a CTA transforms item k from shared memory, the
// cp.async copies of item k + gridDim.x are in flight, so HBM reads overlap the
// register FFTs instead of alternating with them. Each thread stages exactly
// the elements it later reads (rows t + P*i of its column), so the staging
// buffers need no block barrier: cp.async.wait_group orders a thread's own
// copies before its reads.
// Shared memory: two staging tiles (2 L W elements). A tile, once loaded into
// registers, is the transpose buffer of its own item: in the first transpose
// thread t writes rows k2*P + t, which are rows it staged itself (rows = t mod P),
// and the inverse transpose follows a block barrier.
// ---------------------------------------------------------------------------
template <int BYTES>
__device__ __forceinline__ void cp_async_elem(void* smem, const void* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    if constexpr (BYTES == 16) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
    } else {
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(BYTES) : "memory");
    }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <typename R, int P, int Q, int W, int OP>
__global__ void __launch_bounds__(cmax(P, Q) * W, WFS_MINB_PIPE)
    fft_strided_pipe_kernel(const PassArgs<R> a, int64_t nitems) {
    constexpr int L = P * Q;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cx<R>* stage = reinterpret_cast<Cx<R>*>(smem_raw);  // [2][L][W]
    const int tid = threadIdx.x, c = tid % W, t = tid / W;
    const int rs = int(a.row_stride);
    auto issue = [&](int64_t item, int slot) {
        const int tile = int(item % a.tiles);
        const int64_t outer = item / a.tiles;
        const int col = tile * W + c;
        if (t < P && col < a.ncols) {
            const Cx<R>* src = a.data + outer * a.outer_stride + col;
            Cx<R>* dst = stage + slot * (L * W) + c;
#pragma unroll
            for (int i = 0; i < Q; ++i) cp_async_elem<sizeof(Cx<R>)>(dst + (t + P * i) * W, src + (t + P * i) * rs);
        }
        cp_async_commit();
    };
    auto sidx_f = [&](int k2, int n1) { return (k2 * P + n1) * W + c; };
    auto sidx_i = [&](int k2, int n1) { return (k2 * Q + n1) * W + c; };
    int64_t item = blockIdx.x;
    if (item < nitems) issue(item, 0);
    int slot = 0;
    for (; item < nitems; item += gridDim.x) {
        const int64_t next = item + gridDim.x;
        if (next < nitems) issue(next, slot ^ 1);
        else cp_async_commit();
        cp_async_wait<1>();
        const int tile = int(item % a.tiles);
        const int64_t outer = item / a.tiles;
        const int col = tile * W + c;
        const bool active = col < a.ncols;
        Cx<R>* base = a.data + outer * a.outer_stride + col;
        Cx<R>* sm = stage + slot * (L * W);  // this item's staging tile, reused as its transpose buffer
        const Cx<R>* src = sm + c;
        Cx<R> a1[Q], a2[P];
        if (t < P) {
#pragma unroll
            for (int i = 0; i < Q; ++i) a1[i] = active ? src[(t + P * i) * W] : mk<R>(R(0), R(0));
        }
        if constexpr (OP == OP_PLAIN) {
            if (a.dir < 0) two_stage<P, Q, -1, TW_ROW>(a1, a2, sm, tw_rows<P, Q, P, Q>(a.tw), t, sidx_f);
            else two_stage<P, Q, +1, TW_ROW>(a1, a2, sm, tw_rows<P, Q, P, Q>(a.tw), t, sidx_f);
            if (active && t < Q) {
#pragma unroll
                for (int k = 0; k < P; ++k) base[(t + Q * k) * rs] = scale(a2[k], a.scale);
            }
        } else {  // OP_KIN
            two_stage<P, Q, -1, TW_ROW>(a1, a2, sm, tw_rows<P, Q, P, Q>(a.tw), t, sidx_f);
            if (t < Q) {
                Cx<R> cf = mk<R>(R(0), R(0));
                if (active) cf = scale(cmul(a.k_c1[col / a.c2n], a.k_c2[col % a.c2n]), a.scale);
#pragma unroll
                for (int k = 0; k < P; ++k) a2[k] = cmul(a2[k], cmul(a.k_row[t + Q * k], cf));
            }
            __syncthreads();
            two_stage<Q, P, +1, TW_ROW>(a2, a1, sm, tw_rows<Q, P, P, Q>(a.tw), t, sidx_i);
            if (active && t < P) {
#pragma unroll
                for (int i = 0; i < Q; ++i) base[(t + P * i) * rs] = a1[i];
            }
        }
        __syncthreads();  // this tile is restaged for the item after next
        slot ^= 1;
    }
    cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// Copy-engine staged strided pass (complex64): the pipelined pass with each
// item's L x W tile brought into shared memory by one 3D tensor copy (x = column,
// y = pencil row, z = outer slab) instead of Q cp.async copies per thread. Thread
// 0 arms the slot's mbarrier and issues the copy of item k + gridDim.x while the
// block transforms item k; the other threads issue no copies and compute no
// addresses for them. Columns past ncols arrive zero-filled and are not stored.
// Item k of a CTA lives in slot k & 1 and completes phase (k >> 1) & 1 of that
// slot's barrier. A wait that gives up sets bit 0 of *status; thread 0 then
// issues no further copies and, before the CTA exits, waits (bounded) for any
// copy still in flight.
// ---------------------------------------------------------------------------
struct StridedStagedArgs {
    PassArgs<float> p;
    TensorMapImage map;  // psi as (ncols, L, outer) complex64 elements, box (W, L, 1)
};

template <int P, int Q, int W, int OP>
__global__ void __launch_bounds__(cmax(P, Q) * W, WFS_MINB_STAGED)
    fft_strided_staged_kernel(const __grid_constant__ StridedStagedArgs sa, int64_t nitems) {
    using R = float;
    constexpr int L = P * Q;
    const PassArgs<R>& a = sa.p;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Cx<R>* stage = reinterpret_cast<Cx<R>*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));  // [2][L][W]
    uint64_t* bars = reinterpret_cast<uint64_t*>(stage + 2 * L * W);
    // the two plans' twiddle rows and the kinetic x factors, copied once per CTA: every thread
    // keeps its row t for all items, and shared-memory reads beat L1 for them (x pass at 256^3:
    // 59.5 us against 60.5 us through L1)
    Cx<R>* tsm = reinterpret_cast<Cx<R>*>(bars + 2);  // [P*Q forward rows][Q*P inverse rows][L x factors]
    const int tid = threadIdx.x, c = tid % W, t = tid / W;
    const int rs = int(a.row_stride);
    if (tid == 0) {
        mbar_init(smem_addr(&bars[0]), 1);
        mbar_init(smem_addr(&bars[1]), 1);
        mbar_init_fence();
    }
    {
        const Cx<R>* twf = tw_rows<P, Q, P, Q>(a.tw);
        const Cx<R>* twi = tw_rows<Q, P, P, Q>(a.tw);
        for (int i = tid; i < L; i += blockDim.x) {
            tsm[i] = twf[i];
            tsm[L + i] = twi[i];
            if constexpr (OP == OP_KIN) tsm[2 * L + i] = a.k_row[i];
        }
    }
    __syncthreads();
    constexpr int TWM = TW_ROW_SMEM;
    const Cx<R>* tw_f = tsm;
    const Cx<R>* tw_i = tsm + L;
    const Cx<R>* k_row = tsm + 2 * L;
    auto issue = [&](int64_t item, int slot) {  // thread 0 only
        const uint32_t bar = smem_addr(&bars[slot]);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar, uint32_t(L * W * sizeof(Cx<R>)));
        tensor_load_3d(smem_addr(stage + slot * (L * W)), &sa.map, int(item % a.tiles) * W, 0, int(item / a.tiles), bar);
    };
    auto sidx_f = [&](int k2, int n1) { return (k2 * P + n1) * W + c; };
    auto sidx_i = [&](int k2, int n1) { return (k2 * Q + n1) * W + c; };
    int64_t item = blockIdx.x;
    if (tid == 0 && item < nitems) issue(item, 0);
    int k = 0;
    for (; item < nitems; item += gridDim.x, ++k) {
        const int slot = k & 1;
        const int64_t next = item + gridDim.x;
        if (tid == 0 && next < nitems) issue(next, slot ^ 1);
        const bool waited =
            mbar_wait_bounded(smem_addr(&bars[slot]), uint32_t((k >> 1) & 1), a.wait_ns ? a.wait_ns : kWaitLimitNs);
        const int tile = int(item % a.tiles);
        const int64_t outer = item / a.tiles;
        const int col = tile * W + c;
        const bool active = col < a.ncols;
        Cx<R>* base = a.data + outer * a.outer_stride + col;
        Cx<R>* sm = stage + slot * (L * W);  // this item's staging tile, reused as its transpose buffer
        const Cx<R>* src = sm + c;
        Cx<R> a1[Q], a2[P];
        if (t < P) {
#pragma unroll
            for (int i = 0; i < Q; ++i) a1[i] = src[(t + P * i) * W];
        }
        if constexpr (OP == OP_PLAIN) {
            if (a.dir < 0) two_stage<P, Q, -1, TWM>(a1, a2, sm, tw_f, t, sidx_f);
            else two_stage<P, Q, +1, TWM>(a1, a2, sm, tw_f, t, sidx_f);
            if (waited && active && t < Q) {
#pragma unroll
                for (int kk = 0; kk < P; ++kk) base[(t + Q * kk) * rs] = scale(a2[kk], a.scale);
            }
        } else {  // OP_KIN
            two_stage<P, Q, -1, TWM>(a1, a2, sm, tw_f, t, sidx_f);
            if (t < Q) {
                Cx<R> cf = mk<R>(R(0), R(0));
                if (active) cf = scale(cmul(a.k_c1[col / a.c2n], a.k_c2[col % a.c2n]), a.scale);
#pragma unroll
                for (int kk = 0; kk < P; ++kk) a2[kk] = cmul(a2[kk], cmul(k_row[t + Q * kk], cf));
            }
            __syncthreads();
            two_stage<Q, P, +1, TWM>(a2, a1, sm, tw_i, t, sidx_i);
            if (waited && active && t < P) {
#pragma unroll
                for (int i = 0; i < Q; ++i) base[(t + P * i) * rs] = a1[i];
            }
        }
        // The barrier that lets this slot be refilled with the item after next also tells
        // every thread whether any thread's wait for this tile ran out. If one did, the CTA
        // reports it (the host reads the status word at its next synchronisation) and
        // stops: the tiles it has not stored are left as they were, no further copies are
        // issued, and thread 0 first waits, with the default bound, for the two copies that
        // may still be landing in this CTA's shared memory (this tile's and the next one's).
        if (__syncthreads_or(!waited)) {
            if (tid == 0) {
                if (a.status) atomicOr(a.status, 1);
                mbar_wait_bounded(smem_addr(&bars[slot]), uint32_t((k >> 1) & 1));
                if (next < nitems) mbar_wait_bounded(smem_addr(&bars[slot ^ 1]), uint32_t(((k + 1) >> 1) & 1));
            }
            return;
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
        if (a.dir < 0) two_stage<P, Q, -1, TW_ANGLE>(a1, a2, sm, a.tw, t, sidx_f);
        else two_stage<P, Q, +1, TW_ANGLE>(a1, a2, sm, a.tw, t, sidx_f);
        if (active && t < Q) {
#pragma unroll
            for (int k = 0; k < P; ++k) rp[t + Q * k] = scale(a2[k], a.scale);
        }
    } else if constexpr (OP == OP_VPH) {  // inverse, potential phase, forward
        two_stage<P, Q, +1, TW_ANGLE>(a1, a2, sm, a.tw, t, sidx_f);
        if (t < Q) {
            const Cx<R>* ep = a.ephase + row * L;
#pragma unroll
            for (int k = 0; k < P; ++k) {
                Cx<R> e = active ? ep[t + Q * k] : mk<R>(R(0), R(0));
                a2[k] = cmul(a2[k], scale(e, a.scale));
            }
        }
        __syncthreads();
        two_stage<Q, P, -1, TW_ANGLE>(a2, a1, sm, a.tw, t, sidx_i);
        if (active && t < P) {
#pragma unroll
            for (int i = 0; i < Q; ++i) rp[t + P * i] = a1[i];
        }
    } else {  // OP_OBS: inverse transform in registers, observe, no store
        two_stage<P, Q, +1, TW_ANGLE>(a1, a2, sm, a.tw, t, sidx_f);
        // |psi|^2 of this thread's elements (z = t + Q*k), then one pass per requested
        // box over those 16 values: a runtime loop over the boxes keeps the code small
        // (the fully unrolled form over all kMaxBox boxes missed the instruction cache)
        const ObsArgs& o = a.obs;
        const bool own = active && t < Q;
        const int x = int(row / o.n[1]), y = int(row % o.n[1]);
        R pk[P];
#pragma unroll
        for (int k = 0; k < P; ++k) pk[k] = own ? abs2(scale(a2[k], a.scale)) : R(0);
        __syncthreads();  // the transpose scratch is reused for the block sums
        double* scratch = reinterpret_cast<double*>(smem_raw);
#pragma unroll 1
        for (int b = 0; b < o.nbox; ++b) {
            const ObsBox bx = o.box[b];
            const R wxy = simpson_w<R>(x, bx.b[0], bx.c[0]) * simpson_w<R>(y, bx.b[1], bx.c[1]);
            CSum<R> sz;
            if (wxy != R(0)) {
#pragma unroll
                for (int k = 0; k < P; ++k) sz.add(simpson_w<R>(t + Q * k, bx.b[2], bx.c[2]) * pk[k]);
            }
            warp_sum_to<R>(sz.scaled(wxy), scratch, b);
        }
        if (o.has_loc) {
            CSum<R> s0, s1, s2;
            const R lxy = simpson_w<R>(x, o.loc.b[0], o.loc.c[0]) * simpson_w<R>(y, o.loc.b[1], o.loc.c[1]);
            if (lxy != R(0)) {
#pragma unroll
                for (int k = 0; k < P; ++k) {
                    const int z = t + Q * k;
                    const R w = simpson_w<R>(z, o.loc.b[2], o.loc.c[2]) * pk[k];
                    const R kz = R(z - o.n[2] / 2);
                    s0.add(w);
                    s1.add(w * kz);
                    s2.add(w * (kz * kz));
                }
            }
            loc_sums_to<R>(s0, s1, s2, lxy, R(x - o.n[0] / 2), R(y - o.n[1] / 2), scratch, o.nbox);
        }
        __syncthreads();
        block_partials(scratch, o.nq, o.partials);
    }
}

// ---------------------------------------------------------------------------
// Host-side plan table and dispatch
// ---------------------------------------------------------------------------
template <int L>
struct PlanOf;
#define WFS_PLAN(L_, P_, Q_) template <> struct PlanOf<L_> { static constexpr int P = P_, Q = Q_; };
WFS_PLAN_LIST(WFS_PLAN)
#undef WFS_PLAN


template <typename R, int T>
struct StridedW {
    static constexpr int value = sizeof(R) == 4 ? (T <= 8 ? 32 : 16) : (T <= 8 ? 16 : 8);
};
template <typename R, int T>
struct ContigW {
    static constexpr int value = (256 / T) > 0 ? (256 / T) : 1;
};

// The pipelined strided pass is used where its two L x W tiles leave room for two
// CTAs per SM; WFS_STRIDED_PIPELINE=0 in the environment selects the plain kernel
// (for A/B timing).
inline bool strided_pipeline_enabled() {
    static const int on = [] {
        const char* e = getenv("WFS_STRIDED_PIPELINE");
        return (e && e[0] == '0') ? 0 : 1;
    }();
    return on != 0;
}
inline int device_sm_count() {
    static PerDevice sms;
    const int dev = current_device();
    int n = sms.get(dev);
    if (n == 0) {
        int v = 0;
        if (dev >= 0 && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0) {
            n = v;
            sms.put(dev, n);
        }
    }
    return n > 0 ? n : 1;
}

template <typename R, int L, int OP>
cudaError_t run_strided_pipe(const PassArgs<R>& a, int64_t outer_count, cudaStream_t s) {
    constexpr int P = PlanOf<L>::P, Q = PlanOf<L>::Q, T = cmax(P, Q);
    constexpr int W = StridedW<R, T>::value;
    const size_t smem = 2 * size_t(L) * W * sizeof(Cx<R>);
    auto kern = fft_strided_pipe_kernel<R, P, Q, W, OP>;
    static PerDevice occupancy;
    const int dev = current_device();
    int blocks_per_sm = occupancy.get(dev);
    if (blocks_per_sm == 0) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        int nb = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, T * W, smem);
        if (e != cudaSuccess) return e;
        blocks_per_sm = nb > 0 ? nb : 1;
        occupancy.put(dev, blocks_per_sm);
    }
    const int64_t nitems = outer_count * a.tiles;
    const int64_t cap = int64_t(blocks_per_sm) * device_sm_count();
    const int64_t grid = nitems < cap ? nitems : cap;
    kern<<<dim3(unsigned(grid)), dim3(T * W), smem, s>>>(a, nitems);
    return cudaGetLastError();
}

template <typename R, int L, int OP>
cudaError_t run_strided(const PassArgs<R>& a0, int64_t outer_count, cudaStream_t s) {
    constexpr int P = PlanOf<L>::P, Q = PlanOf<L>::Q, T = cmax(P, Q);
    constexpr int W = StridedW<R, T>::value;
    PassArgs<R> a = a0;
    a.tiles = (a.ncols + W - 1) / W;
    if constexpr (2 * size_t(L) * W * sizeof(Cx<R>) <= 112 * 1024) {
        if (strided_pipeline_enabled() && outer_count * a.tiles > int64_t(2) * device_sm_count())
            return run_strided_pipe<R, L, OP>(a, outer_count, s);
    }
    const size_t smem = size_t(L) * W * sizeof(Cx<R>);
    auto kern = fft_strided_kernel<R, P, Q, W, OP>;
    static PerDevice attr_set;
    const int dev = current_device();
    if (!attr_set.get(dev)) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        attr_set.put(dev, 1);
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
    static PerDevice attr_set;
    const int dev = current_device();
    if (!attr_set.get(dev)) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        attr_set.put(dev, 1);
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
