// taylor.cu — one term of the power-series propagator
// (sources/sim_state.py:721-752, sources/cuda_kernels/power_series_operator.cu:3-65):
//   s_n = i (dt/n) ( lap(s_{n-1}) / (2m) - V s_{n-1} ),   acc += s_n.
//
// Term 1 reads psi as s_0 and writes acc = psi + s_1 into a separate buffer,
// which removes the reference's per-step copy of psi (sim_state.py:730).
// Later terms update acc in place. Out-of-range stencil neighbours are replaced
// by the centre value (power_series_operator.cu:23-46).
//
// Tiling: each CTA covers a TZ x TY tile of one x-plane and marches along x
// through a chunk of XC planes (short chunks keep many CTAs in flight, which
// hides latency better than long persistent ranges do). The tile (plus a halo of H = stencil_order/2 cells in y and
// z) of each plane is staged in shared memory with cp.async into one of two
// buffers, so the next plane's copy is in flight while the current plane is
// computed; V, the accumulator and the next x-neighbour are loaded one plane
// ahead into registers. The x-neighbours are held in a register queue, so
// s_{n-1} is read from memory about once per site. Each thread's staging copies
// (16-byte pairs when the rows allow it) are addressed once per CTA, and sites
// whose whole stencil lies inside the grid skip the boundary selects.
#include <cstdint>
#include <cstdlib>
#include <type_traits>

#include "fft_kernels.cuh"
#include "kernels.h"

namespace wfs {

#ifndef WFS_MINB_TAYLOR
#define WFS_MINB_TAYLOR 5
#endif

constexpr int kTZ = 32;
constexpr int kTY = 8;
constexpr int kHZ = 2;  // z halo staged on each side: >= H and even, so staged pairs stay 16-byte aligned

// VEC: every staged copy moves a pair of complex64 values (16 bytes); the host
// picks it when nz is even and s_prev is 16-byte aligned, else single elements.
template <typename R, int H, bool VEC>
struct TaylorTile {
    static constexpr int NT = kTZ * kTY;
    static constexpr int SZ = kTZ + 2 * kHZ, SY = kTY + 2 * H;
    static constexpr int E = (VEC && sizeof(Cx<R>) == 8) ? 2 : 1;  // elements per staged copy
    static constexpr int CPR = SZ / E;                              // copies per staged row
    static constexpr int NCH = (SY * CPR + NT - 1) / NT;            // copies per thread and plane
};

// Planes [x0, x1) of the tile (bx, by): the tile of each plane plus its y/z halo
// is staged in tile[buf] one plane ahead; x-neighbours come from a register queue.
template <typename R, int H, bool VEC, int U>
__device__ __forceinline__ void taylor_segment(const TaylorArgs<R>& t, Cx<R> (&tile)[2][kTY + 2 * H][kTZ + 2 * kHZ],
                                               int bx, int by, int x0, int x1) {
    using TT = TaylorTile<R, H, VEC>;
    constexpr int NT = TT::NT, SZ = TT::SZ, SY = TT::SY, E = TT::E, CPR = TT::CPR, NCH = TT::NCH;
    static_assert(U == 2 || U == 4, "planes per unrolled group must be even");
    const int nx = t.n[0], ny = t.n[1], nz = t.n[2];
    const int tz = threadIdx.x % kTZ, ty = threadIdx.x / kTZ;
    const int z = bx * kTZ + tz;
    const int y = by * kTY + ty;
    const bool in = (z < nz) && (y < ny);
    // all stencil neighbours of every column of this warp lie inside the grid in y and
    // z: the warp takes the unchecked path (decided per warp, so no warp runs both)
    const bool inner_yz = __all_sync(0xffffffffu, in && y >= H && y + H < ny && z >= H && z + H < nz);
    const int64_t plane = int64_t(ny) * nz;
    const int zc = z < nz ? z : nz - 1, yc = y < ny ? y : ny - 1;
    const int64_t col = int64_t(yc) * nz + zc;
    const bool term1 = t.acc_in == t.s_prev;  // the accumulator starts from psi = s_0

    // this thread's staging copies: shared-memory slot, offset inside the global plane,
    // and whether the source lies inside the grid (halo cells outside it are not
    // staged; the centre-replacement rule below never reads them)
    int soff[NCH], goff[NCH];
    bool sval[NCH];
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
        const int ch = int(threadIdx.x) + c * NT;
        const int ly = ch / CPR, lz = (ch % CPR) * E;
        const int gy = by * kTY + ly - H;
        const int gz = bx * kTZ + lz - kHZ;
        sval[c] = ch < SY * CPR && gy >= 0 && gy < ny && gz >= 0 && gz < nz;
        soff[c] = ly * SZ + lz;
        goff[c] = gy * nz + gz;
    }
    auto stage = [&](int x, int buf) {
        const Cx<R>* sp = t.s_prev + int64_t(x) * plane;
        Cx<R>* dst = &tile[buf][0][0];
#pragma unroll
        for (int c = 0; c < NCH; ++c)
            if (sval[c]) cp_async_elem<E * sizeof(Cx<R>)>(dst + soff[c], sp + goff[c]);
        cp_async_commit();
    };

    stage(x0, 0);
    // register queue along x: q[H + k] = s at x + k, k in [-H, H]
    // (entries outside the grid are never used: nb_x returns the centre there)
    Cx<R> q[2 * H + 1];
#pragma unroll
    for (int k = -H; k <= H; ++k) {
        int xx = x0 + k;
        if (xx < 0 || xx >= nx) xx = x0;
        q[H + k] = t.s_prev[int64_t(xx) * plane + col];
    }
    float2 vcur = make_float2(0.f, 0.f);
    Cx<R> acur = mk<R>(R(0), R(0));
    if (in) {
        vcur = t.V[int64_t(x0) * plane + col];
        if (!term1) acur = t.acc_in[int64_t(x0) * plane + col];
    }
#pragma unroll 1
    for (int xg = x0; xg < x1; xg += U) {
        // unrolled by U: buffer indices are constants and the register queue is
        // renamed inside the group; x1 is the same for the whole CTA
#pragma unroll
        for (int i = 0; i < U; ++i) {
            const int x = xg + i, buf = i & 1;
            if (x < x1) {
                if (x + 1 < x1) stage(x + 1, buf ^ 1);
                else cp_async_commit();
                // one plane ahead: V, the accumulator and the next x-neighbour
                float2 vnext = vcur;
                Cx<R> anext = acur, qnext = q[2 * H];
                const int xn = x + H + 1;
                if (xn < nx) qnext = t.s_prev[int64_t(xn) * plane + col];
                if (in && x + 1 < x1) {
                    vnext = t.V[int64_t(x + 1) * plane + col];
                    if (!term1) anext = t.acc_in[int64_t(x + 1) * plane + col];
                }
                cp_async_wait<1>();
                __syncthreads();
                auto term = [&](auto fast_c) {
                    constexpr bool FAST = decltype(fast_c)::value;
                    const Cx<R> c = q[H];
                    auto nb_y = [&](int k) -> Cx<R> {
                        if constexpr (FAST) return tile[buf][ty + H + k][tz + kHZ];
                        const int yy = y + k;
                        return (yy < 0 || yy >= ny) ? c : tile[buf][ty + H + k][tz + kHZ];
                    };
                    auto nb_z = [&](int k) -> Cx<R> {
                        if constexpr (FAST) return tile[buf][ty + H][tz + kHZ + k];
                        const int zz = z + k;
                        return (zz < 0 || zz >= nz) ? c : tile[buf][ty + H][tz + kHZ + k];
                    };
                    auto nb_x = [&](int k) -> Cx<R> {
                        if constexpr (FAST) return q[H + k];
                        const int xx = x + k;
                        return (xx < 0 || xx >= nx) ? c : q[H + k];
                    };
                    Cx<R> lap;
                    if constexpr (H == 1) {
                        // power_series_operator.cu:50-58, summed in the reference's order
                        Cx<R> acc = nb_x(-1) + nb_x(1);
                        acc = acc + nb_y(-1);
                        acc = acc - scale(c, R(6));
                        acc = acc + nb_y(1);
                        acc = acc + nb_z(-1);
                        acc = acc + nb_z(1);
                        lap = mk<R>(acc.x / t.dxq / t.dxq, acc.y / t.dxq / t.dxq);
                    } else {
                        auto axis = [&](Cx<R> m2, Cx<R> m1, Cx<R> p1, Cx<R> p2, R cf) {
                            Cx<R> s16 = scale(m1 + p1, R(16));
                            Cx<R> u = (s16 - (m2 + p2)) - scale(c, R(30));
                            return scale(u, cf);
                        };
                        lap = axis(nb_x(-2), nb_x(-1), nb_x(1), nb_x(2), t.c4[0]);
                        lap = lap + axis(nb_y(-2), nb_y(-1), nb_y(1), nb_y(2), t.c4[1]);
                        lap = lap + axis(nb_z(-2), nb_z(-1), nb_z(1), nb_z(2), t.c4[2]);
                    }
                    const int64_t idx = int64_t(x) * plane + col;
                    const Cx<R> vs = cmul(mk<R>(R(vcur.x), R(vcur.y)), c);
                    const Cx<R> inner = mk<R>(t.inv2m * lap.x - vs.x, t.inv2m * lap.y - vs.y);
                    const Cx<R> sn = mk<R>(-t.a * inner.y, t.a * inner.x);
                    if (t.s_next) t.s_next[idx] = sn;
                    const Cx<R> old = term1 ? c : acur;
                    t.acc_out[idx] = old + sn;
                };
                if (inner_yz && x >= H && x + H < nx) term(std::true_type{});
                else if (in) term(std::false_type{});
                __syncthreads();  // tile[buf] is restaged for plane x + 2 in the next iteration
#pragma unroll
                for (int k = 0; k < 2 * H; ++k) q[k] = q[k + 1];
                q[2 * H] = qnext;
                vcur = vnext;
                acur = anext;
            }
        }
    }
    cp_async_wait<0>();
}

// One CTA per tile and chunk of XC x-planes; the chunk length is chosen on the host.
template <typename R, int H, bool VEC, int XC>
__global__ void __launch_bounds__(kTZ* kTY, WFS_MINB_TAYLOR) taylor_term_kernel(const TaylorArgs<R> t) {
    __shared__ __align__(16) Cx<R> tile[2][kTY + 2 * H][kTZ + 2 * kHZ];
    const int x0 = int(blockIdx.z) * XC;
    const int x1 = (x0 + XC < t.n[0]) ? x0 + XC : t.n[0];
    taylor_segment<R, H, VEC, (XC < 4 ? XC : 4)>(t, tile, int(blockIdx.x), int(blockIdx.y), x0, x1);
}

// x planes per CTA: the largest of 8, 4, 2 that still gives at least ~12 CTAs per
// SM over the launch (152 SMs), so that short CTAs keep every SM busy to the end;
// WFS_TAYLOR_XC in the environment fixes it (for tuning runs).
inline int taylor_xc(int64_t tiles_per_plane, int nx) {
    static const int forced = [] {
        const char* e = getenv("WFS_TAYLOR_XC");
        return e ? atoi(e) : 0;
    }();
    if (forced == 2 || forced == 4 || forced == 8) return forced;
    for (int xc : {8, 4}) {
        if (tiles_per_plane * ((nx + xc - 1) / xc) >= 152 * 12) return xc;
    }
    return 2;
}

template <typename R, int H, bool VEC>
cudaError_t run_taylor(const TaylorArgs<R>& t, cudaStream_t s) {
    const int64_t tiles = int64_t((t.n[2] + kTZ - 1) / kTZ) * ((t.n[1] + kTY - 1) / kTY);
    const int xc = taylor_xc(tiles, t.n[0]);
    dim3 grid((t.n[2] + kTZ - 1) / kTZ, (t.n[1] + kTY - 1) / kTY, (t.n[0] + xc - 1) / xc);
    if (xc == 8) taylor_term_kernel<R, H, VEC, 8><<<grid, kTZ * kTY, 0, s>>>(t);
    else if (xc == 4) taylor_term_kernel<R, H, VEC, 4><<<grid, kTZ * kTY, 0, s>>>(t);
    else taylor_term_kernel<R, H, VEC, 2><<<grid, kTZ * kTY, 0, s>>>(t);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_taylor_term(int stencil_order, const TaylorArgs<R>& t, cudaStream_t s) {
    if (int64_t(t.n[1]) * t.n[2] >= (int64_t(1) << 31)) return cudaErrorInvalidValue;
    const bool vec = sizeof(Cx<R>) == 8 && t.n[2] % 2 == 0 && (reinterpret_cast<uintptr_t>(t.s_prev) & 15) == 0;
    if (stencil_order == 2) return vec ? run_taylor<R, 1, true>(t, s) : run_taylor<R, 1, false>(t, s);
    return vec ? run_taylor<R, 2, true>(t, s) : run_taylor<R, 2, false>(t, s);
}
template cudaError_t launch_taylor_term<float>(int, const TaylorArgs<float>&, cudaStream_t);
template cudaError_t launch_taylor_term<double>(int, const TaylorArgs<double>&, cudaStream_t);

}  // namespace wfs
