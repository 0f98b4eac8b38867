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
// through XC planes. The tile (plus a halo of H = stencil_order/2 cells in y and
// z) of each plane is staged in shared memory with cp.async into one of two
// buffers, so the next plane's copy is in flight while the current plane is
// computed; V, the accumulator and the next x-neighbour are loaded one plane
// ahead into registers. The x-neighbours are held in a register queue, so
// s_{n-1} is read from memory about once per site.
#include <cstdlib>

#include "fft_kernels.cuh"
#include "kernels.h"

namespace wfs {

constexpr int kTZ = 32;
constexpr int kTY = 8;

template <typename R, int H, int XC>
__global__ void __launch_bounds__(kTZ* kTY) taylor_term_kernel(const TaylorArgs<R> t) {
    constexpr int SZ = kTZ + 2 * H, SY = kTY + 2 * H;
    __shared__ __align__(16) Cx<R> tile[2][SY][SZ];
    const int nx = t.n[0], ny = t.n[1], nz = t.n[2];
    const int tz = threadIdx.x % kTZ, ty = threadIdx.x / kTZ;
    const int z = blockIdx.x * kTZ + tz;
    const int y = blockIdx.y * kTY + ty;
    const bool in = (z < nz) && (y < ny);
    const int64_t plane = int64_t(ny) * nz;
    const int zc = z < nz ? z : nz - 1, yc = y < ny ? y : ny - 1;
    const int64_t col = int64_t(yc) * nz + zc;
    const bool term1 = t.acc_in == t.s_prev;  // the accumulator starts from psi = s_0

    const int x0 = int(blockIdx.z) * XC;
    const int x1 = (x0 + XC < nx) ? x0 + XC : nx;
    auto stage = [&](int x, int buf) {
        const Cx<R>* sp = t.s_prev + int64_t(x) * plane;
        for (int i = threadIdx.x; i < SY * SZ; i += kTZ * kTY) {
            const int ly = i / SZ, lz = i % SZ;
            int gy = int(blockIdx.y) * kTY + ly - H;
            int gz = int(blockIdx.x) * kTZ + lz - H;
            // clamp to the grid; the centre-replacement rule is applied below
            gy = gy < 0 ? 0 : (gy >= ny ? ny - 1 : gy);
            gz = gz < 0 ? 0 : (gz >= nz ? nz - 1 : gz);
            cp_async_elem<sizeof(Cx<R>)>(&tile[buf][ly][lz], sp + int64_t(gy) * nz + gz);
        }
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
    int buf = 0;
    for (int x = x0; x < x1; ++x) {
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
        if (in) {
            const Cx<R> c = q[H];
            auto nb_y = [&](int k) -> Cx<R> {
                const int yy = y + k;
                return (yy < 0 || yy >= ny) ? c : tile[buf][ty + H + k][tz + H];
            };
            auto nb_z = [&](int k) -> Cx<R> {
                const int zz = z + k;
                return (zz < 0 || zz >= nz) ? c : tile[buf][ty + H][tz + H + k];
            };
            auto nb_x = [&](int k) -> Cx<R> {
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
        }
        __syncthreads();  // tile[buf] is restaged for plane x + 2 in the next iteration
        // advance the register queue
#pragma unroll
        for (int k = 0; k < 2 * H; ++k) q[k] = q[k + 1];
        q[2 * H] = qnext;
        vcur = vnext;
        acur = anext;
        buf ^= 1;
    }
    cp_async_wait<0>();
}

// x planes per CTA: the largest of 16, 8, 4 that still gives at least ~6 CTAs per
// SM (152 SMs); WFS_TAYLOR_XC in the environment fixes it (for tuning runs).
inline int taylor_xc(int64_t tiles_per_plane, int nx) {
    static const int forced = [] {
        const char* e = getenv("WFS_TAYLOR_XC");
        return e ? atoi(e) : 0;
    }();
    if (forced == 4 || forced == 8 || forced == 16) return forced;
    for (int xc : {16, 8}) {
        if (tiles_per_plane * ((nx + xc - 1) / xc) >= 152 * 6) return xc;
    }
    return 4;
}

template <typename R>
cudaError_t launch_taylor_term(int stencil_order, const TaylorArgs<R>& t, cudaStream_t s) {
    const int64_t tiles = int64_t((t.n[2] + kTZ - 1) / kTZ) * ((t.n[1] + kTY - 1) / kTY);
    const int xc = taylor_xc(tiles, t.n[0]);
    dim3 grid((t.n[2] + kTZ - 1) / kTZ, (t.n[1] + kTY - 1) / kTY, (t.n[0] + xc - 1) / xc);
#define WFS_TAYLOR(XC_)                                                                           \
    if (xc == XC_) {                                                                              \
        if (stencil_order == 2) taylor_term_kernel<R, 1, XC_><<<grid, kTZ * kTY, 0, s>>>(t);     \
        else taylor_term_kernel<R, 2, XC_><<<grid, kTZ * kTY, 0, s>>>(t);                        \
    }
    WFS_TAYLOR(16)
    WFS_TAYLOR(8)
    WFS_TAYLOR(4)
#undef WFS_TAYLOR
    return cudaGetLastError();
}
template cudaError_t launch_taylor_term<float>(int, const TaylorArgs<float>&, cudaStream_t);
template cudaError_t launch_taylor_term<double>(int, const TaylorArgs<double>&, cudaStream_t);

}  // namespace wfs
