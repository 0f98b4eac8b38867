// taylor.cu — one term of the power-series propagator
// (sources/sim_state.py:721-752, sources/cuda_kernels/power_series_operator.cu:3-65):
//   s_n = i (dt/n) ( lap(s_{n-1}) / (2m) - V s_{n-1} ),   acc += s_n.
//
// Term 1 reads psi as s_0 and writes acc = psi + s_1 into a separate buffer,
// which removes the reference's per-step copy of psi (sim_state.py:730).
// Later terms update acc in place. Out-of-range stencil neighbours are replaced
// by the centre value (power_series_operator.cu:23-46).
//
// Tiling: each CTA covers a TZ x TY tile of one x-plane and marches along x.
// The tile (plus a halo of H = stencil_order/2 cells in y and z) of the
// current plane is staged in shared memory; the x-neighbours are held in a
// register queue, so s_{n-1} is read from memory about once per site.
#include "kernels.h"

namespace wfs {

constexpr int kTZ = 32;
constexpr int kTY = 8;
constexpr int kXC = 16;  // x-planes marched by one CTA

template <typename R, int H>
__global__ void __launch_bounds__(kTZ* kTY) taylor_term_kernel(const TaylorArgs<R> t) {
    constexpr int SZ = kTZ + 2 * H, SY = kTY + 2 * H;
    __shared__ Cx<R> tile[SY][SZ];
    const int nx = t.n[0], ny = t.n[1], nz = t.n[2];
    const int tz = threadIdx.x % kTZ, ty = threadIdx.x / kTZ;
    const int z = blockIdx.x * kTZ + tz;
    const int y = blockIdx.y * kTY + ty;
    const bool in = (z < nz) && (y < ny);
    const int64_t plane = int64_t(ny) * nz;
    const int zc = z < nz ? z : nz - 1, yc = y < ny ? y : ny - 1;
    const int64_t col = int64_t(yc) * nz + zc;

    const int x0 = int(blockIdx.z) * kXC;
    const int x1 = (x0 + kXC < nx) ? x0 + kXC : nx;
    // register queue along x: q[H + k] = s at x + k, k in [-H, H]
    // (entries outside the grid are never used: nb_x returns the centre there)
    Cx<R> q[2 * H + 1];
#pragma unroll
    for (int k = -H; k <= H; ++k) {
        int xx = x0 + k;
        if (xx < 0 || xx >= nx) xx = x0;
        q[H + k] = t.s_prev[int64_t(xx) * plane + col];
    }

    for (int x = x0; x < x1; ++x) {
        // stage plane x of s_prev (tile + halo) in shared memory
        __syncthreads();
        const Cx<R>* sp = t.s_prev + int64_t(x) * plane;
        for (int i = threadIdx.x; i < SY * SZ; i += kTZ * kTY) {
            const int ly = i / SZ, lz = i % SZ;
            int gy = int(blockIdx.y) * kTY + ly - H;
            int gz = int(blockIdx.x) * kTZ + lz - H;
            // clamp to the grid; the centre-replacement rule is applied below
            gy = gy < 0 ? 0 : (gy >= ny ? ny - 1 : gy);
            gz = gz < 0 ? 0 : (gz >= nz ? nz - 1 : gz);
            tile[ly][lz] = sp[int64_t(gy) * nz + gz];
        }
        __syncthreads();
        if (in) {
            const Cx<R> c = q[H];
            auto nb_y = [&](int k) -> Cx<R> {
                const int yy = y + k;
                return (yy < 0 || yy >= ny) ? c : tile[ty + H + k][tz + H];
            };
            auto nb_z = [&](int k) -> Cx<R> {
                const int zz = z + k;
                return (zz < 0 || zz >= nz) ? c : tile[ty + H][tz + H + k];
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
            const float2 v = t.V[idx];
            const Cx<R> vs = cmul(mk<R>(R(v.x), R(v.y)), c);
            const Cx<R> inner = mk<R>(t.inv2m * lap.x - vs.x, t.inv2m * lap.y - vs.y);
            const Cx<R> sn = mk<R>(-t.a * inner.y, t.a * inner.x);
            if (t.s_next) t.s_next[idx] = sn;
            const Cx<R> old = (t.acc_in == t.s_prev) ? c : t.acc_in[idx];
            t.acc_out[idx] = old + sn;
        }
        // advance the register queue
#pragma unroll
        for (int k = 0; k < 2 * H; ++k) q[k] = q[k + 1];
        const int xn = x + H + 1;
        if (xn < nx) q[2 * H] = t.s_prev[int64_t(xn) * plane + col];
    }
}

template <typename R>
cudaError_t launch_taylor_term(int stencil_order, const TaylorArgs<R>& t, cudaStream_t s) {
    dim3 grid((t.n[2] + kTZ - 1) / kTZ, (t.n[1] + kTY - 1) / kTY, (t.n[0] + kXC - 1) / kXC);
    if (stencil_order == 2) taylor_term_kernel<R, 1><<<grid, kTZ * kTY, 0, s>>>(t);
    else taylor_term_kernel<R, 2><<<grid, kTZ * kTY, 0, s>>>(t);
    return cudaGetLastError();
}
template cudaError_t launch_taylor_term<float>(int, const TaylorArgs<float>&, cudaStream_t);
template cudaError_t launch_taylor_term<double>(int, const TaylorArgs<double>&, cudaStream_t);

}  // namespace wfs
