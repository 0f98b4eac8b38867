// current.cu — probability flux through a sampled plane
// (sources/cuda_kernels/probability_current_density.cu:11-218, sources/measurement.py:190-303).
//
// Sample (px, py) of an sx x sy grid on the plane sits at
//   r = c + (right*dW)*(px - sx/2) + (up*dH)*(py - sy/2)            (float32, each op rounded)
// and takes psi and its 6th-order central derivative along the normal at the
// voxel trunc(r/dx + N/2) (clamped to the grid; out-of-range stencil
// neighbours are replaced by the centre, as in the reference). The density is
//   j.n = (-hbar/2m) Re(i (psi* dpsi - psi dpsi*)) = Im(psi* dpsi) / m,
// integrated with 2D Simpson weights; per-thread and warp sums compensated
// (CSum, fft_kernels.cuh), block and grid sums in FP64 (deterministic order).
#include "fft_kernels.cuh"

namespace wfs {

__device__ __forceinline__ float cfm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float cfa(float a, float b) { return __fadd_rn(a, b); }

template <typename R>
__global__ void __launch_bounds__(256) plane_current_kernel(const Cx<R>* __restrict__ psi, PlaneCurrentArgs a,
                                                            double* __restrict__ partials, R* __restrict__ density) {
    __shared__ double red[32];
    const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
    const int64_t total = int64_t(a.sx) * a.sy;
    CSum<R> acc;
    for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < total; p += int64_t(gridDim.x) * blockDim.x) {
        const int px = int(p / a.sy), py = int(p % a.sy);
        const float ax = float(px - a.sx / 2), ay = float(py - a.sy / 2);
        float rr[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
            rr[k] = cfa(cfa(a.center[k], cfm(cfm(a.right[k], a.dWf), ax)), cfm(cfm(a.up[k], a.dHf), ay));
        int v[3];
        const int N[3] = {nx, ny, nz};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const R fv = R(rr[k]) / R(a.dx[k]) + R(0.5) * R(N[k]);
            int iv = fv > R(0) ? int(fv) : 0;
            v[k] = iv >= N[k] ? N[k] - 1 : iv;
        }
        auto at = [&](int x, int y, int z) { return psi[(int64_t(x) * ny + y) * nz + z]; };
        const Cx<R> c = at(v[0], v[1], v[2]);
        Cx<R> dpsi = mk<R>(R(0), R(0));
#pragma unroll
        for (int axis = 0; axis < 3; ++axis) {
            auto nb = [&](int k) {
                int w[3] = {v[0], v[1], v[2]};
                const int m = w[axis] + k;
                if (m >= 0 && m <= N[axis] - 1) w[axis] = m;
                return at(w[0], w[1], w[2]);
            };
            const Cx<R> p3 = nb(3), p2 = nb(2), p1 = nb(1), m1 = nb(-1), m2 = nb(-2), m3 = nb(-3);
            const R inv = R(1) / (R(60) * R(a.dx[axis]));
            const R gx = ((p3.x - R(9) * p2.x) + R(45) * (p1.x - m1.x) + R(9) * m2.x - m3.x) * inv;
            const R gy = ((p3.y - R(9) * p2.y) + R(45) * (p1.y - m1.y) + R(9) * m2.y - m3.y) * inv;
            dpsi.x += R(a.normal[axis]) * gx;
            dpsi.y += R(a.normal[axis]) * gy;
        }
        const R dens = (c.x * dpsi.y - c.y * dpsi.x) / R(a.mass);
        if (density) density[p] = dens;
        R wx = (px == 0 || px == a.sx - 1) ? R(1) : ((px & 1) ? R(4) : R(2));
        R wy = (py == 0 || py == a.sy - 1) ? R(1) : ((py & 1) ? R(4) : R(2));
        acc.add(dens * (wx * wy));
    }
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) acc.merge(acc.shfl_xor(m));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = acc.value();
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) s += red[w];
        partials[blockIdx.x] = s;
    }
}

template <typename R>
cudaError_t launch_plane_current(const Cx<R>* psi, const PlaneCurrentArgs& a, double* partials, int max_blocks,
                                 R* density, cudaStream_t s, int* grid_out) {
    const int64_t total = int64_t(a.sx) * a.sy;
    int grid = int((total + 255) / 256);
    if (grid > max_blocks) grid = max_blocks;
    if (grid < 1) grid = 1;
    *grid_out = grid;
    plane_current_kernel<R><<<grid, 256, 0, s>>>(psi, a, partials, density);
    return cudaGetLastError();
}
template cudaError_t launch_plane_current<float>(const Cx<float>*, const PlaneCurrentArgs&, double*, int, float*,
                                                 cudaStream_t, int*);
template cudaError_t launch_plane_current<double>(const Cx<double>*, const PlaneCurrentArgs&, double*, int, double*,
                                                  cudaStream_t, int*);

}  // namespace wfs
