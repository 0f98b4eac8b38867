// field_kernels.cu — construction of psi0 and V, phase tables, observables.
//
// The potential builders restate the reference's float32 formulas
// (sources/cuda_kernels/potential_wall.cu:4-83, absorbing_potential.cu:3-307)
// with every rounding spelled out: separately rounded multiplies and adds
// (__fmul_rn/__fadd_rn) where the reference's compiled code rounds them, and a
// fused multiply-add (__fmaf_rn) exactly where its compiler contracts a product
// into the add or subtract that consumes it. The reference is compiled with
// contraction on (NVRTC's default); in a sum or difference of two products the
// first product is fused, and a product added to an earlier result is fused into
// it. These fusions decide the voxels that lie exactly on a wall's plateau or
// slit edge, so the potential matches the reference's bit for bit.
#include "fft_kernels.cuh"

namespace wfs {

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }

__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// common.cu:65-68 as compiled: fma(a.z, b.z, fma(a.x, b.x, a.y*b.y))
__device__ __forceinline__ float dot3c(float ax, float ay, float az, float bx, float by, float bz) {
    return fma_(az, bz, fma_(ax, bx, fm(ay, by)));
}

// ---------------------------------------------------------------------------
// Potential wall — potential_wall.cu:30-82. Each thread forms the wall's frame
// (potential_wall.cu:39-45 with common.cu:70-77 cross, :220-223 normalize and
// :348-369 rotate_vector) as the reference's device code does, with the same
// cosf/sinf of the half angle and the same fused multiply-adds.
// ---------------------------------------------------------------------------
__device__ void wall_right(const WallDev& w, float r[3]) {
    float upx = 0.f, upy = 1.f, upz = 0.f;
    if (fabsf(dot3c(w.nx, w.ny, w.nz, upx, upy, upz)) > 0.99f) { upx = 0.f; upz = 1.f; }
    const float c0 = fma_(w.ny, upz, -fm(w.nz, upy));
    const float c1 = fma_(w.nz, upx, -fm(w.nx, upz));
    const float c2 = fma_(w.nx, upy, -fm(w.ny, upx));
    const float ln = __fsqrt_rn(dot3c(c0, c1, c2, c0, c1, c2));
    const float rt[3] = {__fdiv_rn(c0, ln), __fdiv_rn(c1, ln), __fdiv_rn(c2, ln)};
    const float half = __fdiv_rn(w.rot, 2.0f);
    const float q0 = cosf(half), sh = sinf(half);
    const float q1 = fm(sh, w.nx), q2 = fm(sh, w.ny), q3 = fm(sh, w.nz);
    float Q[3][3];
    Q[0][0] = fma_(-q3, q3, fma_(-q2, q2, fma_(q0, q0, fm(q1, q1))));
    Q[0][1] = fm(2.0f, fma_(q1, q2, -fm(q0, q3)));
    Q[0][2] = fm(2.0f, fma_(q1, q3, fm(q0, q2)));
    Q[1][0] = fm(2.0f, fma_(q2, q1, fm(q0, q3)));
    Q[1][1] = fma_(-q3, q3, fma_(q2, q2, fma_(q0, q0, -fm(q1, q1))));
    Q[1][2] = fm(2.0f, fma_(q2, q3, -fm(q0, q1)));
    Q[2][0] = fm(2.0f, fma_(q3, q1, -fm(q0, q2)));
    Q[2][1] = fm(2.0f, fma_(q3, q2, fm(q0, q1)));
    Q[2][2] = fma_(q3, q3, fma_(-q2, q2, fma_(q0, q0, -fm(q1, q1))));
    for (int i = 0; i < 3; ++i) r[i] = fma_(Q[i][2], rt[2], fma_(Q[i][0], rt[0], fm(Q[i][1], rt[1])));
}

// Voxel position dx * (v - N/2) of potential_wall.cu:34 (transform_corner_origin_to_center_origin_system).
__device__ __forceinline__ float wall_coord(int v, int n, float d) { return fm(d, fs(float(v), fm(0.5f, float(n)))); }

// Distance of the voxel at r from the wall's mid-plane, |n.(r - c)|.
__device__ __forceinline__ float wall_distance(const WallDev& w, float cx, float cy, float cz, float rx, float ry,
                                               float rz) {
    return fabsf(dot3c(w.nx, w.ny, w.nz, fs(rx, cx), fs(ry, cy), fs(rz, cz)));
}

// Adds the wall's value at r to acc (potential_wall.cu:46-82): nothing inside a slit or
// beyond the slope, U on the plateau, U (1 - (d - p/2)/s)^e on the slope.
__device__ __forceinline__ float wall_add(const WallDev& w, const float right[3], float acc, float rx, float ry,
                                          float rz) {
    const float ax = fs(rx, w.cx), ay = fs(ry, w.cy), az = fs(rz, w.cz);
    const float d = fabsf(dot3c(w.nx, w.ny, w.nz, ax, ay, az));
    const float dR = fabsf(dot3c(right[0], right[1], right[2], ax, ay, az));
    const float sw = w.slit_width, sp = w.slit_spacing;
    bool skip = false;
    switch (w.slit_count) {
        case 1: skip = dR < fm(sw, 0.5f); break;
        case 2: skip = dR > fm(fs(sp, sw), 0.5f) && dR < fm(fa(sp, sw), 0.5f); break;
        case 3:
            skip = (dR < fm(sw, 0.5f)) || (dR > fs(sp, fm(sw, 0.5f)) && dR < fa(sp, fm(sw, 0.5f)));
            break;
        case 4:
            skip = (dR > fm(fs(sp, sw), 0.5f) && dR < fm(fa(sp, sw), 0.5f)) ||
                   (dR > fma_(sp, 1.5f, -fm(sw, 0.5f)) && dR < fma_(sp, 1.5f, fm(sw, 0.5f)));
            break;
        default: break;
    }
    if (skip) return acc;
    const float p2 = fm(w.plateau, 0.5f);
    if (d <= p2) return fa(acc, w.U);
    if (d <= fa(p2, w.slope)) {
        const float tt = fs(1.0f, __fdiv_rn(fs(d, p2), w.slope));
        return fa(acc, fm(w.U, powf(tt, w.slope_exp)));
    }
    return acc;
}

__global__ void wall_kernel(float2* __restrict__ V, int nx, int ny, int nz, float dxx, float dxy, float dxz, WallDev w) {
    const int64_t total = int64_t(nx) * ny * nz;
    float right[3];
    wall_right(w, right);
    for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < total; idx += int64_t(gridDim.x) * blockDim.x) {
        const int z = int(idx % nz);
        const int y = int((idx / nz) % ny);
        const int x = int(idx / (int64_t(ny) * nz));
        const float rx = wall_coord(x, nx, dxx), ry = wall_coord(y, ny, dxy), rz = wall_coord(z, nz, dxz);
        const float v0 = V[idx].x;
        const float v1 = wall_add(w, right, v0, rx, ry, rz);
        if (v1 != v0 || __float_as_uint(v1) != __float_as_uint(v0)) V[idx].x = v1;
    }
}

cudaError_t launch_wall(float2* V, const int n[3], const float dx[3], const WallDev& w, cudaStream_t s) {
    const int64_t total = int64_t(n[0]) * n[1] * n[2];
    int grid = int((total + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    wall_kernel<<<grid, 256, 0, s>>>(V, n[0], n[1], n[2], dx[0], dx[1], dx[2], w);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Dynamic potential mode (sources/sim_state.py:466-509, sources/potential.py:508-522):
// after each step the moving walls advect and V is rebuilt from the walls and the
// absorbing ramp. Only voxels within a moving wall's reach (plateau/2 + slope) before or
// after the move can change; this kernel recomputes V.x there as the rebuild does (zero,
// then every wall in order) and refreshes the phase table entry with vphase's formula.
// ---------------------------------------------------------------------------
__global__ void wall_frames_kernel(float* __restrict__ frames, const WallDev* __restrict__ walls, int nwall) {
    const int i = threadIdx.x;
    if (i < nwall) wall_right(walls[i], frames + 3 * i);
}

cudaError_t launch_wall_frames(float* frames, const WallDev* walls, int nwall, cudaStream_t s) {
    wall_frames_kernel<<<1, 32, 0, s>>>(frames, walls, nwall);
    return cudaGetLastError();
}

template <typename R>
__device__ __forceinline__ Cx<R> vphase_one(float2 v, R dt);

template <typename R>
__global__ void __launch_bounds__(256) wall_band_kernel(float2* __restrict__ V, Cx<R>* __restrict__ e, R dt, int nx,
                                                        int ny, int nz, float dxx, float dxy, float dxz,
                                                        const DynWallsDev d) {
    // one thread per voxel of the box d.lo..d.hi: z from the thread, y and x from the grid
    const int z = d.lo[2] + int(blockIdx.x * blockDim.x + threadIdx.x);
    const int y = d.lo[1] + int(blockIdx.y);
    const int x = d.lo[0] + int(blockIdx.z);
    if (z > d.hi[2]) return;
    const float rx = wall_coord(x, nx, dxx), ry = wall_coord(y, ny, dxy), rz = wall_coord(z, nz, dxz);
    bool touched = false;
    for (int i = 0; i < d.nwall && !touched; ++i) {
        if (!d.moving[i]) continue;
        const WallDev& w = d.w[i];
        const float p2 = fm(w.plateau, 0.5f);
        const float reach = fmaxf(p2, fa(p2, w.slope));
        touched = wall_distance(w, w.cx, w.cy, w.cz, rx, ry, rz) <= reach ||
                  wall_distance(w, d.old_c[i][0], d.old_c[i][1], d.old_c[i][2], rx, ry, rz) <= reach;
    }
    if (!touched) return;
    float vr = 0.0f;
    for (int i = 0; i < d.nwall; ++i) {
        const float right[3] = {d.frames[3 * i], d.frames[3 * i + 1], d.frames[3 * i + 2]};
        vr = wall_add(d.w[i], right, vr, rx, ry, rz);
    }
    const int64_t idx = (int64_t(x) * ny + y) * nz + z;
    float2 v = V[idx];
    v.x = vr;
    V[idx] = v;
    if (e) e[idx] = vphase_one<R>(v, dt);
}

template <typename R>
cudaError_t launch_wall_band(float2* V, Cx<R>* e, double dt, const int n[3], const float dx[3], const DynWallsDev& d,
                             cudaStream_t s) {
    const int nzb = d.hi[2] - d.lo[2] + 1, nyb = d.hi[1] - d.lo[1] + 1, nxb = d.hi[0] - d.lo[0] + 1;
    if (nzb < 1 || nyb < 1 || nxb < 1) return cudaSuccess;
    const int block = nzb < 256 ? ((nzb + 31) / 32) * 32 : 256;
    const dim3 grid(unsigned((nzb + block - 1) / block), unsigned(nyb), unsigned(nxb));
    wall_band_kernel<R><<<grid, block, 0, s>>>(V, e, R(dt), n[0], n[1], n[2], dx[0], dx[1], dx[2], d);
    return cudaGetLastError();
}
template cudaError_t launch_wall_band<float>(float2*, Cx<float>*, double, const int*, const float*, const DynWallsDev&,
                                             cudaStream_t);
template cudaError_t launch_wall_band<double>(float2*, Cx<double>*, double, const int*, const float*,
                                              const DynWallsDev&, cudaStream_t);

// ---------------------------------------------------------------------------
// Absorbing boundary — absorbing_potential.cu:37-306
// ---------------------------------------------------------------------------
struct F3 { float x, y, z; };
__device__ __forceinline__ F3 f3(float a, float b, float c) { return F3{a, b, c}; }
// common.cu:394-397
// common.cu:394-397 as compiled: fma(z, w, (1-w) * fma(y, u, x*(1-u)))
__device__ __forceinline__ float mixf(F3 v, float u, float w) {
    return fma_(v.z, w, fm(fs(1.0f, w), fma_(v.y, u, fm(v.x, fs(1.0f, u)))));
}
// length(): sqrtf(dot(v, v)) (common.cu:215-218)
__device__ __forceinline__ float len3(float a, float b, float c) {
    return __fsqrt_rn(dot3c(a, b, c, a, b, c));
}
// sqrtf(a*a + b*b) as compiled: sqrt(fma(a, a, b*b))
__device__ __forceinline__ float hyp2(float a, float b) {
    return __fsqrt_rn(fma_(a, a, fm(b, b)));
}
__device__ __forceinline__ float ramp(float dist, float off, float maxD, float e, float pot) {
    return fm(powf(__fdiv_rn(fmaxf(fs(dist, off), 0.0f), maxD), e), pot);
}
__device__ __forceinline__ float ang(float num, float den) {  // atan(num/den)/pi*2
    return fm(__fdiv_rn(atanf(__fdiv_rn(num, den)), 3.14159265358979323846f), 2.0f);
}

__global__ void absorbing_kernel(float2* __restrict__ V, int nx, int ny, int nz, float dxx, float dxy, float dxz, AbsorbDev a) {
    const int64_t total = int64_t(nx) * ny * nz;
    const float off = a.offset;
    const F3 box_half = f3(fm(fm(0.5f, float(nx)), dxx), fm(fm(0.5f, float(ny)), dxy), fm(fm(0.5f, float(nz)), dxz));
    const F3 ab = f3(fabsf(a.bottom[0]), fabsf(a.bottom[1]), fabsf(a.bottom[2]));
    const F3 at = f3(fabsf(a.top[0]), fabsf(a.top[1]), fabsf(a.top[2]));
    for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < total; idx += int64_t(gridDim.x) * blockDim.x) {
        const int z = int(idx % nz);
        const int y = int((idx / nz) % ny);
        const int x = int(idx / (int64_t(ny) * nz));
        // delta_r * voxel - 0.5 N delta_r, the first product fused
        const float rx = fma_(dxx, float(x), -box_half.x);
        const float ry = fma_(dxy, float(y), -box_half.y);
        const float rz = fma_(dxz, float(z), -box_half.z);
        const float Bx = fs(rx, a.bottom[0]), By = fs(ry, a.bottom[1]), Bz = fs(rz, a.bottom[2]);
        const float Tx = fs(rx, a.top[0]), Ty = fs(ry, a.top[1]), Tz = fs(rz, a.top[2]);
        float pot = 0.0f;
        // maxD = box_half - (|corner| + offset), per component
        auto md = [&](float hx, float hy, float hz, float cx, float cy, float cz, float ox, float oy, float oz) {
            return f3(fs(hx, fa(cx, ox)), fs(hy, fa(cy, oy)), fs(hz, fa(cz, oz)));
        };
        const float h = 0.0f;
        // corners of the bottom plate
        if (Bx < 0.f && By < 0.f && Bz < 0.f) {
            float u = ang(By, Bx), v = ang(-Bz, hyp2(Bx, By));
            F3 m = md(box_half.x, box_half.y, box_half.z, ab.x, ab.y, ab.z, off, off, off);
            pot = ramp(len3(Bx, By, Bz), off, mixf(m, u, v), mixf(f3(a.en[0], a.en[1], a.en[2]), u, v), mixf(f3(a.pn[0], a.pn[1], a.pn[2]), u, v));
        } else if (Bx < 0.f && By < 0.f && Tz > 0.f) {
            float u = ang(By, Bx), v = ang(Tz, hyp2(Bx, By));
            F3 m = md(box_half.x, box_half.y, box_half.z, ab.x, ab.y, at.z, off, off, off);
            pot = ramp(len3(Bx, By, Tz), off, mixf(m, u, v), mixf(f3(a.en[0], a.en[1], a.ep[2]), u, v), mixf(f3(a.pn[0], a.pn[1], a.pp[2]), u, v));
        } else if (By < 0.f && Tx > 0.f && Tz > 0.f) {
            float u = ang(-By, Tx), v = ang(Tz, hyp2(Tx, By));
            F3 m = md(box_half.x, box_half.y, box_half.z, at.x, ab.y, at.z, off, off, off);
            pot = ramp(len3(Tx, By, Tz), off, mixf(m, u, v), mixf(f3(a.ep[0], a.en[1], a.ep[2]), u, v), mixf(f3(a.pp[0], a.pn[1], a.pp[2]), u, v));
        } else if (By < 0.f && Bz < 0.f && Tx > 0.f) {
            float u = ang(-By, Tx), v = ang(-Bz, hyp2(Tx, By));
            F3 m = md(box_half.x, box_half.y, box_half.z, at.x, ab.y, ab.z, off, off, off);
            pot = ramp(len3(Tx, By, Bz), off, mixf(m, u, v), mixf(f3(a.ep[0], a.en[1], a.en[2]), u, v), mixf(f3(a.pp[0], a.pn[1], a.pn[2]), u, v));
        }
        // corners of the top plate
        else if (Tx > 0.f && Ty > 0.f && Tz > 0.f) {
            float u = ang(Ty, Tx), v = ang(Tz, hyp2(Tx, Ty));
            F3 m = md(box_half.x, box_half.y, box_half.z, at.x, at.y, at.z, off, off, off);
            pot = ramp(len3(Tx, Ty, Tz), off, mixf(m, u, v), mixf(f3(a.ep[0], a.ep[1], a.ep[2]), u, v), mixf(f3(a.pp[0], a.pp[1], a.pp[2]), u, v));
        } else if (Bz < 0.f && Tx > 0.f && Ty > 0.f) {
            float u = ang(Ty, Tx), v = ang(-Bz, hyp2(Tx, Ty));
            F3 m = md(box_half.x, box_half.y, box_half.z, at.x, at.y, ab.z, off, off, off);
            pot = ramp(len3(Tx, Ty, Bz), off, mixf(m, u, v), mixf(f3(a.ep[0], a.ep[1], a.en[2]), u, v), mixf(f3(a.pp[0], a.pp[1], a.pn[2]), u, v));
        } else if (Bx < 0.f && Bz < 0.f && Ty > 0.f) {
            float u = ang(Ty, -Bx), v = ang(-Bz, hyp2(Bx, Ty));
            F3 m = md(box_half.x, box_half.y, box_half.z, ab.x, at.y, ab.z, off, off, off);
            pot = ramp(len3(Bx, Ty, Bz), off, mixf(m, u, v), mixf(f3(a.en[0], a.ep[1], a.en[2]), u, v), mixf(f3(a.pn[0], a.pp[1], a.pn[2]), u, v));
        } else if (Bx < 0.f && Ty > 0.f && Tz > 0.f) {
            float u = ang(Ty, -Bx), v = ang(Tz, hyp2(Bx, Ty));
            F3 m = md(box_half.x, box_half.y, box_half.z, ab.x, at.y, at.z, off, off, off);
            pot = ramp(len3(Bx, Ty, Tz), off, mixf(m, u, v), mixf(f3(a.en[0], a.ep[1], a.ep[2]), u, v), mixf(f3(a.pn[0], a.pp[1], a.pp[2]), u, v));
        }
        // bottom edges
        else if (Bx < 0.f && By < 0.f && Bz > 0.f && Tz < 0.f) {
            float u = ang(By, Bx);
            F3 m = md(box_half.x, box_half.y, box_half.z, ab.x, ab.y, h, off, off, h);
            pot = ramp(len3(Bx, By, h), off, mixf(m, u, 0.f), mixf(f3(a.en[0], a.en[1], h), u, 0.f), mixf(f3(a.pn[0], a.pn[1], h), u, 0.f));
        } else if (Bx > 0.f && By < 0.f && Tx < 0.f && Tz > 0.f) {
            float v = ang(Tz, -By);
            F3 m = md(box_half.x, box_half.y, box_half.z, h, ab.y, at.z, h, off, off);
            pot = ramp(len3(h, By, Tz), off, mixf(m, 0.f, v), mixf(f3(h, a.en[1], a.ep[2]), 1.f, v), mixf(f3(h, a.pn[1], a.pp[2]), 1.f, v));
        } else if (By < 0.f && Bz > 0.f && Tx > 0.f && Tz < 0.f) {
            float u = ang(-By, Tx);
            F3 m = md(box_half.x, box_half.y, box_half.z, at.x, ab.y, h, off, off, h);
            pot = ramp(len3(Tx, By, h), off, mixf(m, u, 0.f), mixf(f3(a.ep[0], a.en[1], h), u, 0.f), mixf(f3(a.pp[0], a.pn[1], h), u, 0.f));
        } else if (Bx > 0.f && By < 0.f && Bz < 0.f && Tx < 0.f) {
            float v = ang(Bz, By);
            F3 m = md(box_half.x, box_half.y, box_half.z, h, ab.y, ab.z, h, off, off);
            pot = ramp(len3(h, By, Bz), off, mixf(m, 0.f, v), mixf(f3(h, a.en[1], a.en[2]), 1.f, v), mixf(f3(h, a.pn[1], a.pn[2]), 1.f, v));
        }
        // pillar edges
        else if (Bx < 0.f && By > 0.f && Bz < 0.f && Ty < 0.f) {
            float v = ang(Bz, Bx);
            F3 m = md(box_half.x, box_half.y, box_half.z, ab.x, h, ab.z, off, h, off);
            pot = ramp(len3(Bx, h, Bz), off, mixf(m, 0.f, v), mixf(f3(a.en[0], h, a.en[2]), 0.f, v), mixf(f3(a.pn[0], h, a.pn[2]), 0.f, v));
        } else if (Bx < 0.f && By > 0.f && Ty < 0.f && Tz > 0.f) {
            float v = ang(Tz, -Bx);
            F3 m = md(box_half.x, box_half.y, box_half.z, ab.x, h, at.z, off, h, off);
            pot = ramp(len3(Bx, h, Tz), off, mixf(m, 0.f, v), mixf(f3(a.en[0], h, a.ep[2]), 0.f, v), mixf(f3(a.pn[0], h, a.pp[2]), 0.f, v));
        } else if (By > 0.f && Tx > 0.f && Ty < 0.f && Tz > 0.f) {
            float v = ang(Tz, Tx);
            F3 m = md(box_half.x, box_half.y, box_half.z, at.x, h, at.z, off, h, off);
            pot = ramp(len3(Tx, h, Tz), off, mixf(m, 0.f, v), mixf(f3(a.ep[0], h, a.ep[2]), 0.f, v), mixf(f3(a.pp[0], h, a.pp[2]), 0.f, v));
        } else if (By > 0.f && Bz < 0.f && Tx > 0.f && Ty < 0.f) {
            float v = ang(-Bz, Tx);
            F3 m = md(box_half.x, box_half.y, box_half.z, at.x, h, ab.z, off, h, off);
            pot = ramp(len3(Tx, h, Bz), off, mixf(m, 0.f, v), mixf(f3(a.ep[0], h, a.en[2]), 0.f, v), mixf(f3(a.pp[0], h, a.pn[2]), 0.f, v));
        }
        // top plane edges
        else if (Bx < 0.f && Bz > 0.f && Ty > 0.f && Tz < 0.f) {
            float u = ang(Ty, -Bx);
            F3 m = md(box_half.x, box_half.y, box_half.z, ab.x, at.y, h, off, off, h);
            pot = ramp(len3(Bx, Ty, h), off, mixf(m, u, 0.f), mixf(f3(a.en[0], a.ep[1], h), u, 0.f), mixf(f3(a.pn[0], a.pp[1], h), u, 0.f));
        } else if (Bx > 0.f && Tx < 0.f && Ty > 0.f && Tz > 0.f) {
            float v = ang(Tz, Ty);
            F3 m = md(box_half.x, box_half.y, box_half.z, h, at.y, at.z, h, off, off);
            pot = ramp(len3(h, Ty, Tz), off, mixf(m, 1.f, v), mixf(f3(h, a.ep[1], a.ep[2]), 1.f, v), mixf(f3(h, a.pp[1], a.pp[2]), 1.f, v));
        } else if (Bz > 0.f && Tx > 0.f && Ty > 0.f && Tz < 0.f) {
            float u = ang(Ty, Tx);
            F3 m = md(box_half.x, box_half.y, box_half.z, at.x, at.y, h, off, off, h);
            pot = ramp(len3(Tx, Ty, h), off, mixf(m, u, 0.f), mixf(f3(a.ep[0], a.ep[1], h), u, 0.f), mixf(f3(a.pp[0], a.pp[1], h), u, 0.f));
        } else if (Bx > 0.f && Bz < 0.f && Tx < 0.f && Ty > 0.f) {
            float v = ang(-Bz, Ty);
            F3 m = md(box_half.x, box_half.y, box_half.z, h, at.y, ab.z, h, off, off);
            pot = ramp(len3(h, Ty, Bz), off, mixf(m, 0.f, v), mixf(f3(h, a.ep[1], a.en[2]), 0.f, v), mixf(f3(h, a.pp[1], a.pn[2]), 0.f, v));
        }
        // box sides
        else if (Bx > 0.f && By < 0.f && Bz > 0.f && Tx < 0.f && Tz < 0.f) {
            pot = ramp(-By, off, fs(box_half.y, fa(ab.y, off)), a.en[1], a.pn[1]);
        } else if (Bx > 0.f && By > 0.f && Tx < 0.f && Ty < 0.f && Tz > 0.f) {
            pot = ramp(Tz, off, fs(box_half.z, fa(at.z, off)), a.ep[2], a.pp[2]);
        } else if (By > 0.f && Bz > 0.f && Tx > 0.f && Ty < 0.f && Tz < 0.f) {
            pot = ramp(Tx, off, fs(box_half.x, fa(at.x, off)), a.ep[0], a.pp[0]);
        } else if (Bx > 0.f && By > 0.f && Bz < 0.f && Tx < 0.f && Ty < 0.f) {
            pot = ramp(-Bz, off, fs(box_half.z, fa(ab.z, off)), a.en[2], a.pn[2]);
        } else if (Bx < 0.f && By > 0.f && Bz > 0.f && Ty < 0.f && Tz < 0.f) {
            pot = ramp(-Bx, off, fs(box_half.x, fa(ab.x, off)), a.en[0], a.pn[0]);
        } else if (Bx > 0.f && Bz > 0.f && Tx < 0.f && Ty > 0.f && Tz < 0.f) {
            pot = ramp(Ty, off, fs(box_half.y, fa(at.y, off)), a.ep[1], a.pp[1]);
        }
        V[idx].y = fa(V[idx].y, pot);
    }
}

cudaError_t launch_absorbing(float2* V, const int n[3], const float dx[3], const AbsorbDev& a, cudaStream_t s) {
    const int64_t total = int64_t(n[0]) * n[1] * n[2];
    int grid = int((total + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    absorbing_kernel<<<grid, 256, 0, s>>>(V, n[0], n[1], n[2], dx[0], dx[1], dx[2], a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Raw pre-initialised potential — sources/potential.py:47-55
// ---------------------------------------------------------------------------
__global__ void add_raw_kernel(float2* __restrict__ V, const void* __restrict__ src, int type, int64_t count) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x) {
        float re = 0.f, im = 0.f;
        switch (type) {
            case 0: re = reinterpret_cast<const float*>(src)[i]; break;
            case 1: re = float(reinterpret_cast<const double*>(src)[i]); break;
            case 2: { float2 v = reinterpret_cast<const float2*>(src)[i]; re = v.x; im = v.y; } break;
            default: { double2 v = reinterpret_cast<const double2*>(src)[i]; re = float(v.x); im = float(v.y); } break;
        }
        V[i].x += re;
        V[i].y += im;
    }
}
cudaError_t launch_add_raw(float2* V, const void* src, int raw_type, int64_t count, cudaStream_t s) {
    int grid = int((count + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    add_raw_kernel<<<grid, 256, 0, s>>>(V, src, raw_type, count);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Gaussian packet — gaussian_wave_packet.cu:27-42, common.cu:569-605.
// The per-axis envelopes g_d and coordinates r_d are precomputed (they depend
// on one index only); the product is formed in the reference's order.
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R rmul(R a, R b);
template <> __device__ __forceinline__ float rmul<float>(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double rmul<double>(double a, double b) { return __dmul_rn(a, b); }
template <typename R>
__device__ __forceinline__ R radd(R a, R b);
template <> __device__ __forceinline__ float radd<float>(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ double radd<double>(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ void sincos_r(float a, float* s, float* c) { sincosf(a, s, c); }
__device__ __forceinline__ void sincos_r(double a, double* s, double* c) { sincos(a, s, c); }
__device__ __forceinline__ float exp_r(float a) { return expf(a); }
__device__ __forceinline__ double exp_r(double a) { return exp(a); }

template <typename R>
__global__ void gaussian_kernel(Cx<R>* __restrict__ psi, int nx, int ny, int nz, const R* __restrict__ gx,
                                const R* __restrict__ gy, const R* __restrict__ gz, const R* __restrict__ rx,
                                const R* __restrict__ ry, const R* __restrict__ rz, R kx, R ky, R kz) {
    const int64_t total = int64_t(nx) * ny * nz;
    for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < total; idx += int64_t(gridDim.x) * blockDim.x) {
        const int z = int(idx % nz);
        const int y = int((idx / nz) % ny);
        const int x = int(idx / (int64_t(ny) * nz));
        const R g = rmul(rmul(gx[x], gy[y]), gz[z]);
        const R ph = radd(radd(rmul(kx, rx[x]), rmul(ky, ry[y])), rmul(kz, rz[z]));
        R s, c;
        sincos_r(ph, &s, &c);
        psi[idx] = mk<R>(rmul(g, c), rmul(g, s));
    }
}
template <typename R>
cudaError_t launch_gaussian(Cx<R>* psi, const int n[3], const R* gx, const R* gy, const R* gz, const R* rx,
                            const R* ry, const R* rz, R kx, R ky, R kz, cudaStream_t s) {
    const int64_t total = int64_t(n[0]) * n[1] * n[2];
    int grid = int((total + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    gaussian_kernel<R><<<grid, 256, 0, s>>>(psi, n[0], n[1], n[2], gx, gy, gz, rx, ry, rz, kx, ky, kz);
    return cudaGetLastError();
}
template cudaError_t launch_gaussian<float>(Cx<float>*, const int*, const float*, const float*, const float*,
                                            const float*, const float*, const float*, float, float, float, cudaStream_t);
template cudaError_t launch_gaussian<double>(Cx<double>*, const int*, const double*, const double*, const double*,
                                             const double*, const double*, const double*, double, double, double,
                                             cudaStream_t);

// ---------------------------------------------------------------------------
// Potential phase table e = cexp_i(-dt V) = e^{-i dt ReV} e^{dt ImV}
// (potential_operator.cu:11-15, common.cu:98-111), in the wave function's precision.
// ---------------------------------------------------------------------------
// exp(-i dt V) = (cos(-dt Vr), sin(-dt Vr)) exp(dt Vi) (potential_operator.cu:11-15, common.cu:98-111)
template <typename R>
__device__ __forceinline__ Cx<R> vphase_one(float2 v, R dt) {
    const R re = -dt * R(v.x);
    const R im = -dt * R(v.y);
    R s, c;
    sincos_r(re, &s, &c);
    const R m = exp_r(-im);
    return mk<R>(c * m, s * m);
}

template <typename R>
__global__ void vphase_kernel(Cx<R>* __restrict__ e, const float2* __restrict__ V, R dt, int64_t count) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x)
        e[i] = vphase_one<R>(V[i], dt);
}
template <typename R>
cudaError_t launch_vphase(Cx<R>* e, const float2* V, double dt, int64_t count, cudaStream_t s) {
    int grid = int((count + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    vphase_kernel<R><<<grid, 256, 0, s>>>(e, V, R(dt), count);
    return cudaGetLastError();
}
template cudaError_t launch_vphase<float>(Cx<float>*, const float2*, double, int64_t, cudaStream_t);
template cudaError_t launch_vphase<double>(Cx<double>*, const float2*, double, int64_t, cudaStream_t);

// out[x][y][z] = kx[x] * ky[y] * kz[z]  (kinetic operator array for the operators module)
template <typename R>
__global__ void kin_product_kernel(Cx<R>* __restrict__ out, const Cx<R>* kx, const Cx<R>* ky, const Cx<R>* kz, int nx, int ny, int nz) {
    const int64_t total = int64_t(nx) * ny * nz;
    for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < total; idx += int64_t(gridDim.x) * blockDim.x) {
        const int z = int(idx % nz);
        const int y = int((idx / nz) % ny);
        const int x = int(idx / (int64_t(ny) * nz));
        out[idx] = cmul(cmul(kx[x], ky[y]), kz[z]);
    }
}
template <typename R>
cudaError_t launch_kin_product(Cx<R>* out, const Cx<R>* kx, const Cx<R>* ky, const Cx<R>* kz, const int n[3], cudaStream_t s) {
    const int64_t total = int64_t(n[0]) * n[1] * n[2];
    int grid = int((total + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    kin_product_kernel<R><<<grid, 256, 0, s>>>(out, kx, ky, kz, n[0], n[1], n[2]);
    return cudaGetLastError();
}
template cudaError_t launch_kin_product<float>(Cx<float>*, const Cx<float>*, const Cx<float>*, const Cx<float>*, const int*, cudaStream_t);
template cudaError_t launch_kin_product<double>(Cx<double>*, const Cx<double>*, const Cx<double>*, const Cx<double>*, const int*, cudaStream_t);

template <typename R>
__global__ void mul_inplace_kernel(Cx<R>* __restrict__ io, const Cx<R>* __restrict__ f, int64_t count) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x)
        io[i] = cmul(io[i], f[i]);
}
template <typename R>
cudaError_t launch_mul_inplace(Cx<R>* inout, const Cx<R>* f, int64_t count, cudaStream_t s) {
    int grid = int((count + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    mul_inplace_kernel<R><<<grid, 256, 0, s>>>(inout, f, count);
    return cudaGetLastError();
}
template cudaError_t launch_mul_inplace<float>(Cx<float>*, const Cx<float>*, int64_t, cudaStream_t);
template cudaError_t launch_mul_inplace<double>(Cx<double>*, const Cx<double>*, int64_t, cudaStream_t);

// ---------------------------------------------------------------------------
// Observables on real-space psi: one warp per (x, y) row, per-CTA FP64 partials.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(32 * kObsRowsPerCta) observe_real_kernel(const Cx<R>* __restrict__ psi, const ObsArgs o) {
    __shared__ double scratch[(kMaxBox + kLocQ) * 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t nrows = int64_t(o.n[0]) * o.n[1];
    const int64_t row = int64_t(blockIdx.x) * kObsRowsPerCta + warp;
    const bool own = row < nrows;
    const int x = own ? int(row / o.n[1]) : 0, y = own ? int(row % o.n[1]) : 0;
    const Cx<R>* rp = psi + (own ? row : 0) * o.n[2];
    auto p2 = [&](int z) { return abs2(rp[z]); };
    // one pass per requested box over the z range where its Simpson weight is nonzero
#pragma unroll 1
    for (int b = 0; b < o.nbox; ++b) {
        const ObsBox bx = o.box[b];
        const R wxy = own ? simpson_w<R>(x, bx.b[0], bx.c[0]) * simpson_w<R>(y, bx.b[1], bx.c[1]) : R(0);
        CSum<R> sz;
        if (wxy != R(0)) {
            const int z0 = bx.b[2] > 0 ? bx.b[2] : 0;
            const int z1 = (bx.b[2] + bx.c[2]) < o.n[2] ? (bx.b[2] + bx.c[2]) : o.n[2];
            for (int z = z0 + lane; z < z1; z += 32) sz.add(simpson_w<R>(z, bx.b[2], bx.c[2]) * p2(z));
        }
        warp_sum_to<R>(sz.scaled(wxy), scratch, b);
    }
    if (o.has_loc) {
        const R lxy = own ? simpson_w<R>(x, o.loc.b[0], o.loc.c[0]) * simpson_w<R>(y, o.loc.b[1], o.loc.c[1]) : R(0);
        CSum<R> s0, s1, s2;
        if (lxy != R(0)) {
            const int z0 = o.loc.b[2] > 0 ? o.loc.b[2] : 0;
            const int z1 = (o.loc.b[2] + o.loc.c[2]) < o.n[2] ? (o.loc.b[2] + o.loc.c[2]) : o.n[2];
            for (int z = z0 + lane; z < z1; z += 32) {
                const R w = simpson_w<R>(z, o.loc.b[2], o.loc.c[2]) * p2(z);
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
template <typename R>
cudaError_t launch_observe_real(const Cx<R>* psi, const ObsArgs& o, cudaStream_t s, int* grid_out) {
    const int64_t nrows = int64_t(o.n[0]) * o.n[1];
    const int grid = int((nrows + kObsRowsPerCta - 1) / kObsRowsPerCta);
    *grid_out = grid;
    observe_real_kernel<R><<<grid, 32 * kObsRowsPerCta, 0, s>>>(psi, o);
    return cudaGetLastError();
}
template cudaError_t launch_observe_real<float>(const Cx<float>*, const ObsArgs&, cudaStream_t, int*);
template cudaError_t launch_observe_real<double>(const Cx<double>*, const ObsArgs&, cudaStream_t, int*);

// Deterministic second stage: out[q] = sum over CTAs of partials[cta][q].
__global__ void reduce_partials_kernel(const double* __restrict__ partials, int nblocks, int nq, double* __restrict__ out) {
    __shared__ double sh[256];
    for (int q = 0; q < nq; ++q) {
        double s = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[int64_t(b) * nq + q];
        sh[threadIdx.x] = s;
        __syncthreads();
        for (int off = blockDim.x / 2; off > 0; off >>= 1) {
            if (threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[q] = sh[0];
        __syncthreads();
    }
}
cudaError_t launch_reduce_partials(const double* partials, int nblocks, int nq, double* out, cudaStream_t s) {
    reduce_partials_kernel<<<1, 256, 0, s>>>(partials, nblocks, nq, out);
    return cudaGetLastError();
}

// FP64 norm over the whole grid and a non-finite flag.
template <typename R>
__global__ void __launch_bounds__(256) norm_kernel(const Cx<R>* __restrict__ psi, int64_t count, double* partials, int* flag) {
    __shared__ double scratch[32];
    CSum<R> st;  // compensated per-thread sum
    bool bad = false;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x) {
        const R p = abs2(psi[i]);
        if (!isfinite(p)) bad = true;
        st.add(p);
    }
    if (bad) atomicExch(flag, 1);
    double s = st.value();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) scratch[warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) t += scratch[w];
        partials[blockIdx.x] = t;
    }
}
template <typename R>
cudaError_t launch_norm(const Cx<R>* psi, int64_t count, double* partials, int* nblocks, int* flag, cudaStream_t s) {
    int grid = int((count + 255) / 256);
    if (grid > 152 * 8) grid = 152 * 8;
    *nblocks = grid;
    norm_kernel<R><<<grid, 256, 0, s>>>(psi, count, partials, flag);
    return cudaGetLastError();
}
template cudaError_t launch_norm<float>(const Cx<float>*, int64_t, double*, int*, int*, cudaStream_t);
template cudaError_t launch_norm<double>(const Cx<double>*, int64_t, double*, int*, int*, cudaStream_t);

}  // namespace wfs
