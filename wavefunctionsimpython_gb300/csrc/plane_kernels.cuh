// plane_kernels.cuh — the y/z half of a split step in one launch.
//
//   Y[Fy^-1]  ->  Z[Fz^-1, E, Fz]  ->  Y[Fy]      on every x-plane
//
// One thread-block cluster owns one yz-plane. Its CTAs split the plane's
// y-pencil tiles (stage 1 and 3) and z-row tiles (stage 2) between them and
// meet at a cluster barrier between stages; the plane travels between the
// stages through L2 (in-place global writes, L2-only loads and stores), so HBM
// sees psi read once, psi written once and the phase table read once per site:
// 24 B/site for complex64, plus 16 B/site for the x pass = 40 B per site-step.
// Only the planes of the clusters in flight (a few tens of 512 KiB planes at
// 256^2 complex64) are live in L2 at any time, far below its 129 MB.
#pragma once

#include <cooperative_groups.h>

#include "fft_kernels.cuh"

namespace wfs {

template <typename R>
struct PlaneArgs {
    Cx<R>* data;             // psi, [nx][ny][nz]
    const Cx<R>* tw_y;       // roots of length ny
    const Cx<R>* tw_z;       // roots of length nz
    const Cx<R>* ephase;     // exp(-i dt V), [nx][ny][nz]
    int64_t plane_elems;     // ny * nz
    R scale_y;               // 1 / sqrt(ny) for each y stage
    R scale_z;               // 1 / nz for the z stage (inverse and forward)
};

template <typename R>
__device__ __forceinline__ Cx<R> ld_l2(const Cx<R>* p);
template <>
__device__ __forceinline__ Cx<float> ld_l2<float>(const Cx<float>* p) {
    float2 v = __ldcg(reinterpret_cast<const float2*>(p));
    return mk<float>(v.x, v.y);
}
template <>
__device__ __forceinline__ Cx<double> ld_l2<double>(const Cx<double>* p) {
    double2 v = __ldcg(reinterpret_cast<const double2*>(p));
    return mk<double>(v.x, v.y);
}
template <typename R>
__device__ __forceinline__ void st_l2(Cx<R>* p, Cx<R> v);
template <>
__device__ __forceinline__ void st_l2<float>(Cx<float>* p, Cx<float> v) {
    __stcg(reinterpret_cast<float2*>(p), make_float2(v.x, v.y));
}
template <>
__device__ __forceinline__ void st_l2<double>(Cx<double>* p, Cx<double> v) {
    __stcg(reinterpret_cast<double2*>(p), make_double2(v.x, v.y));
}
template <typename R>
__device__ __forceinline__ Cx<R> ld_stream(const Cx<R>* p);
template <>
__device__ __forceinline__ Cx<float> ld_stream<float>(const Cx<float>* p) {
    float2 v = __ldcs(reinterpret_cast<const float2*>(p));
    return mk<float>(v.x, v.y);
}
template <>
__device__ __forceinline__ Cx<double> ld_stream<double>(const Cx<double>* p) {
    double2 v = __ldcs(reinterpret_cast<const double2*>(p));
    return mk<double>(v.x, v.y);
}

// One y-pencil tile (LY rows x W contiguous z columns) of the plane, in place. tw is the axis
// table (TWL = TW_ROW) or, with TWL = TW_ROW_SMEM, the plan's row block in shared memory.
// (TP, TQ) is the plan the axis table was built for; (P, Q) may be its transpose.
template <typename R, int P, int Q, int W, int SIGN, int TWL = TW_ROW, int TP = P, int TQ = Q>
__device__ __forceinline__ void plane_y_tile(Cx<R>* plane, int nz, int tile, const Cx<R>* tw, R sc, Cx<R>* sm, int tid,
                                             int nthreads) {
    constexpr int T = cmax(P, Q);
    const bool in_block = tid < T * W;
    const int c = tid % W, t = tid / W;
    const int col = tile * W + c;
    const bool active = in_block && col < nz;
    Cx<R>* base = plane + col;
    Cx<R> a1[Q], a2[P];
    if (t < P) {
#pragma unroll
        for (int i = 0; i < Q; ++i) a1[i] = active ? ld_l2<R>(base + int64_t(t + P * i) * nz) : mk<R>(R(0), R(0));
    }
    auto sidx = [&](int k2, int n1) { return (k2 * P + n1) * W + c; };
    const Cx<R>* rows = (TWL == TW_ROW) ? tw_rows<P, Q, TP, TQ>(tw) : tw;
    two_stage<P, Q, SIGN, TWL>(a1, a2, sm, rows, in_block ? t : T, sidx);
    if (active && t < Q) {
#pragma unroll
        for (int k = 0; k < P; ++k) st_l2<R>(base + int64_t(t + Q * k) * nz, scale(a2[k], sc));
    }
    (void)nthreads;
}

// W rows of the plane: Fz^-1, multiply by e, Fz, in place.
template <typename R, int P, int Q, int W>
__device__ __forceinline__ void plane_z_tile(Cx<R>* plane, const Cx<R>* eplane, int ny, int tile, const Cx<R>* tw, R sc,
                                             Cx<R>* sm, int tid) {
    constexpr int L = P * Q, T = cmax(P, Q);
    constexpr int RS = cmax(Q * (P + 1), P * (Q + 1));
    const bool in_block = tid < T * W;
    const int t = tid % T, r = tid / T;
    const int row = tile * W + r;
    const bool active = in_block && row < ny;
    Cx<R>* rp = plane + int64_t(row) * L;
    const Cx<R>* ep = eplane + int64_t(row) * L;
    Cx<R> a1[Q], a2[P];
    if (t < P) {
#pragma unroll
        for (int i = 0; i < Q; ++i) a1[i] = active ? ld_l2<R>(rp + t + P * i) : mk<R>(R(0), R(0));
    }
    auto sidx_f = [&](int k2, int n1) { return r * RS + k2 * (P + 1) + n1; };
    auto sidx_i = [&](int k2, int n1) { return r * RS + k2 * (Q + 1) + n1; };
    const int tt = in_block ? t : T;
    two_stage<P, Q, +1, TW_ANGLE>(a1, a2, sm, tw, tt, sidx_f);
    if (tt < Q) {
#pragma unroll
        for (int k = 0; k < P; ++k) {
            Cx<R> e = active ? ld_stream<R>(ep + t + Q * k) : mk<R>(R(0), R(0));
            a2[k] = cmul(a2[k], scale(e, sc));
        }
    }
    __syncthreads();
    two_stage<Q, P, -1, TW_ANGLE>(a2, a1, sm, tw, tt, sidx_i);
    if (active && t < P) {
#pragma unroll
        for (int i = 0; i < Q; ++i) st_l2<R>(rp + t + P * i, a1[i]);
    }
}

template <typename R, int LY, int LZ, int CL, int NT, bool TSM = false>
__global__ void __launch_bounds__(NT, WFS_MINB_PLANE) plane_step_kernel(const PlaneArgs<R> a) {
    constexpr int PY = PlanOf<LY>::P, QY = PlanOf<LY>::Q, TY = cmax(PY, QY);
    constexpr int PZ = PlanOf<LZ>::P, QZ = PlanOf<LZ>::Q, TZ = cmax(PZ, QZ);
    constexpr int WY = StridedW<R, TY>::value;
    constexpr int WZ = ContigW<R, TZ>::value;
    static_assert(TY * WY <= NT && TZ * WZ <= NT, "block too small");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cx<R>* sm = reinterpret_cast<Cx<R>*>(smem_raw);
    const int tid = threadIdx.x;
    const int rank = int(blockIdx.x % CL);
    const int64_t plane_id = blockIdx.x / CL;
    Cx<R>* plane = a.data + plane_id * a.plane_elems;
    const Cx<R>* eplane = a.ephase + plane_id * a.plane_elems;
    constexpr int ntile_y = (LZ + WY - 1) / WY;
    constexpr int ntile_z = (LY + WZ - 1) / WZ;
    namespace cg = cooperative_groups;

    // the phase rows of this CTA's stage-2 tiles are contiguous blocks of W rows: L2 is
    // asked for them while the cluster waits at the stage barrier, so the phase loads of
    // stage 2 hit L2 (measured at 256^3: 154 -> 150 us per plane pass; issuing it when
    // the CTA starts gains less, and prefetching the second stage-1 tile gains nothing)
    auto prefetch_phase = [&]() {
        if (tid == 0) {
            for (int tile = rank; tile < ntile_z; tile += CL) {
                const int r0 = tile * WZ, nr = (LY - r0) < WZ ? (LY - r0) : WZ;
                const size_t bytes = size_t(nr) * LZ * sizeof(Cx<R>);
                const Cx<R>* p = eplane + int64_t(r0) * LZ;
                if ((reinterpret_cast<uintptr_t>(p) & 15) == 0 && (bytes & 15) == 0)
                    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(p), "r"(unsigned(bytes)) : "memory");
            }
        }
    };
    // TSM: the y plan's twiddle rows and the z angle table, copied once per CTA behind the
    // transpose buffer; every tile of the CTA reads them from shared memory instead of L1
    constexpr int RSZ = cmax(QZ * (PZ + 1), PZ * (QZ + 1));
    constexpr int TWL_Y = TSM ? TW_ROW_SMEM : TW_ROW;
    const Cx<R>* tw_y = a.tw_y;
    const Cx<R>* tw_z = a.tw_z;
    if constexpr (TSM) {
        Cx<R>* ty = sm + cmax(LY * WY, WZ * RSZ);
        Cx<R>* tz = ty + PY * QY;
        const Cx<R>* rows = tw_rows<PY, QY, PY, QY>(a.tw_y);
        for (int i = tid; i < PY * QY; i += NT) ty[i] = rows[i];
        for (int i = tid; i < LZ; i += NT) tz[i] = a.tw_z[i];
        __syncthreads();
        tw_y = ty;
        tw_z = tz;
    }
    for (int tile = rank; tile < ntile_y; tile += CL) {
        plane_y_tile<R, PY, QY, WY, +1, TWL_Y>(plane, LZ, tile, tw_y, a.scale_y, sm, tid, NT);
        __syncthreads();
    }
    prefetch_phase();
    if constexpr (CL > 1) cg::this_cluster().sync(); else __syncthreads();
    for (int tile = rank; tile < ntile_z; tile += CL) {
        plane_z_tile<R, PZ, QZ, WZ>(plane, eplane, LY, tile, tw_z, a.scale_z, sm, tid);
        __syncthreads();
    }
    if constexpr (CL > 1) cg::this_cluster().sync(); else __syncthreads();
    for (int tile = rank; tile < ntile_y; tile += CL) {
        plane_y_tile<R, PY, QY, WY, -1, TWL_Y>(plane, LZ, tile, tw_y, a.scale_y, sm, tid, NT);
        __syncthreads();
    }
}

// The plane pass reads its twiddles from shared memory (copied once per CTA);
// WFS_PLANE_SMEM_TABLES=0 in the environment reads them through L1 (for A/B timing).
inline bool plane_smem_tables_enabled() {
    static const int on = [] {
        const char* e = getenv("WFS_PLANE_SMEM_TABLES");
        return (e && e[0] == '0') ? 0 : 1;
    }();
    return on != 0;
}

template <typename R, int LY, int LZ, int CL, bool TSM_ON = true>
cudaError_t run_plane(const PlaneArgs<R>& a, int64_t nplanes, cudaStream_t s) {
    // complex64 only: the tables of a complex128 plane would cost the third CTA per SM
    constexpr bool TSM = TSM_ON && sizeof(R) == 4;
    if constexpr (TSM) {
        if (!plane_smem_tables_enabled()) return run_plane<R, LY, LZ, CL, false>(a, nplanes, s);
    }
    constexpr int PY = PlanOf<LY>::P, QY = PlanOf<LY>::Q, TY = cmax(PY, QY);
    constexpr int PZ = PlanOf<LZ>::P, QZ = PlanOf<LZ>::Q, TZ = cmax(PZ, QZ);
    constexpr int WY = StridedW<R, TY>::value;
    constexpr int WZ = ContigW<R, TZ>::value;
    constexpr int NT = cmax(TY * WY, TZ * WZ);
    constexpr int RSZ = cmax(QZ * (PZ + 1), PZ * (QZ + 1));
    const size_t smem = sizeof(Cx<R>) * (size_t(cmax(LY * WY, WZ * RSZ)) + (TSM ? size_t(PY * QY + LZ) : 0));
    auto kern = plane_step_kernel<R, LY, LZ, CL, NT, TSM>;
    static PerDevice attr_set;
    const int dev = current_device();
    if (!attr_set.get(dev)) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        if (CL > 8) {
            e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            if (e != cudaSuccess) return e;
        }
        attr_set.put(dev, 1);
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(nplanes * CL));
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a);
}

// Supported plane shapes: ny == nz from the list below; the cluster size grows with the plane.
#define WFS_FOR_EACH_PLANE(M) M(32, 1) M(48, 1) M(64, 2) M(96, 4) M(128, 8) M(192, 8) M(256, 8) M(384, 8) M(512, 8)

template <typename R>
cudaError_t dispatch_plane(int ny, int nz, const PlaneArgs<R>& a, int64_t nplanes, cudaStream_t s) {
    if (ny != nz) return cudaErrorInvalidValue;
#define WFS_CASE(L_, CL_) \
    case L_:              \
        return run_plane<R, L_, L_, CL_>(a, nplanes, s);
    switch (ny) {
        WFS_FOR_EACH_PLANE(WFS_CASE)
        default:
            return cudaErrorInvalidValue;
    }
#undef WFS_CASE
}

inline bool plane_supported(int ny, int nz) {
    if (ny != nz) return false;
    switch (ny) {
        case 32: case 48: case 64: case 96: case 128: case 192: case 256: case 384: case 512: return true;
        default: return false;
    }
}

}  // namespace wfs
