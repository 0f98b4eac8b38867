// batch.cu — batched split-step sweep engine (many packets on uneven grids).
//
// All instances live in one slab (instance-major, each a C-ordered L^3
// complex64 cube). One kernel launch advances every instance by one Strang
// step: a thread-block cluster owns one instance and walks it through
//   X[Fx K Fx^-1] -> Y[Fy^-1] -> Z[Fz^-1 E Fz] -> Y[Fy]
// with a cluster barrier between stages. The instance travels between stages
// through L2 (L2-only loads/stores), so HBM sees psi read once, written once
// and E read once per site-step: 24 B/site-step for complex64. Clusters take
// instances largest first, so the hardware's cluster scheduler load-balances
// the uneven sizes. Launches of a run are captured in a CUDA graph and
// replayed. The cluster size and the radix orientation of every size class
// are chosen by timing (wfs_batch_autotune).
//
// Two-pass mode (cluster setting 0, the default): each step is, per size class,
//   an x pass X[Fx K Fx^-1] with one (instance, column tile) per CTA, then
//   a plane pass with one yz-plane per CTA held whole in shared memory
//   (an L = 96 plane is 72 KB): Y[Fy^-1] -> Z[Fz^-1 E Fz] -> Y[Fy] there,
// so psi is read and written once per pass and E once per step (40 B/site-step)
// with no cluster barriers and no stage data in L2. The one-launch cluster mode
// reads less in principle (24 B/site-step) but the 16 96^3 instances of the sweep
// run together and their live stage data overflows L2. Entering and leaving the
// frequency-space representation use the cluster programs in both modes.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/wfs.h"
#include "host_helpers.h"
#include "per_device.h"
#include "plane_kernels.cuh"

using namespace wfs;

namespace {

struct InstDesc {
    Cx<float>* psi;
    const Cx<float>* ephase;
    const Cx<float>* kin;   // [half x][half y][half z][full x][full y][full z], L each
    const Cx<float>* tw;    // two-stage twiddle table (3L entries, two_stage_roots)
    int L;
    float sy;               // 1/sqrt(L) rounded from double on the host (y stages, unpaired z stages)
};

enum Prog { PROG_ENTER = 0, PROG_STEP_HALF = 1, PROG_STEP_FULL = 2, PROG_FINISH = 3 };

template <bool SWAP, int L>
struct BPlan {
    // (P, Q): the plan the kernels run; (TP, TQ): the plan of the axis table (two_stage_roots),
    // whose row blocks are addressed by it
    static constexpr int TP = PlanOf<L>::P, TQ = PlanOf<L>::Q;
    static constexpr int P = SWAP ? PlanOf<L>::Q : PlanOf<L>::P;
    static constexpr int Q = SWAP ? PlanOf<L>::P : PlanOf<L>::Q;
    static constexpr int T = cmax(P, Q);
    static constexpr int WS = StridedW<float, T>::value;
    static constexpr int WC = ContigW<float, T>::value;
};

// x pass over one instance: pencils along x (row stride L^2), W columns per tile.
template <int P, int Q, int W, int TP, int TQ>
__device__ __forceinline__ void x_kin_tile(const InstDesc& in, int tile, const Cx<float>* k3, Cx<float>* sm, int tid) {
    constexpr int T = cmax(P, Q);
    const int L = in.L;
    const int64_t plane = int64_t(L) * L;
    const bool in_block = tid < T * W;
    const int c = tid % W, t = tid / W;
    const int col = tile * W + c;
    const bool active = in_block && col < plane;
    Cx<float>* base = in.psi + col;
    Cx<float> a1[Q], a2[P];
    if (t < P) {
#pragma unroll
        for (int i = 0; i < Q; ++i) a1[i] = active ? ld_l2<float>(base + int64_t(t + P * i) * plane) : mk<float>(0.f, 0.f);
    }
    auto sf = [&](int k2, int n1) { return (k2 * P + n1) * W + c; };
    auto si = [&](int k2, int n1) { return (k2 * Q + n1) * W + c; };
    const int tt = in_block ? t : T;
    two_stage<P, Q, -1, TW_ROW>(a1, a2, sm, tw_rows<P, Q, TP, TQ>(in.tw), tt, sf);
    if (tt < Q) {
        Cx<float> cf = mk<float>(0.f, 0.f);
        if (active) cf = scale(cmul(k3[L + col / L], k3[2 * L + col % L]), 1.0f / float(L));
#pragma unroll
        for (int k = 0; k < P; ++k) a2[k] = cmul(a2[k], cmul(k3[t + Q * k], cf));
    }
    __syncthreads();
    two_stage<Q, P, +1, TW_ROW>(a2, a1, sm, tw_rows<Q, P, TP, TQ>(in.tw), tt, si);
    if (active && t < P) {
#pragma unroll
        for (int i = 0; i < Q; ++i) st_l2<float>(base + int64_t(t + P * i) * plane, a1[i]);
    }
}

// plain z transform of W rows (forward SIGN -1 / inverse +1), scale 1/sqrt(L)
template <int P, int Q, int W, int SIGN>
__device__ __forceinline__ void z_plain_tile(const InstDesc& in, int tile, Cx<float>* sm, int tid) {
    constexpr int T = cmax(P, Q), RS = cmax(Q * (P + 1), P * (Q + 1));
    const int L = in.L;
    const bool in_block = tid < T * W;
    const int t = tid % T, r = tid / T;
    const int row = tile * W + r;
    const bool active = in_block && row < L * L;
    Cx<float>* rp = in.psi + int64_t(row) * L;
    Cx<float> a1[Q], a2[P];
    if (t < P) {
#pragma unroll
        for (int i = 0; i < Q; ++i) a1[i] = active ? ld_l2<float>(rp + t + P * i) : mk<float>(0.f, 0.f);
    }
    auto sf = [&](int k2, int n1) { return r * RS + k2 * (P + 1) + n1; };
    const int tt = in_block ? t : T;
    two_stage<P, Q, SIGN, TW_ANGLE>(a1, a2, sm, in.tw, tt, sf);
    const float sc = in.sy;
    if (active && t < Q) {
#pragma unroll
        for (int k = 0; k < P; ++k) st_l2<float>(rp + t + Q * k, scale(a2[k], sc));
    }
}

template <bool SWAP, int L>
__device__ __forceinline__ void run_prog(const InstDesc& in, int prog, int rank, int CL, Cx<float>* sm, int tid) {
    using B = BPlan<SWAP, L>;
    namespace cg = cooperative_groups;
    auto sync = [&]() {
        if (CL > 1) cg::this_cluster().sync(); else __syncthreads();
    };
    const int64_t plane = int64_t(L) * L;
    const int ntile_x = int((plane + B::WS - 1) / B::WS);
    const int ntile_yp = (L + B::WS - 1) / B::WS;          // y tiles per plane
    const int ntile_y = ntile_yp * L;
    const int ntile_z = int((plane + B::WC - 1) / B::WC);   // z rows of the instance
    const float sy = in.sy;
    auto y_stage = [&](auto SIGNc) {
        constexpr int SIGN = decltype(SIGNc)::value;
        for (int tile = rank; tile < ntile_y; tile += CL) {
            const int p = tile / ntile_yp, tc = tile % ntile_yp;
            plane_y_tile<float, B::P, B::Q, B::WS, SIGN, TW_ROW, B::TP, B::TQ>(in.psi + int64_t(p) * plane, L, tc, in.tw,
                                                                              sy, sm, tid, 0);
            __syncthreads();
        }
    };
    if (prog == PROG_ENTER) {
        for (int tile = rank; tile < ntile_z; tile += CL) {
            z_plain_tile<B::P, B::Q, B::WC, -1>(in, tile, sm, tid);
            __syncthreads();
        }
        sync();
        y_stage(ic<-1>{});
        return;
    }
    const Cx<float>* k3 = in.kin + ((prog == PROG_STEP_FULL) ? 3 * L : 0);
    for (int tile = rank; tile < ntile_x; tile += CL) {
        x_kin_tile<B::P, B::Q, B::WS, B::TP, B::TQ>(in, tile, k3, sm, tid);
        __syncthreads();
    }
    sync();
    y_stage(ic<+1>{});
    sync();
    if (prog == PROG_FINISH) {
        for (int tile = rank; tile < ntile_z; tile += CL) {
            z_plain_tile<B::P, B::Q, B::WC, +1>(in, tile, sm, tid);
            __syncthreads();
        }
        return;
    }
    for (int tile = rank; tile < ntile_z; tile += CL) {
        plane_z_tile<float, B::P, B::Q, B::WC>(in.psi, in.ephase, L * L, tile, in.tw, 1.0f / float(L), sm, tid);
        __syncthreads();
    }
    sync();
    y_stage(ic<-1>{});
}

constexpr int kBatchThreads = 256;
// resident blocks per SM the batch kernel is register-budgeted for (build-time tuning knob);
// measured on the 256-instance sweep: 0.580 ms per step at 2, 0.611 ms at 3 (small spills,
// and more instances in flight overflow L2 further)
#ifndef WFS_MINB_BATCH
#define WFS_MINB_BATCH 2
#endif
constexpr size_t kBatchSmem = 24 * 1024;

template <bool SWAP>
__global__ void __launch_bounds__(kBatchThreads, WFS_MINB_BATCH) batch_kernel(const InstDesc* __restrict__ insts,
                                                              const int* __restrict__ order, int prog) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cx<float>* sm = reinterpret_cast<Cx<float>*>(smem_raw);
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int CL = int(cl.num_blocks());
    const int rank = int(cl.block_rank());
    const int id = order[blockIdx.x / CL];
    const InstDesc in = insts[id];
    switch (in.L) {
        case 32: run_prog<SWAP, 32>(in, prog, rank, CL, sm, threadIdx.x); break;
        case 48: run_prog<SWAP, 48>(in, prog, rank, CL, sm, threadIdx.x); break;
        case 64: run_prog<SWAP, 64>(in, prog, rank, CL, sm, threadIdx.x); break;
        case 96: run_prog<SWAP, 96>(in, prog, rank, CL, sm, threadIdx.x); break;
        case 128: run_prog<SWAP, 128>(in, prog, rank, CL, sm, threadIdx.x); break;
        default: break;
    }
}

// ---- two-pass mode ---------------------------------------------------------------------
// x pass: CTA (tile, j) transforms the column tile `tile` of instance ids[j].
template <bool SWAP, int L>
__global__ void __launch_bounds__(kBatchThreads) batch_x_kernel(const InstDesc* __restrict__ insts,
                                                                 const int* __restrict__ ids, int full) {
    using B = BPlan<SWAP, L>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cx<float>* sm = reinterpret_cast<Cx<float>*>(smem_raw);
    const InstDesc in = insts[ids[blockIdx.y]];
    const Cx<float>* k3 = in.kin + (full ? 3 * L : 0);
    x_kin_tile<B::P, B::Q, B::WS, B::TP, B::TQ>(in, int(blockIdx.x), k3, sm, threadIdx.x);
}

// One y tile of a plane held in shared memory (ps, row stride L): the transform of
// plane_y_tile with its loads and stores in shared memory. tw is the axis table (TWL =
// TW_ROW) or, with TW_ROW_SMEM, the plan's row block copied into shared memory.
template <int L, int P, int Q, int W, int SIGN, int TP, int TQ, int TWL = TW_ROW>
__device__ __forceinline__ void smem_y_tile(Cx<float>* ps, int tile, const Cx<float>* tw, float sc, Cx<float>* sm,
                                            int tid) {
    constexpr int T = cmax(P, Q);
    const bool in_block = tid < T * W;
    const int c = tid % W, t = tid / W;
    const int col = tile * W + c;
    const bool active = in_block && col < L;
    Cx<float> a1[Q], a2[P];
    if (t < P) {
#pragma unroll
        for (int i = 0; i < Q; ++i) a1[i] = active ? ps[(t + P * i) * L + col] : mk<float>(0.f, 0.f);
    }
    auto sidx = [&](int k2, int n1) { return (k2 * P + n1) * W + c; };
    const Cx<float>* rows = (TWL == TW_ROW) ? tw_rows<P, Q, TP, TQ>(tw) : tw;
    two_stage<P, Q, SIGN, TWL>(a1, a2, sm, rows, in_block ? t : T, sidx);
    if (active && t < Q) {
#pragma unroll
        for (int k = 0; k < P; ++k) ps[(t + Q * k) * L + col] = scale(a2[k], sc);
    }
}

// W rows of a plane held in shared memory: Fz^-1, times e (from global), Fz, as plane_z_tile.
template <int L, int P, int Q, int W>
__device__ __forceinline__ void smem_z_tile(Cx<float>* ps, const Cx<float>* eplane, int tile, const Cx<float>* tw,
                                            float sc, Cx<float>* sm, int tid) {
    constexpr int T = cmax(P, Q);
    constexpr int RS = cmax(Q * (P + 1), P * (Q + 1));
    const bool in_block = tid < T * W;
    const int t = tid % T, r = tid / T;
    const int row = tile * W + r;
    const bool active = in_block && row < L;
    Cx<float>* rp = ps + row * L;
    const Cx<float>* ep = eplane + int64_t(row) * L;
    Cx<float> a1[Q], a2[P];
    if (t < P) {
#pragma unroll
        for (int i = 0; i < Q; ++i) a1[i] = active ? rp[t + P * i] : mk<float>(0.f, 0.f);
    }
    auto sidx_f = [&](int k2, int n1) { return r * RS + k2 * (P + 1) + n1; };
    auto sidx_i = [&](int k2, int n1) { return r * RS + k2 * (Q + 1) + n1; };
    const int tt = in_block ? t : T;
    two_stage<P, Q, +1, TW_ANGLE>(a1, a2, sm, tw, tt, sidx_f);
    if (tt < Q) {
#pragma unroll
        for (int k = 0; k < P; ++k) {
            Cx<float> e = active ? ld_stream<float>(ep + t + Q * k) : mk<float>(0.f, 0.f);
            a2[k] = cmul(a2[k], scale(e, sc));
        }
    }
    __syncthreads();
    two_stage<Q, P, -1, TW_ANGLE>(a2, a1, sm, tw, tt, sidx_i);
    if (active && t < P) {
#pragma unroll
        for (int i = 0; i < Q; ++i) rp[t + P * i] = a1[i];
    }
}

template <bool SWAP, int L>
struct PlaneSmem {
    using B = BPlan<SWAP, L>;
    static constexpr int RS = cmax(B::Q * (B::P + 1), B::P * (B::Q + 1));
    static constexpr int kTile = cmax(L * B::WS, B::WC * RS);  // transpose buffer (complex)
    // the plane, the transpose buffer, the y plan's twiddle rows and the z angle table
    static constexpr size_t bytes = sizeof(Cx<float>) * (size_t(L) * L + kTile + 2 * L);
};

// plane pass: CTA (x, j) takes yz-plane x of instance ids[j] into shared memory, applies
// Y[Fy^-1] Z[Fz^-1 E Fz] Y[Fy] there and writes it back.
template <bool SWAP, int L>
__global__ void __launch_bounds__(kBatchThreads) batch_plane_kernel(const InstDesc* __restrict__ insts,
                                                                     const int* __restrict__ ids) {
    using B = BPlan<SWAP, L>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cx<float>* ps = reinterpret_cast<Cx<float>*>(smem_raw);
    Cx<float>* sm = ps + L * L;
    Cx<float>* tw_y = sm + PlaneSmem<SWAP, L>::kTile;   // read by every y tile of the plane
    Cx<float>* tw_z = tw_y + L;                         // read by every z tile
    const InstDesc in = insts[ids[blockIdx.y]];
    const int tid = threadIdx.x;
    const int64_t off = int64_t(blockIdx.x) * L * L;
    const float4* g4 = reinterpret_cast<const float4*>(in.psi + off);
    float4* s4 = reinterpret_cast<float4*>(ps);
    for (int i = tid; i < L * L / 2; i += kBatchThreads) s4[i] = __ldcs(g4 + i);
    const Cx<float>* rows = tw_rows<B::P, B::Q, B::TP, B::TQ>(in.tw);
    for (int i = tid; i < L; i += kBatchThreads) {
        tw_y[i] = rows[i];
        tw_z[i] = in.tw[i];
    }
    __syncthreads();
    constexpr int ntile_y = (L + B::WS - 1) / B::WS;
    constexpr int ntile_z = (L + B::WC - 1) / B::WC;
    for (int tile = 0; tile < ntile_y; ++tile) {
        smem_y_tile<L, B::P, B::Q, B::WS, +1, B::TP, B::TQ, TW_ROW_SMEM>(ps, tile, tw_y, in.sy, sm, tid);
        __syncthreads();
    }
    for (int tile = 0; tile < ntile_z; ++tile) {
        smem_z_tile<L, B::P, B::Q, B::WC>(ps, in.ephase + off, tile, tw_z, 1.0f / float(L), sm, tid);
        __syncthreads();
    }
    for (int tile = 0; tile < ntile_y; ++tile) {
        smem_y_tile<L, B::P, B::Q, B::WS, -1, B::TP, B::TQ, TW_ROW_SMEM>(ps, tile, tw_y, in.sy, sm, tid);
        __syncthreads();
    }
    float4* d4 = reinterpret_cast<float4*>(in.psi + off);
    for (int i = tid; i < L * L / 2; i += kBatchThreads) __stcs(d4 + i, s4[i]);
}

bool batch_size_supported(int L) { return L == 32 || L == 48 || L == 64 || L == 96 || L == 128; }

std::map<std::string, std::pair<int, int>> g_tuned;   // size signature -> (cluster, swap)
thread_local std::string g_batch_error;

}  // namespace

struct wfs_batch {
    int ninst;
    std::vector<int> L;
    std::vector<double> extent;
    std::vector<int64_t> off;     // element offset of each instance
    int64_t total;
    int device;
    cudaStream_t stream;
    bool own_stream;
    Cx<float>* psi;
    float2* V;
    Cx<float>* ephase;
    Cx<float>* kin;               // 6 L per instance
    std::vector<int64_t> kin_off;
    Cx<float>* tw;                // two-stage twiddle tables per distinct L
    std::map<int, int64_t> tw_off;
    InstDesc* dinst;
    int* dorder;
    std::vector<std::pair<int, std::pair<int, int>>> classes;  // (L, (offset into dclass, count))
    int* dclass;                  // instance ids grouped by size class
    std::vector<cudaStream_t> side;   // one stream per size class after the first (two-pass mode)
    std::vector<cudaEvent_t> ev;      // fork event, then one join event per side stream
    double kin_dt, kin_mass, e_dt;
    bool e_valid;
    int rep;                      // 0 real, 2 H, 3 pending
    int cluster, swap;
    cudaGraphExec_t graph;
    int graph_steps, graph_first, graph_cluster, graph_swap;
    int64_t graph_launches;
    double* partials;
    size_t partials_cap;
    double* dres;
    int64_t launches;
    std::string err;
    std::string sig;
};

namespace {

int berr(wfs_batch* b, int code, const std::string& m) {
    if (b) b->err = m;
    g_batch_error = m;
    return code;
}
#define BCK(call)                                                                                   \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return berr(b, WFS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

cudaError_t launch_batch(wfs_batch* b, int prog, int cluster, int swap) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(b->ninst * cluster));
    cfg.blockDim = dim3(kBatchThreads);
    cfg.dynamicSmemBytes = kBatchSmem;
    cfg.stream = b->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = unsigned(cluster);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    b->launches += 1;
    if (swap) return cudaLaunchKernelEx(&cfg, batch_kernel<true>, (const InstDesc*)b->dinst, (const int*)b->dorder, prog);
    return cudaLaunchKernelEx(&cfg, batch_kernel<false>, (const InstDesc*)b->dinst, (const int*)b->dorder, prog);
}

template <bool SWAP, int L>
cudaError_t launch_two_pass_class(wfs_batch* b, int full, const int* ids, int count, cudaStream_t st) {
    using B = BPlan<SWAP, L>;
    const int64_t plane = int64_t(L) * L;
    const size_t xs = sizeof(Cx<float>) * size_t(L) * B::WS;
    batch_x_kernel<SWAP, L><<<dim3(unsigned((plane + B::WS - 1) / B::WS), unsigned(count)), kBatchThreads, xs,
                              st>>>((const InstDesc*)b->dinst, ids, full);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    batch_plane_kernel<SWAP, L><<<dim3(unsigned(L), unsigned(count)), kBatchThreads, PlaneSmem<SWAP, L>::bytes,
                                  st>>>((const InstDesc*)b->dinst, ids);
    b->launches += 2;
    return cudaGetLastError();
}

// One step in two-pass mode: x pass and plane pass of every size class. Launched eagerly,
// the largest class runs on the batch's stream and every other class on a side stream
// forked from it and joined back, so the classes share the GPU (0.539 against 0.559 ms
// per step for the 256-instance sweep). In a captured graph the classes stay in one
// stream: replayed as parallel branches the same step took 0.583 ms.
cudaError_t launch_two_pass(wfs_batch* b, int prog, int swap) {
    const int full = prog == PROG_STEP_FULL;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(b->stream, &cap) != cudaSuccess) cap = cudaStreamCaptureStatusNone;
    const bool branches = cap == cudaStreamCaptureStatusNone;
    const size_t nside = (branches && b->classes.size() > 1) ? b->classes.size() - 1 : 0;
    cudaError_t e = cudaSuccess;
    if (nside) {
        e = cudaEventRecord(b->ev[0], b->stream);
        for (size_t k = 0; k < nside && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(b->side[k], b->ev[0], 0);
    }
    for (size_t k = 0; k < b->classes.size() && e == cudaSuccess; ++k) {
        const auto& c = b->classes[k];
        const int* ids = b->dclass + c.second.first;
        const int count = c.second.second;
        cudaStream_t st = (k == 0 || !nside) ? b->stream : b->side[k - 1];
        e = cudaErrorInvalidValue;
#define WFS_BCASE(L_)                                                                                  \
    case L_:                                                                                           \
        e = swap ? launch_two_pass_class<true, L_>(b, full, ids, count, st)                          \
                 : launch_two_pass_class<false, L_>(b, full, ids, count, st);                         \
        break;
        switch (c.first) {
            WFS_BCASE(32) WFS_BCASE(48) WFS_BCASE(64) WFS_BCASE(96) WFS_BCASE(128)
            default: break;
        }
#undef WFS_BCASE
        if (e == cudaSuccess && k > 0 && nside) e = cudaEventRecord(b->ev[k], st);
    }
    for (size_t k = 1; k <= nside && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(b->stream, b->ev[k], 0);
    return e;
}

// One launch of a step program: two-pass mode for the step programs when the cluster
// setting is 0, the cluster kernel otherwise (entering and finishing use 8-CTA clusters).
cudaError_t launch_prog(wfs_batch* b, int prog) {
    if (b->cluster == 0) {
        if (prog == PROG_STEP_HALF || prog == PROG_STEP_FULL) return launch_two_pass(b, prog, b->swap);
        return launch_batch(b, prog, 8, b->swap);
    }
    return launch_batch(b, prog, b->cluster, b->swap);
}

template <bool SWAP, int L>
cudaError_t set_two_pass_attrs() {
    using B = BPlan<SWAP, L>;
    cudaError_t e = cudaFuncSetAttribute(batch_plane_kernel<SWAP, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(PlaneSmem<SWAP, L>::bytes));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(batch_x_kernel<SWAP, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(sizeof(Cx<float>) * L * B::WS));
    return e;
}

int set_kernel_attrs() {
    static PerDevice done;
    const int dev = current_device();
    if (done.get(dev)) return 0;
    for (auto k : {batch_kernel<false>, batch_kernel<true>}) {
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kBatchSmem)) != cudaSuccess) return 1;
        if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) return 1;
    }
    cudaError_t e = cudaSuccess;
#define WFS_BATTR(L_)                                                   \
    if (e == cudaSuccess) e = set_two_pass_attrs<false, L_>();          \
    if (e == cudaSuccess) e = set_two_pass_attrs<true, L_>();
    WFS_BATTR(32) WFS_BATTR(48) WFS_BATTR(64) WFS_BATTR(96) WFS_BATTR(128)
#undef WFS_BATTR
    if (e != cudaSuccess) return 1;
    done.put(dev, 1);
    return 0;
}

int ensure_tables(wfs_batch* b, double dt, double mass) {
    if (!(b->kin_dt == dt && b->kin_mass == mass)) {
        BCK(cudaStreamSynchronize(b->stream));
        std::vector<Cx<float>> h(b->kin_off.back());
        for (int i = 0; i < b->ninst; ++i) {
            const int L = b->L[i];
            const double dx = b->extent[i] / L;
            Cx<float>* p = h.data() + b->kin_off[i];
            // A run of S steps makes S + 1 x passes (S steps and the finishing half step) and
            // S + 1 sets of y/z transforms (S steps, plus the entry and exit transforms), so
            // each x factor carries the inverse gain of one x pass and one y/z set.
            const int n3[3] = {L, L, L};
            double gx = 1.0, gyz = 1.0;
            split_step_gains<float>(n3, &gx, &gyz);
            const double amp = 1.0 / std::sqrt(gx * gyz);
            for (int a = 0; a < 3; ++a) kinetic_axis<float>(L, dx, dt, mass, 0.25, p + a * L, a == 0 ? amp : 1.0);
            for (int a = 0; a < 3; ++a) kinetic_axis<float>(L, dx, dt, mass, 0.5, p + (3 + a) * L, a == 0 ? amp : 1.0);
        }
        BCK(cudaMemcpy(b->kin, h.data(), h.size() * sizeof(Cx<float>), cudaMemcpyHostToDevice));
        b->kin_dt = dt;
        b->kin_mass = mass;
    }
    if (!(b->e_valid && b->e_dt == dt)) {
        BCK(launch_vphase<float>(b->ephase, b->V, dt, b->total, b->stream));
        b->launches += 1;
        b->e_dt = dt;
        b->e_valid = true;
    }
    return WFS_OK;
}

int materialize(wfs_batch* b) {
    if (b->rep == 0) return WFS_OK;
    if (b->rep == 3) {  // pending: X[K/2], then Y^-1, Z^-1 to real space
        BCK(launch_prog(b, PROG_FINISH));
    } else {            // H: ENTER's inverse is not a program of its own; run FINISH with K/2 = identity
        return berr(b, WFS_ERR_STATE, "internal: unexpected representation");
    }
    b->rep = 0;
    return WFS_OK;
}

int run_steps(wfs_batch* b, int nsteps, double dt, double mass, int use_graph) {
    if (nsteps <= 0) return WFS_OK;
    if (b->rep == 3 && !(b->kin_dt == dt && b->kin_mass == mass)) {
        int rc = materialize(b);
        if (rc) return rc;
    }
    int rc = ensure_tables(b, dt, mass);
    if (rc) return rc;
    if (b->rep == 0) {
        BCK(launch_prog(b, PROG_ENTER));
        b->rep = 2;
    }
    const int first = (b->rep == 2) ? PROG_STEP_HALF : PROG_STEP_FULL;
    if (!use_graph) {
        for (int s = 0; s < nsteps; ++s) BCK(launch_prog(b, s == 0 ? first : PROG_STEP_FULL));
    } else {
        if (!(b->graph && b->graph_steps == nsteps && b->graph_first == first && b->graph_cluster == b->cluster &&
              b->graph_swap == b->swap)) {
            if (b->graph) cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
            cudaGraph_t g;
            BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = cudaSuccess;
            const int64_t l0 = b->launches;
            for (int s = 0; s < nsteps && e == cudaSuccess; ++s) e = launch_prog(b, s == 0 ? first : PROG_STEP_FULL);
            const int64_t per_replay = b->launches - l0;
            cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
            if (e != cudaSuccess) return berr(b, WFS_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
            if (e2 != cudaSuccess) return berr(b, WFS_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e2));
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return berr(b, WFS_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
            b->graph_steps = nsteps;
            b->graph_first = first;
            b->graph_cluster = b->cluster;
            b->graph_swap = b->swap;
            b->graph_launches = per_replay;
            b->launches -= per_replay;  // counted again at each replay
        }
        BCK(cudaGraphLaunch(b->graph, b->stream));
        b->launches += b->graph_launches;
    }
    b->rep = 3;
    return WFS_OK;
}

int check_inst(wfs_batch* b, int i) {
    if (!b) return berr(nullptr, WFS_ERR_ARG, "null batch");
    if (i < 0 || i >= b->ninst) return berr(b, WFS_ERR_ARG, "instance index out of range");
    return WFS_OK;
}

}  // namespace

extern "C" {

const char* wfs_batch_last_error(const wfs_batch* b) { return b ? b->err.c_str() : g_batch_error.c_str(); }

int wfs_batch_create(const wfs_batch_desc* d, wfs_batch** out) {
    wfs_batch* b = nullptr;
    if (!d || !out || d->ninst <= 0 || !d->n || !d->extent) return berr(nullptr, WFS_ERR_ARG, "invalid batch descriptor");
    *out = nullptr;
    for (int i = 0; i < d->ninst; ++i) {
        if (!batch_size_supported(d->n[i]))
            return berr(nullptr, WFS_ERR_UNSUPPORTED, "batch instance size " + std::to_string(d->n[i]) + " not in {32,48,64,96,128}");
        if (!(d->extent[i] > 0)) return berr(nullptr, WFS_ERR_ARG, "extent must be positive");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return berr(nullptr, WFS_ERR_CUDA, "no CUDA device available");
    if (cudaSetDevice(d->device) != cudaSuccess) return berr(nullptr, WFS_ERR_CUDA, "cudaSetDevice failed");
    if (set_kernel_attrs()) return berr(nullptr, WFS_ERR_CUDA, "cudaFuncSetAttribute failed");
    b = new wfs_batch();
    b->ninst = d->ninst;
    b->device = d->device;
    b->total = 0;
    b->psi = nullptr; b->V = nullptr; b->ephase = nullptr; b->kin = nullptr; b->tw = nullptr;
    b->dinst = nullptr; b->dorder = nullptr; b->graph = nullptr; b->partials = nullptr; b->dres = nullptr;
    b->dclass = nullptr;
    b->partials_cap = 0;
    b->kin_dt = b->kin_mass = b->e_dt = std::nan("");
    b->e_valid = false;
    b->rep = 0;
    b->cluster = 0;
    b->swap = 0;
    b->graph_steps = 0;
    b->graph_launches = 0;
    b->launches = 0;
    int64_t koff = 0;
    for (int i = 0; i < d->ninst; ++i) {
        b->L.push_back(d->n[i]);
        b->extent.push_back(d->extent[i]);
        b->off.push_back(b->total);
        b->total += int64_t(d->n[i]) * d->n[i] * d->n[i];
        b->kin_off.push_back(koff);
        koff += 6 * d->n[i];
    }
    b->kin_off.push_back(koff);
    std::vector<int> sorted = b->L;
    std::sort(sorted.begin(), sorted.end());
    for (int v : sorted) b->sig += std::to_string(v) + ",";
    auto fail = [&](const std::string& m) {
        wfs_batch_destroy(b);
        return berr(nullptr, WFS_ERR_CUDA, m);
    };
    if (d->stream) {
        b->stream = reinterpret_cast<cudaStream_t>(d->stream);
        b->own_stream = false;
    } else {
        if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return fail("stream");
        b->own_stream = true;
    }
    cudaError_t e = cudaMalloc(&b->psi, b->total * sizeof(Cx<float>));
    if (e == cudaSuccess) e = cudaMalloc(&b->V, b->total * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&b->ephase, b->total * sizeof(Cx<float>));
    if (e == cudaSuccess) e = cudaMalloc(&b->kin, koff * sizeof(Cx<float>));
    if (e == cudaSuccess) e = cudaMalloc(&b->dres, 4096 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->psi, 0, b->total * sizeof(Cx<float>), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->V, 0, b->total * sizeof(float2), b->stream);
    if (e != cudaSuccess) return fail(std::string("allocation: ") + cudaGetErrorString(e));
    // roots per distinct size
    std::vector<Cx<float>> roots;
    for (int v : sorted)
        if (!b->tw_off.count(v)) {
            b->tw_off[v] = int64_t(roots.size());
            roots.resize(roots.size() + 3 * v);
            two_stage_roots<float>(v, roots.data() + b->tw_off[v]);
        }
    e = cudaMalloc(&b->tw, roots.size() * sizeof(Cx<float>));
    if (e == cudaSuccess) e = cudaMemcpy(b->tw, roots.data(), roots.size() * sizeof(Cx<float>), cudaMemcpyHostToDevice);
    std::vector<InstDesc> hd(b->ninst);
    for (int i = 0; i < b->ninst; ++i) {
        hd[i].psi = b->psi + b->off[i];
        hd[i].ephase = b->ephase + b->off[i];
        hd[i].kin = b->kin + b->kin_off[i];
        hd[i].tw = b->tw + b->tw_off[b->L[i]];
        hd[i].L = b->L[i];
        hd[i].sy = float(1.0 / std::sqrt(double(b->L[i])));
    }
    std::vector<int> ord(b->ninst);
    for (int i = 0; i < b->ninst; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return b->L[a] > b->L[c]; });
    if (e == cudaSuccess) e = cudaMalloc(&b->dinst, b->ninst * sizeof(InstDesc));
    if (e == cudaSuccess) e = cudaMalloc(&b->dorder, b->ninst * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(b->dinst, hd.data(), hd.size() * sizeof(InstDesc), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->dorder, ord.data(), ord.size() * sizeof(int), cudaMemcpyHostToDevice);
    // size classes for the two-pass mode, largest first (ord is sorted by size)
    std::vector<int> cls_ids;
    for (int k = 0; k < b->ninst; ++k) {
        const int id = ord[k], L = b->L[id];
        if (b->classes.empty() || b->classes.back().first != L)
            b->classes.push_back({L, {int(cls_ids.size()), 0}});
        cls_ids.push_back(id);
        b->classes.back().second.second += 1;
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->dclass, cls_ids.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(b->dclass, cls_ids.data(), cls_ids.size() * sizeof(int), cudaMemcpyHostToDevice);
    for (size_t k = 0; k < b->classes.size() && e == cudaSuccess; ++k) {
        cudaEvent_t ev = nullptr;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) b->ev.push_back(ev);
        if (e == cudaSuccess && k > 0) {
            cudaStream_t st = nullptr;
            e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
            if (e == cudaSuccess) b->side.push_back(st);
        }
    }
    if (e != cudaSuccess) return fail(std::string("tables: ") + cudaGetErrorString(e));
    auto it = g_tuned.find(b->sig);
    if (it != g_tuned.end()) {
        b->cluster = it->second.first;
        b->swap = it->second.second;
    }
    *out = b;
    return WFS_OK;
}

int wfs_batch_destroy(wfs_batch* b) {
    if (!b) return WFS_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (cudaStream_t st : b->side) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    for (cudaEvent_t ev : b->ev) cudaEventDestroy(ev);
    void* bufs[] = {b->psi, b->V, b->ephase, b->kin, b->tw, b->dinst, b->dorder, b->partials, b->dres, b->dclass};
    for (void* p : bufs)
        if (p) cudaFree(p);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return WFS_OK;
}

int wfs_batch_init_gaussian(wfs_batch* b, int32_t i, const double sigma[3], const double r0[3], const double k0[3]) {
    int rc = check_inst(b, i);
    if (rc) return rc;
    BCK(cudaStreamSynchronize(b->stream));
    int rcm = materialize(b);
    if (rcm) return rcm;
    const int L = b->L[i];
    const int n[3] = {L, L, L};
    const double dxv = b->extent[i] / L;
    const double dx[3] = {dxv, dxv, dxv};
    std::vector<float> g, r;
    gaussian_axes<float>(n, dx, sigma, r0, g, r);
    float* dbuf = nullptr;
    BCK(cudaMalloc(&dbuf, 2 * g.size() * sizeof(float)));
    BCK(cudaMemcpy(dbuf, g.data(), g.size() * sizeof(float), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(dbuf + g.size(), r.data(), r.size() * sizeof(float), cudaMemcpyHostToDevice));
    cudaError_t e = launch_gaussian<float>(b->psi + b->off[i], n, dbuf, dbuf + L, dbuf + 2 * L, dbuf + g.size(),
                                           dbuf + g.size() + L, dbuf + g.size() + 2 * L, float(k0[0]), float(k0[1]),
                                           float(k0[2]), b->stream);
    cudaStreamSynchronize(b->stream);
    cudaFree(dbuf);
    if (e != cudaSuccess) return berr(b, WFS_ERR_CUDA, std::string("gaussian: ") + cudaGetErrorString(e));
    return WFS_OK;
}

int wfs_batch_add_wall(wfs_batch* b, int32_t i, const wfs_wall* w) {
    int rc = check_inst(b, i);
    if (rc) return rc;
    WallDev wd;
    if (!w || !wall_frame(w, wd)) return berr(b, WFS_ERR_ARG, "invalid wall");
    const int L = b->L[i];
    const int n[3] = {L, L, L};
    const float dxv = float(b->extent[i] / L);
    const float dx[3] = {dxv, dxv, dxv};
    BCK(launch_wall(b->V + b->off[i], n, dx, wd, b->stream));
    b->e_valid = false;
    return WFS_OK;
}

int wfs_batch_add_absorbing(wfs_batch* b, int32_t i, const wfs_absorbing* a) {
    int rc = check_inst(b, i);
    if (rc) return rc;
    if (!a) return berr(b, WFS_ERR_ARG, "null absorbing description");
    const int L = b->L[i];
    const int n[3] = {L, L, L};
    const float dxv = float(b->extent[i] / L);
    const float dx[3] = {dxv, dxv, dxv};
    BCK(launch_absorbing(b->V + b->off[i], n, dx, absorbing_dev(a), b->stream));
    b->e_valid = false;
    return WFS_OK;
}

int wfs_batch_set_potential(wfs_batch* b, int32_t i, const void* v, int32_t on_device) {
    int rc = check_inst(b, i);
    if (rc) return rc;
    if (!v) return berr(b, WFS_ERR_ARG, "null potential");
    const int64_t cnt = int64_t(b->L[i]) * b->L[i] * b->L[i];
    BCK(cudaMemcpyAsync(b->V + b->off[i], v, cnt * sizeof(float2), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    b->e_valid = false;
    return WFS_OK;
}

int wfs_batch_set_psi(wfs_batch* b, int32_t i, const void* psi, int32_t on_device) {
    int rc = check_inst(b, i);
    if (rc) return rc;
    if (!psi) return berr(b, WFS_ERR_ARG, "null psi");
    if ((rc = materialize(b))) return rc;
    const int64_t cnt = int64_t(b->L[i]) * b->L[i] * b->L[i];
    BCK(cudaMemcpyAsync(b->psi + b->off[i], psi, cnt * sizeof(float2), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return WFS_OK;
}

int wfs_batch_get_psi(wfs_batch* b, int32_t i, void* psi, int32_t to_device) {
    int rc = check_inst(b, i);
    if (rc) return rc;
    if (!psi) return berr(b, WFS_ERR_ARG, "null output");
    if ((rc = materialize(b))) return rc;
    const int64_t cnt = int64_t(b->L[i]) * b->L[i] * b->L[i];
    BCK(cudaMemcpyAsync(psi, b->psi + b->off[i], cnt * sizeof(float2), to_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return WFS_OK;
}

int wfs_batch_run(wfs_batch* b, int32_t nsteps, double dt, double mass, int32_t use_graph) {
    if (!b) return berr(nullptr, WFS_ERR_ARG, "null batch");
    if (nsteps < 0 || !(mass > 0) || !std::isfinite(dt)) return berr(b, WFS_ERR_ARG, "invalid nsteps, dt or mass");
    return run_steps(b, nsteps, dt, mass, use_graph);
}

int wfs_batch_observe(wfs_batch* b, const wfs_box* boxes, double* prob_out) {
    if (!b) return berr(nullptr, WFS_ERR_ARG, "null batch");
    if (!boxes || !prob_out) return berr(b, WFS_ERR_ARG, "null boxes or output");
    int rc = materialize(b);
    if (rc) return rc;
    const int maxrows = 128 * 128;
    const size_t need = size_t((maxrows + 7) / 8) * 1;
    if (b->partials_cap < need) {
        if (b->partials) cudaFree(b->partials);
        b->partials = nullptr;
        BCK(cudaMalloc(&b->partials, need * sizeof(double)));
        b->partials_cap = need;
    }
    double* dout = nullptr;
    BCK(cudaMalloc(&dout, b->ninst * sizeof(double)));
    for (int i = 0; i < b->ninst; ++i) {
        const int L = b->L[i];
        ObsArgs o;
        std::memset(&o, 0, sizeof(o));
        o.nbox = 1;
        for (int a = 0; a < 3; ++a) {
            if (boxes[i].count[a] < 1 || boxes[i].bottom[a] < 0 || boxes[i].bottom[a] + boxes[i].count[a] > L) {
                cudaFree(dout);
                return berr(b, WFS_ERR_ARG, "observation box outside instance " + std::to_string(i));
            }
            o.box[0].b[a] = boxes[i].bottom[a];
            o.box[0].c[a] = boxes[i].count[a];
            o.n[a] = L;
            o.dx[a] = b->extent[i] / L;
        }
        o.nq = 1;
        o.partials = b->partials;
        int grid = 0;
        cudaError_t e = launch_observe_real<float>(b->psi + b->off[i], o, b->stream, &grid);
        if (e == cudaSuccess) e = launch_reduce_partials(b->partials, grid, 1, dout + i, b->stream);
        b->launches += 2;
        if (e != cudaSuccess) {
            cudaFree(dout);
            return berr(b, WFS_ERR_CUDA, std::string("observe: ") + cudaGetErrorString(e));
        }
    }
    std::vector<double> raw(b->ninst);
    cudaError_t e = cudaMemcpyAsync(raw.data(), dout, b->ninst * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    cudaFree(dout);
    if (e != cudaSuccess) return berr(b, WFS_ERR_CUDA, std::string("observe copy: ") + cudaGetErrorString(e));
    for (int i = 0; i < b->ninst; ++i) {
        const double dxv = b->extent[i] / b->L[i];
        prob_out[i] = raw[i] * dxv * dxv * dxv / 27.0;
    }
    return WFS_OK;
}

int wfs_batch_set_config(wfs_batch* b, int32_t cluster, int32_t swap) {
    if (!b) return berr(nullptr, WFS_ERR_ARG, "null batch");
    if (cluster != 0 && cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8 && cluster != 16)
        return berr(b, WFS_ERR_ARG, "cluster must be 0 (two-pass mode), 1, 2, 4, 8 or 16");
    if (cluster == 0) {
        if (b->rep != 0 && (b->cluster != 0 || b->swap != (swap ? 1 : 0))) {
            int rc = materialize(b);
            if (rc) return rc;
        }
        b->cluster = 0;
        b->swap = swap ? 1 : 0;
        return WFS_OK;
    }
    int ncl = 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(b->ninst * cluster));
    cfg.blockDim = dim3(kBatchThreads);
    cfg.dynamicSmemBytes = kBatchSmem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = unsigned(cluster);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = swap ? cudaOccupancyMaxActiveClusters(&ncl, batch_kernel<true>, &cfg)
                         : cudaOccupancyMaxActiveClusters(&ncl, batch_kernel<false>, &cfg);
    if (e != cudaSuccess || ncl < 1) return berr(b, WFS_ERR_UNSUPPORTED, "cluster size cannot be scheduled on this device");
    if (b->rep != 0 && (b->cluster != cluster || b->swap != (swap ? 1 : 0))) {
        // finish with the configuration that entered, then switch
        int rc = materialize(b);
        if (rc) return rc;
    }
    b->cluster = cluster;
    b->swap = swap ? 1 : 0;
    return WFS_OK;
}

int wfs_batch_autotune(wfs_batch* b, double dt, double mass, int32_t steps, int32_t* cluster_out, int32_t* swap_out,
                       double* ms_out /* [12]: cluster setting {0,1,2,4,8,16} x swap {0,1} */) {
    if (!b) return berr(nullptr, WFS_ERR_ARG, "null batch");
    if (steps < 1) steps = 1;
    std::vector<Cx<float>> saved(b->total);
    int rc = materialize(b);
    if (rc) return rc;
    BCK(cudaStreamSynchronize(b->stream));
    BCK(cudaMemcpy(saved.data(), b->psi, b->total * sizeof(Cx<float>), cudaMemcpyDeviceToHost));
    const int cls[6] = {0, 1, 2, 4, 8, 16};
    double best = 1e30;
    int bc = b->cluster, bs = b->swap;
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    for (int si = 0; si < 2; ++si)
        for (int ci = 0; ci < 6; ++ci) {
            double ms_v = -1.0;
            if (wfs_batch_set_config(b, cls[ci], si) == WFS_OK) {
                rc = run_steps(b, 2, dt, mass, 0);  // warm-up
                if (rc) break;
                BCK(cudaEventRecord(e0, b->stream));
                rc = run_steps(b, steps, dt, mass, 0);
                if (rc) break;
                BCK(cudaEventRecord(e1, b->stream));
                BCK(cudaEventSynchronize(e1));
                float ms = 0.f;
                BCK(cudaEventElapsedTime(&ms, e0, e1));
                ms_v = ms / steps;
                if (ms_v < best) {
                    best = ms_v;
                    bc = cls[ci];
                    bs = si;
                }
                rc = materialize(b);
                if (rc) break;
            }
            if (ms_out) ms_out[si * 6 + ci] = ms_v;
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    BCK(cudaStreamSynchronize(b->stream));  // the last timed configuration may still be running
    BCK(cudaMemcpy(b->psi, saved.data(), b->total * sizeof(Cx<float>), cudaMemcpyHostToDevice));
    b->rep = 0;
    b->cluster = bc;
    b->swap = bs;
    g_tuned[b->sig] = {bc, bs};
    if (cluster_out) *cluster_out = bc;
    if (swap_out) *swap_out = bs;
    return WFS_OK;
}

int wfs_batch_launch_count(wfs_batch* b, int64_t* out) {
    if (!b || !out) return berr(b, WFS_ERR_ARG, "null argument");
    *out = b->launches;
    return WFS_OK;
}

int wfs_batch_synchronize(wfs_batch* b) {
    if (!b) return berr(nullptr, WFS_ERR_ARG, "null batch");
    BCK(cudaStreamSynchronize(b->stream));
    return WFS_OK;
}

}  // extern "C"
