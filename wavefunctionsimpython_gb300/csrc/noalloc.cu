// noalloc.cu — wfs_observe_noalloc: the observable reduction without any allocation.
//
// Who needs this: code that runs where allocating device memory is not
// allowed or not possible — a custom allocator that owns all device memory
// (so cudaMalloc would fight it), a host thread inside a real-time loop that
// must not take the allocator's locks or risk a device-wide synchronisation,
// or a plugin that only receives device pointers from its host application.
// Such callers cannot create an engine handle (wfs_create allocates psi, V
// and scratch), but they can still ask for the Simpson-weighted volume
// probabilities and <r>, <r^2> of a psi they already hold on the device.
//
// The reduction needs scratch for its per-block partial sums. Here it lives in
// one file-scope __device__ array of fixed size (kNoAllocScratchDoubles
// doubles, 1 MiB); every GPU that loads this library keeps it until the
// process exits. Its device address is looked up with cudaGetSymbolAddress
// (host code must not use the symbol's name as an address) on the first call
// made in each CUDA context, i.e. once per device for callers of the runtime
// API, and cached under that context's unique ID; make that first call before
// capturing any stream into a CUDA graph. Because the ID is unique for the
// life of the process, a context created after cudaDeviceReset, or a
// non-primary context the caller made current, gets its own lookup instead of
// a stale address.
//
// All calls on a device share the one array and it keeps what the last call
// left in it. Every slot a call reads is written earlier in the same call
// (per-block sums, then the block-reduced sums), so nothing has to be cleared;
// but two calls whose kernels overlap on the GPU (different streams, no
// ordering between them) race on the array and give wrong results. Order
// them on one stream, or synchronise between them.
#include <mutex>
#include <string>

#include "../../include/wfs.h"
#include "kernels.h"

namespace wfs {

constexpr int kNoAllocScratchDoubles = WFS_NOALLOC_SCRATCH_DOUBLES;
constexpr int kNoAllocRawSlot = kNoAllocScratchDoubles - 16;   // 16 doubles for the block-reduced sums

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

// raw sums -> caller's output: probabilities, then <r>[3] and <r^2>[3] (the location
// sums carry integer offsets from the grid centre; the spacing is applied here)
__global__ void noalloc_finish_kernel(const double* __restrict__ raw, int nbox, int has_loc, double dv, double dx,
                                      double dy, double dz, double* __restrict__ out) {
    const int i = threadIdx.x;
    if (i < nbox) out[i] = raw[i] * dv;
    if (has_loc && i < 3) {
        const double d = i == 0 ? dx : (i == 1 ? dy : dz);
        out[nbox + i] = raw[nbox + 1 + i] * d * dv;
        out[nbox + 3 + i] = raw[nbox + 4 + i] * (d * d) * dv;
    }
}

namespace {

// Scratch addresses by CUDA context: cuCtxGetCurrent and cuCtxGetId reached through the
// runtime's driver entry points (no link-time libcuda dependency).
using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);
template <typename F>
F driver_fn(const char* name, int version) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, version, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
        p = nullptr;
    return reinterpret_cast<F>(p);
}

struct ScratchSlot {
    unsigned long long ctx_id;
    double* ptr;
};
constexpr int kScratchSlots = 64;
std::mutex g_noalloc_mutex;
ScratchSlot g_noalloc_slot[kScratchSlots] = {};
int g_noalloc_next = 0;

// The current context's unique ID; 0 when it cannot be read (then nothing is cached).
unsigned long long current_context_id() {
    static const CtxGetCurrentFn get_current = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent", 4000);
    static const CtxGetIdFn get_id = driver_fn<CtxGetIdFn>("cuCtxGetId", 12000);
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

}  // namespace

void record_global_error(const std::string& m);  // engine.cu: read back with wfs_global_error()

namespace {
int fail(int code, const std::string& m) {
    record_global_error(m);
    return code;
}
}  // namespace
}  // namespace wfs

using namespace wfs;

extern "C" int wfs_observe_noalloc(const void* psi_device, int32_t dtype, const int32_t n[3], const double extent[3],
                                   const wfs_box* boxes, int32_t nbox, const wfs_box* loc, double* out_device,
                                   void* stream) {
    if (!psi_device || !n || !extent || !out_device) return fail(WFS_ERR_ARG, "null argument");
    if (dtype != WFS_C64 && dtype != WFS_C128) return fail(WFS_ERR_ARG, "dtype must be WFS_C64 or WFS_C128");
    if (nbox < 0 || nbox > kMaxBox) return fail(WFS_ERR_ARG, "nbox must be in [0, 8]");
    if (nbox > 0 && !boxes) return fail(WFS_ERR_ARG, "boxes is null");
    if (nbox == 0 && !loc) return fail(WFS_ERR_ARG, "nothing to observe");
    ObsArgs o;
    memset(&o, 0, sizeof(o));
    for (int a = 0; a < 3; ++a) {
        if (n[a] < 1 || !(extent[a] > 0)) return fail(WFS_ERR_ARG, "invalid grid");
        o.n[a] = n[a];
        o.dx[a] = extent[a] / n[a];
    }
    auto cp = [&](const wfs_box& b, ObsBox& d) -> bool {
        for (int a = 0; a < 3; ++a) {
            if (b.count[a] < 1 || b.bottom[a] < 0 || b.bottom[a] + b.count[a] > n[a]) return false;
            d.b[a] = b.bottom[a];
            d.c[a] = b.count[a];
        }
        return true;
    };
    o.nbox = nbox;
    for (int b = 0; b < nbox; ++b)
        if (!cp(boxes[b], o.box[b])) return fail(WFS_ERR_ARG, "observation box outside the grid");
    o.has_loc = loc ? 1 : 0;
    if (loc && !cp(*loc, o.loc)) return fail(WFS_ERR_ARG, "location box outside the grid");
    o.nq = nbox + (loc ? kLocQ : 0);
    // the reduction (launch_observe_real) uses one block per kObsRowsPerCta (x, y) rows and
    // nq partial sums per block
    const int64_t rows = int64_t(n[0]) * n[1];
    const int64_t blocks = (rows + kObsRowsPerCta - 1) / kObsRowsPerCta;
    if (blocks * o.nq > kNoAllocRawSlot)
        return fail(WFS_ERR_UNSUPPORTED,
                    "grid too large for the fixed scratch: ceil(nx*ny/" + std::to_string(kObsRowsPerCta) +
                        ") * (quantities) must be <= " + std::to_string(kNoAllocRawSlot) + ", got " +
                        std::to_string(blocks * o.nq));
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(WFS_ERR_CUDA, "no current CUDA device");
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mutex);
        const unsigned long long id = current_context_id();
        for (int i = 0; id && i < kScratchSlots && !scratch; ++i)
            if (g_noalloc_slot[i].ctx_id == id) scratch = g_noalloc_slot[i].ptr;
        if (!scratch) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p)
                return fail(WFS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            scratch = static_cast<double*>(p);
            if (id) {
                g_noalloc_slot[g_noalloc_next] = {id, scratch};
                g_noalloc_next = (g_noalloc_next + 1) % kScratchSlots;
            }
        }
    }
    o.partials = scratch;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int grid = 0;
    cudaError_t e = cudaSuccess;
    if (blocks > INT32_MAX) return fail(WFS_ERR_UNSUPPORTED, "grid too large");
    e = (dtype == WFS_C64)
                        ? launch_observe_real<float>(reinterpret_cast<const Cx<float>*>(psi_device), o, s, &grid)
                        : launch_observe_real<double>(reinterpret_cast<const Cx<double>*>(psi_device), o, s, &grid);
    if (e == cudaSuccess) e = launch_reduce_partials(scratch, grid, o.nq, scratch + kNoAllocRawSlot, s);
    if (e == cudaSuccess) {
        const double dv = o.dx[0] * o.dx[1] * o.dx[2] / 27.0;
        noalloc_finish_kernel<<<1, 32, 0, s>>>(scratch + kNoAllocRawSlot, nbox, o.has_loc, dv, o.dx[0], o.dx[1], o.dx[2],
                                               out_device);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return fail(WFS_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return WFS_OK;
}
