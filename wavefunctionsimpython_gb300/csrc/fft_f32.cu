// fft_f32.cu — complex64 instantiations of the pencil FFT passes.
#include <cudaTypedefs.h>

#include <cstdlib>
#include <cstring>
#include <mutex>

#include "fft_kernels.cuh"

namespace wfs {

namespace {

static_assert(sizeof(CUtensorMap) == sizeof(TensorMapImage), "tensor map image size");

// cuTensorMapEncodeTiled of the driver the runtime loaded (no link-time libcuda dependency).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// Encoded tensor maps of recent launches. A map describes psi's address, shape and
// strides; the split step launches the x pass on the same psi every step, so the
// encoding (a host call of a few microseconds) is done once per array instead of
// once per launch. Keyed by device, address, shape, strides and tile width.
struct MapKey {
    int dev;
    const void* data;
    int64_t ncols, rows, outer, row_stride, outer_stride;
    int width;
    bool operator==(const MapKey& o) const {
        return dev == o.dev && data == o.data && ncols == o.ncols && rows == o.rows && outer == o.outer &&
               row_stride == o.row_stride && outer_stride == o.outer_stride && width == o.width;
    }
};
struct MapCache {
    static constexpr int kSlots = 8;
    std::mutex mu;
    MapKey key[kSlots];
    CUtensorMap map[kSlots];
    bool used[kSlots] = {};
    int next = 0;
};
MapCache g_maps;

bool cached_map(const MapKey& k, CUtensorMap* out) {
    std::lock_guard<std::mutex> lk(g_maps.mu);
    for (int i = 0; i < MapCache::kSlots; ++i)
        if (g_maps.used[i] && g_maps.key[i] == k) {
            *out = g_maps.map[i];
            return true;
        }
    return false;
}

void store_map(const MapKey& k, const CUtensorMap& m) {
    std::lock_guard<std::mutex> lk(g_maps.mu);
    const int i = g_maps.next;
    g_maps.key[i] = k;
    g_maps.map[i] = m;
    g_maps.used[i] = true;
    g_maps.next = (i + 1) % MapCache::kSlots;
}

// The copy-staged strided pass is the default where it applies; WFS_STRIDED_STAGED=0 in the
// environment selects the cp.async pipelined pass (for A/B timing).
bool staged_enabled() {
    static const int on = [] {
        const char* e = getenv("WFS_STRIDED_STAGED");
        return (e && e[0] == '0') ? 0 : 1;
    }();
    return on != 0;
}

template <int L, int OP>
cudaError_t run_strided_staged(const PassArgs<float>& a0, int64_t outer_count, cudaStream_t s, bool* used) {
    constexpr int P = PlanOf<L>::P, Q = PlanOf<L>::Q, T = cmax(P, Q);
    constexpr int W = StridedW<float, T>::value;
    *used = false;
    if constexpr (L > 256 || 2 * size_t(L) * W * sizeof(Cx<float>) > 112 * 1024) {
        return cudaSuccess;
    } else {
        const int64_t tiles = (a0.ncols + W - 1) / W;
        if (outer_count * tiles <= int64_t(2) * device_sm_count()) return cudaSuccess;  // too few items to pipeline
        auto encode = tensor_map_encoder();
        if (!encode) return cudaSuccess;
        StridedStagedArgs sa;
        std::memset(&sa, 0, sizeof(sa));
        sa.p = a0;
        sa.p.tiles = int32_t(tiles);
        // psi as a 3D array of 8-byte elements: x = column, y = pencil row, z = outer slab
        const int64_t zs = outer_count > 1 ? a0.outer_stride : int64_t(L) * a0.row_stride;
        const cuuint64_t dims[3] = {cuuint64_t(a0.ncols), cuuint64_t(L), cuuint64_t(outer_count)};
        const cuuint64_t strides[2] = {cuuint64_t(a0.row_stride) * sizeof(Cx<float>), cuuint64_t(zs) * sizeof(Cx<float>)};
        const cuuint32_t box[3] = {cuuint32_t(W), cuuint32_t(L), 1};
        const cuuint32_t estr[3] = {1, 1, 1};
        if ((strides[0] % 16) || (strides[1] % 16) || a0.row_stride < a0.ncols || zs < int64_t(L) * a0.row_stride)
            return cudaSuccess;
        const int dev = current_device();
        const MapKey key{dev, a0.data, int64_t(a0.ncols), int64_t(L), outer_count, int64_t(a0.row_stride), zs, W};
        CUtensorMap map;
        if (!cached_map(key, &map)) {
            if (encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, a0.data, dims, strides, box, estr,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                return cudaSuccess;
            store_map(key, map);
        }
        std::memcpy(&sa.map, &map, sizeof(map));
        // staging slots, two mbarriers, twiddle rows of both plans and the kinetic x factors
        const size_t smem = 128 + 2 * size_t(L) * W * sizeof(Cx<float>) + 2 * sizeof(uint64_t) +
                            3 * size_t(L) * sizeof(Cx<float>);
        auto kern = fft_strided_staged_kernel<P, Q, W, OP>;
        static PerDevice occupancy;
        int blocks_per_sm = occupancy.get(dev);
        if (blocks_per_sm == 0) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if (e == cudaSuccess)  // WFS_MINB_STAGED blocks of two L x W tiles each need the largest carveout
                e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         int(cudaSharedmemCarveoutMaxShared));
            if (e != cudaSuccess) return e;
            int nb = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, T * W, smem);
            if (e != cudaSuccess) return e;
            blocks_per_sm = nb > 0 ? nb : 1;
            occupancy.put(dev, blocks_per_sm);
        }
        const int64_t nitems = outer_count * tiles;
        const int64_t cap = int64_t(blocks_per_sm) * device_sm_count();
        const int64_t grid = nitems < cap ? nitems : cap;
        kern<<<dim3(unsigned(grid)), dim3(T * W), smem, s>>>(sa, nitems);
        *used = true;
        return cudaGetLastError();
    }
}

}  // namespace

template <>
cudaError_t launch_fft_strided<float>(int L, int op, const PassArgs<float>& a, int64_t outer_count, cudaStream_t s) {
    if (staged_enabled()) {
        bool used = false;
        cudaError_t e = cudaSuccess;
#define WFS_CASE(L_)                                                                                        \
    case L_:                                                                                                \
        e = op == OP_KIN ? run_strided_staged<L_, OP_KIN>(a, outer_count, s, &used)                         \
                         : run_strided_staged<L_, OP_PLAIN>(a, outer_count, s, &used);                      \
        break;
        switch (L) {
            WFS_FOR_EACH_L(WFS_CASE)
            default:
                break;
        }
#undef WFS_CASE
        if (e != cudaSuccess || used) return e;
    }
    return dispatch_strided<float>(L, op, a, outer_count, s);
}
template <>
cudaError_t launch_fft_contig<float>(int L, int op, const PassArgs<float>& a, cudaStream_t s, int* grid_out) {
    return dispatch_contig<float>(L, op, a, s, grid_out);
}

bool fft_length_supported(int L, bool dbl) {
    switch (L) {
        case 2: case 3: case 4: case 6: case 8: case 12: case 16: case 24: case 32: case 48: case 64:
        case 96: case 128: case 192: case 256: case 384: case 512: case 768: case 1024:
            return true;
        default:
            return false;
    }
    (void)dbl;
}

#define WFS_ROWS(L_) case L_: return dbl ? ContigW<double, cmax(PlanOf<L_>::P, PlanOf<L_>::Q)>::value : ContigW<float, cmax(PlanOf<L_>::P, PlanOf<L_>::Q)>::value;
int fft_contig_rows_per_cta(int L, bool dbl) {
    switch (L) {
        WFS_FOR_EACH_L(WFS_ROWS)
        default:
            return 0;
    }
}
#undef WFS_ROWS
#define WFS_COLS(L_) case L_: return dbl ? StridedW<double, cmax(PlanOf<L_>::P, PlanOf<L_>::Q)>::value : StridedW<float, cmax(PlanOf<L_>::P, PlanOf<L_>::Q)>::value;
int fft_strided_cols_per_cta(int L, bool dbl) {
    switch (L) {
        WFS_FOR_EACH_L(WFS_COLS)
        default:
            return 0;
    }
}
#undef WFS_COLS

}  // namespace wfs
