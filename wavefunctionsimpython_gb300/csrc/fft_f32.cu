// fft_f32.cu — complex64 instantiations of the pencil FFT passes.
#include "fft_kernels.cuh"

namespace wfs {

template <>
cudaError_t launch_fft_strided<float>(int L, int op, const PassArgs<float>& a, int64_t outer_count, cudaStream_t s) {
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
