// fft_f64.cu — complex128 instantiations of the pencil FFT passes.
#include "fft_kernels.cuh"

namespace wfs {

template <>
cudaError_t launch_fft_strided<double>(int L, int op, const PassArgs<double>& a, int64_t outer_count, cudaStream_t s) {
    return dispatch_strided<double>(L, op, a, outer_count, s);
}
template <>
cudaError_t launch_fft_contig<double>(int L, int op, const PassArgs<double>& a, cudaStream_t s, int* grid_out) {
    return dispatch_contig<double>(L, op, a, s, grid_out);
}

}  // namespace wfs
