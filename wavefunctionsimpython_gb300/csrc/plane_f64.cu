// plane_f64.cu — complex128 instantiations of the fused yz-plane pass.
#include "plane_kernels.cuh"

namespace wfs {

template <>
cudaError_t launch_plane<double>(int ny, int nz, const PlaneArgs<double>& a, int64_t nplanes, cudaStream_t s) {
    return dispatch_plane<double>(ny, nz, a, nplanes, s);
}

}  // namespace wfs
