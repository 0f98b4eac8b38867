// plane_f32.cu — complex64 instantiations of the fused yz-plane pass.
#include "plane_kernels.cuh"

namespace wfs {

template <>
cudaError_t launch_plane<float>(int ny, int nz, const PlaneArgs<float>& a, int64_t nplanes, cudaStream_t s) {
    return dispatch_plane<float>(ny, nz, a, nplanes, s);
}

bool plane_pass_supported(int ny, int nz) { return plane_supported(ny, nz); }

}  // namespace wfs
