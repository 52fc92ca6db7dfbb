// drr_adjoint.cu -- instantiations of the adjoint kernel (drr_adjoint.cuh), one per material bucket.
#include "drr_adjoint.cuh"

namespace drr {

template <int M>
cudaError_t launch_adjoint(const AdjointParams &p, cudaStream_t stream) {
    const dim3 grid((p.s.width + kTileW - 1) / kTileW, (p.s.height + kTileH - 1) / kTileH, p.n_views);
    adjoint_kernel<M><<<grid, kBlockThreads, 0, stream>>>(p);
    return cudaGetLastError();
}

template cudaError_t launch_adjoint<2>(const AdjointParams &, cudaStream_t);
template cudaError_t launch_adjoint<3>(const AdjointParams &, cudaStream_t);
template cudaError_t launch_adjoint<4>(const AdjointParams &, cudaStream_t);
template cudaError_t launch_adjoint<6>(const AdjointParams &, cudaStream_t);
template cudaError_t launch_adjoint<8>(const AdjointParams &, cudaStream_t);
template cudaError_t launch_adjoint<16>(const AdjointParams &, cudaStream_t);

}  // namespace drr
