// drr_launch.cuh -- launcher template for the forward kernel; each drr_inst_nv*.cu instantiates it
// for one volume count and every material bucket, so the instantiations compile in parallel.
#pragma once

#include "drr_forward.cuh"

namespace drr {

template <int NV, int M>
cudaError_t launch_forward(const ForwardParams<NV> &p, cudaStream_t stream) {
    dim3 grid((p.width + kTileW - 1) / kTileW, (p.height + kTileH - 1) / kTileH, p.n_views);
    forward_kernel<NV, M><<<grid, kBlockThreads, 0, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace drr

#define DRR_INSTANTIATE_FORWARD(NV)                                                             \
    namespace drr {                                                                             \
    template cudaError_t launch_forward<NV, 2>(const ForwardParams<NV> &, cudaStream_t);        \
    template cudaError_t launch_forward<NV, 3>(const ForwardParams<NV> &, cudaStream_t);        \
    template cudaError_t launch_forward<NV, 4>(const ForwardParams<NV> &, cudaStream_t);        \
    template cudaError_t launch_forward<NV, 6>(const ForwardParams<NV> &, cudaStream_t);        \
    template cudaError_t launch_forward<NV, 8>(const ForwardParams<NV> &, cudaStream_t);        \
    template cudaError_t launch_forward<NV, 16>(const ForwardParams<NV> &, cudaStream_t);       \
    }
