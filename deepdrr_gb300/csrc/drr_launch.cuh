// drr_launch.cuh -- launcher templates for the forward kernels; each drr_inst_nv*.cu instantiates
// them for one volume count and every material bucket, so the instantiations compile in parallel.
#pragma once

#include "drr_forward.cuh"

namespace drr {

template <int NV, int M>
cudaError_t launch_forward(const ForwardParams<NV> &p, cudaStream_t stream) {
    dim3 grid((p.s.width + kTileW - 1) / kTileW, (p.s.height + kTileH - 1) / kTileH, p.n_views);
    forward_kernel<NV, M><<<grid, kBlockThreads, 0, stream>>>(p);
    return cudaGetLastError();
}

template <int NV, int M>
cudaError_t launch_persistent(const PersistentParams<NV> &p, int grid_blocks, cudaStream_t stream) {
    forward_persistent_kernel<NV, M><<<grid_blocks, kBlockThreads, 0, stream>>>(p);
    return cudaGetLastError();
}

// Resident blocks per SM of the persistent kernel (0 on error).
template <int NV, int M>
int persistent_occupancy() {
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, forward_persistent_kernel<NV, M>, kBlockThreads, 0) !=
        cudaSuccess)
        return 0;
    return blocks;
}

}  // namespace drr

#define DRR_INSTANTIATE_ONE(NV, M)                                                                  \
    template cudaError_t launch_forward<NV, M>(const ForwardParams<NV> &, cudaStream_t);            \
    template cudaError_t launch_persistent<NV, M>(const PersistentParams<NV> &, int, cudaStream_t); \
    template int persistent_occupancy<NV, M>();

#define DRR_INSTANTIATE_FORWARD(NV) \
    namespace drr {                 \
    DRR_INSTANTIATE_ONE(NV, 2)      \
    DRR_INSTANTIATE_ONE(NV, 3)      \
    DRR_INSTANTIATE_ONE(NV, 4)      \
    DRR_INSTANTIATE_ONE(NV, 6)      \
    DRR_INSTANTIATE_ONE(NV, 8)      \
    DRR_INSTANTIATE_ONE(NV, 16)     \
    }
