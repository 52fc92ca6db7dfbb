// drr_measure.cu -- the texture unit's filtered-fetch rate, the ceiling of the forward march.
//
// Every sample of the forward kernel costs one trilinear-filtered tex3D fetch of the density
// (project_kernel.cu:550 does the same fetch); the kernel's other work is ALU and one 32-bit label
// load per sample. drr_texture_rate measures how many such fetches per second this GPU's texture
// units return when nothing else limits them: a 16^3 texture (16 KB float32, 8 KB float16) that
// stays in L1, the forward kernel's launch shape (128-thread blocks, 8 per SM), and a loop of two
// instructions per fetch (the fetch and one add that keeps its result live). Twelve fixed
// coordinates per thread, distinct across threads and away from texel centres, cycle through the
// loop, so every fetch blends eight texels.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "drr_internal.h"

namespace {

constexpr int kEdge = 16;
constexpr int kThreads = 128;
constexpr int kBlocksPerSm = 8;
constexpr int kCoords = 12;
constexpr int kRounds = 384;  // rounds of kCoords fetches per thread and launch

__global__ void __launch_bounds__(kThreads, kBlocksPerSm) texture_rate_kernel(cudaTextureObject_t tex, float *out) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    float x[kCoords], y[kCoords], z[kCoords];
#pragma unroll
    for (int k = 0; k < kCoords; k++) {
        // in [1.6, 14.4] on each axis: interior, fractional parts spread over (0, 1)
        x[k] = 1.6f + (float)((tid * 7 + k * 5) % 61) * 0.21f;
        y[k] = 1.6f + (float)((tid * 3 + k * 11) % 59) * 0.217f;
        z[k] = 1.6f + (float)((tid + k * 13) % 53) * 0.2415f;
    }
    float acc0 = 0.0f, acc1 = 0.0f;
    for (int r = 0; r < kRounds; r++) {
#pragma unroll
        for (int k = 0; k < kCoords; k += 2) {
            acc0 += tex3D<float>(tex, x[k], y[k], z[k]);
            acc1 += tex3D<float>(tex, x[k + 1], y[k + 1], z[k + 1]);
        }
    }
    out[tid] = acc0 + acc1;
}

}  // namespace

extern "C" drr_status drr_texture_rate(int32_t density_type, void *stream, double *fetches_per_second) {
    drr::set_last_error("");
    if (!fetches_per_second) return drr::fail(DRR_ERR_INVALID_ARGUMENT, "drr_texture_rate: NULL output");
    if (density_type != DRR_DENSITY_F32 && density_type != DRR_DENSITY_F16)
        return drr::fail(DRR_ERR_UNSUPPORTED, "drr_texture_rate: float32 or float16 textures only");
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return drr::cuda_fail(e, "drr_texture_rate: device query");
    const bool half = density_type == DRR_DENSITY_F16;
    const size_t n = (size_t)kEdge * kEdge * kEdge;
    std::vector<float> f32(n);
    std::vector<__half> f16(n);
    for (size_t i = 0; i < n; i++) {
        f32[i] = 0.25f + (float)((i * 2654435761u) % 1000u) * 1e-3f;
        f16[i] = __float2half_rn(f32[i]);
    }
    cudaChannelFormatDesc fd = cudaCreateChannelDesc(half ? 16 : 32, 0, 0, 0, cudaChannelFormatKindFloat);
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    float *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const int blocks = sms * kBlocksPerSm;
    double best = 0.0;
    e = cudaMalloc3DArray(&arr, &fd, make_cudaExtent(kEdge, kEdge, kEdge), 0);
    if (e == cudaSuccess) {
        cudaMemcpy3DParms cp;
        std::memset(&cp, 0, sizeof(cp));
        cp.srcPtr = make_cudaPitchedPtr(half ? (void *)f16.data() : (void *)f32.data(),
                                        (size_t)kEdge * (half ? 2 : 4), kEdge, kEdge);
        cp.dstArray = arr;
        cp.extent = make_cudaExtent(kEdge, kEdge, kEdge);
        cp.kind = cudaMemcpyHostToDevice;
        e = cudaMemcpy3D(&cp);
    }
    if (e == cudaSuccess) {
        cudaResourceDesc rd;
        std::memset(&rd, 0, sizeof(rd));
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
        cudaTextureDesc td;
        std::memset(&td, 0, sizeof(td));
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModeLinear;
        td.readMode = cudaReadModeElementType;
        e = cudaCreateTextureObject(&tex, &rd, &td, nullptr);
    }
    if (e == cudaSuccess) e = cudaMalloc(&out, sizeof(float) * (size_t)blocks * kThreads);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        texture_rate_kernel<<<blocks, kThreads, 0, s>>>(tex, out);  // warm-up
        e = cudaGetLastError();
    }
    const double fetches = (double)blocks * kThreads * kRounds * kCoords;
    for (int rep = 0; rep < 5 && e == cudaSuccess; rep++) {
        cudaEventRecord(e0, s);
        texture_rate_kernel<<<blocks, kThreads, 0, s>>>(tex, out);
        cudaEventRecord(e1, s);
        e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && ms > 0.0f && fetches / (ms * 1e-3) > best) best = fetches / (ms * 1e-3);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (out) cudaFree(out);
    if (tex) cudaDestroyTextureObject(tex);
    if (arr) cudaFreeArray(arr);
    if (e != cudaSuccess) return drr::cuda_fail(e, "drr_texture_rate");
    *fetches_per_second = best;
    return DRR_OK;
}
