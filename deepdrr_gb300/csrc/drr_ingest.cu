// drr_ingest.cu -- volume ingest on the GPU: Hounsfield units -> densities and material labels.
//
// Replaces the host-side numpy work of Volume.from_hu (deepdrr/vol/volume.py:281-302): the density
// conversion _convert_hounsfield_to_density (volume.py:339-351) and the threshold segmentation
// conv_hu_to_materials_thresholding (deepdrr/load_dicom.py:132-143), followed by the layout change
// of Projector.initialize (np.moveaxis to i-fastest, projector.py:1469). One pass reads the HU
// volume in the reference's [i][j][k] order (k fastest) and writes densities and labels in the
// texture layout [k][j][i] (i fastest) through a 32 x 32 shared-memory tile per (i, k) block of one
// j plane, so both the reads and the writes are coalesced.
//
// Arithmetic follows numpy's: float32 HU stay float32 (0.001029 * hu rounds, + 1.030 rounds; the
// constants are the float32 roundings of the literals); int16 and float64 HU are converted in
// float64 and rounded to float32 at the end, as Volume casts them. NaN HU give NaN densities.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/drr_gb300.h"
#include "drr_internal.h"

using drr::cuda_fail;
using drr::fail;

namespace {

constexpr int kTile = 32;
constexpr int kRows = 8;

__device__ __forceinline__ float density_f32(float h) {
    const float a = __fadd_rn(__fmul_rn(0.001029f, h), 1.030f);
    const float b = __fadd_rn(__fmul_rn(0.0005886f, h), 1.03f);
    if (h != h) return h;
    return fmaxf(fminf(a, b), 0.0f);
}

__device__ __forceinline__ float density_f64(double h) {
    const double a = __dadd_rn(__dmul_rn(0.001029, h), 1.030);
    const double b = __dadd_rn(__dmul_rn(0.0005886, h), 1.03);
    if (h != h) return (float)h;
    return (float)fmax(fmin(a, b), 0.0);
}

template <typename HU>
__device__ __forceinline__ float to_density(HU h);
template <>
__device__ __forceinline__ float to_density<float>(float h) { return density_f32(h); }
template <>
__device__ __forceinline__ float to_density<int16_t>(int16_t h) { return density_f64((double)h); }
template <>
__device__ __forceinline__ float to_density<double>(double h) { return density_f64(h); }

// load_dicom.py:132-143: air HU <= -800, soft tissue -800 < HU <= 350, bone HU > 350. A NaN HU is
// in no mask and keeps _format_materials' initial id 0, which is air's (the first mask).
template <typename HU>
__device__ __forceinline__ uint8_t to_label(HU h, uint8_t air, uint8_t soft, uint8_t bone) {
    const double x = (double)h;
    if (x > 350.0) return bone;
    if (x > -800.0) return soft;
    return air;
}

template <typename OUT>
__device__ __forceinline__ OUT store_density(float d);
template <>
__device__ __forceinline__ float store_density<float>(float d) { return d; }
template <>
__device__ __forceinline__ __half store_density<__half>(float d) { return __float2half_rn(d); }
template <>
__device__ __forceinline__ __nv_bfloat16 store_density<__nv_bfloat16>(float d) { return __float2bfloat16_rn(d); }

template <typename HU, typename OUT>
__global__ void __launch_bounds__(kTile *kRows)
    ingest_hu_kernel(const HU *__restrict__ hu, int ni, int nj, int nk, uint8_t air, uint8_t soft, uint8_t bone,
                     OUT *__restrict__ density, uint8_t *__restrict__ labels) {
    __shared__ float s_d[kTile][kTile + 1];
    __shared__ uint8_t s_l[kTile][kTile + 4];
    const int k0 = blockIdx.x * kTile, i0 = blockIdx.y * kTile, j = blockIdx.z;
    // read hu[i][j][k]: threads along k
#pragma unroll
    for (int r = 0; r < kTile; r += kRows) {
        const int i = i0 + threadIdx.y + r, k = k0 + threadIdx.x;
        if (i < ni && k < nk) {
            const HU h = hu[((size_t)i * nj + j) * nk + k];
            s_d[threadIdx.y + r][threadIdx.x] = to_density<HU>(h);
            s_l[threadIdx.y + r][threadIdx.x] = to_label<HU>(h, air, soft, bone);
        }
    }
    __syncthreads();
    // write [k][j][i]: threads along i
#pragma unroll
    for (int r = 0; r < kTile; r += kRows) {
        const int k = k0 + threadIdx.y + r, i = i0 + threadIdx.x;
        if (i < ni && k < nk) {
            const size_t o = ((size_t)k * nj + j) * ni + i;
            density[o] = store_density<OUT>(s_d[threadIdx.x][threadIdx.y + r]);
            labels[o] = s_l[threadIdx.x][threadIdx.y + r];
        }
    }
}

template <typename HU>
cudaError_t launch_ingest(const void *hu, int ni, int nj, int nk, const uint8_t cls[3], void *density,
                          int32_t density_type, uint8_t *labels, cudaStream_t s) {
    const dim3 grid((nk + kTile - 1) / kTile, (ni + kTile - 1) / kTile, nj), block(kTile, kRows);
    const HU *h = (const HU *)hu;
    switch (density_type) {
        case DRR_DENSITY_F16:
            ingest_hu_kernel<HU, __half><<<grid, block, 0, s>>>(h, ni, nj, nk, cls[0], cls[1], cls[2], (__half *)density,
                                                               labels);
            break;
        case DRR_DENSITY_BF16:
            ingest_hu_kernel<HU, __nv_bfloat16><<<grid, block, 0, s>>>(h, ni, nj, nk, cls[0], cls[1], cls[2],
                                                                      (__nv_bfloat16 *)density, labels);
            break;
        default:
            ingest_hu_kernel<HU, float><<<grid, block, 0, s>>>(h, ni, nj, nk, cls[0], cls[1], cls[2], (float *)density,
                                                              labels);
    }
    return cudaGetLastError();
}

}  // namespace

extern "C" drr_status drr_ingest_hu(const void *hu, int32_t hu_type, int32_t ni, int32_t nj, int32_t nk,
                                    const uint8_t class_labels[3], void *density, int32_t density_type,
                                    uint8_t *labels, void *stream) {
    drr::set_last_error("");
    if (!hu || !class_labels || !density || !labels) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_ingest_hu: NULL pointer");
    if (ni < 1 || nj < 1 || nk < 1) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_ingest_hu: empty volume");
    if (nj > 65535) return fail(DRR_ERR_UNSUPPORTED, "drr_ingest_hu: nj above 65535");
    if (density_type != DRR_DENSITY_F32 && density_type != DRR_DENSITY_F16 && density_type != DRR_DENSITY_BF16)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_ingest_hu: unknown density type");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    switch (hu_type) {
        case DRR_HU_F32: e = launch_ingest<float>(hu, ni, nj, nk, class_labels, density, density_type, labels, s); break;
        case DRR_HU_I16: e = launch_ingest<int16_t>(hu, ni, nj, nk, class_labels, density, density_type, labels, s); break;
        case DRR_HU_F64: e = launch_ingest<double>(hu, ni, nj, nk, class_labels, density, density_type, labels, s); break;
        default: return fail(DRR_ERR_INVALID_ARGUMENT, "drr_ingest_hu: unknown HU type");
    }
    if (e != cudaSuccess) return cuda_fail(e, "drr_ingest_hu: launch");
    return DRR_OK;
}
