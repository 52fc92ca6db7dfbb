// drr_noise.cu -- detector noise of Projector(add_noise=True) on the GPU.
//
// Replaces deepdrr/projector/analytic_generators.py:10-18 (add_noise, called by Projector.project at
// projector.py:691-695). Per view, with lambda = photon_prob * photon_count:
//     shot  = (Poisson(lambda) - lambda) * intensity / lambda
//     shot  = convolve2d(shot, K, mode="same")  (zero fill; K the 3x3 kernel of analytic_generators.py:6)
//     out   = clip(intensity + shot, 0, 1e31)
// The reference also adds electronic noise scaled by factor_electronic_noise, which it sets to 0
// (analytic_generators.py:7), so that term is identically zero and is not generated.
//
// Variates come from Philox4x32-10 keyed by the caller's seed with the pixel's flat index
// (view * H * W + row * W + column) as the counter, so a block recomputes its halo pixels' variates
// exactly and drr_poisson_sample over the same lambdas and seed returns the same variates.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/drr_gb300.h"
#include "drr_internal.h"
#include "drr_philox.h"

using drr::cuda_fail;
using drr::fail;

namespace {

constexpr int kNoiseTileW = 32;
constexpr int kNoiseTileH = 8;

// analytic_generators.py:6 (Wang et al., Med Phys 41(7), 2014), row-major [i][j]
__constant__ double c_shot_kernel[3][3] = {{0.03, 0.06, 0.02}, {0.11, 0.98, 0.11}, {0.02, 0.06, 0.03}};

__global__ void poisson_kernel(const float *__restrict__ lam, int64_t n, uint64_t seed, float *__restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        drr::UniformStream u(seed, (uint64_t)i);
        out[i] = (float)drr::poisson((double)lam[i], u);
    }
}

__global__ void __launch_bounds__(kNoiseTileW *kNoiseTileH)
    add_noise_kernel(const float *__restrict__ intensity, const float *__restrict__ prob, float *__restrict__ out,
                     int H, int W, float photon_count, uint64_t seed) {
    __shared__ double s_shot[kNoiseTileH + 2][kNoiseTileW + 2];
    const int x0 = blockIdx.x * kNoiseTileW - 1, y0 = blockIdx.y * kNoiseTileH - 1;
    const size_t plane = (size_t)H * W;
    const size_t base = (size_t)blockIdx.z * plane;
    const int tid = threadIdx.y * kNoiseTileW + threadIdx.x;
    for (int s = tid; s < (kNoiseTileH + 2) * (kNoiseTileW + 2); s += kNoiseTileW * kNoiseTileH) {
        const int ty = s / (kNoiseTileW + 2), tx = s % (kNoiseTileW + 2);
        const int y = y0 + ty, x = x0 + tx;
        double shot = 0.0;  // zero fill outside the image
        if (y >= 0 && y < H && x >= 0 && x < W) {
            const size_t g = base + (size_t)y * W + x;
            const float lam = __fmul_rn(prob[g], photon_count);
            drr::UniformStream u(seed, (uint64_t)g);
            const double k = drr::poisson((double)lam, u);
            shot = (k - (double)lam) * (double)intensity[g] / (double)lam;
        }
        s_shot[ty][tx] = shot;
    }
    __syncthreads();
    const int x = x0 + 1 + threadIdx.x, y = y0 + 1 + threadIdx.y;
    if (x >= W || y >= H) return;
    // convolve2d: sum_ij K[i][j] shot[y + 1 - i][x + 1 - j]
    double acc = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) acc += c_shot_kernel[i][j] * s_shot[threadIdx.y + 2 - i][threadIdx.x + 2 - j];
    const size_t g = base + (size_t)y * W + x;
    const double v = (double)intensity[g] + acc;
    out[g] = v != v ? (float)v : (float)fmin(fmax(v, 0.0), 1.0e31);
}

}  // namespace

extern "C" drr_status drr_poisson_sample(const float *lambda, int64_t n, uint64_t seed, float *out, void *stream) {
    drr::set_last_error("");
    if (n < 0) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_poisson_sample: n < 0");
    if (n == 0) return DRR_OK;
    if (!lambda || !out) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_poisson_sample: NULL pointer");
    const int64_t blocks = (n + 255) / 256;
    poisson_kernel<<<(unsigned)(blocks < 4864 ? blocks : 4864), 256, 0, (cudaStream_t)stream>>>(lambda, n, seed, out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "drr_poisson_sample: launch");
    return DRR_OK;
}

extern "C" drr_status drr_add_noise(const float *intensity, const float *photon_prob, float *out, int32_t n_views,
                                    int32_t height, int32_t width, double photon_count, uint64_t seed, void *stream) {
    drr::set_last_error("");
    if (n_views < 0 || height < 0 || width < 0) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_add_noise: negative size");
    if (n_views == 0 || height == 0 || width == 0) return DRR_OK;
    if (!intensity || !photon_prob || !out) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_add_noise: NULL pointer");
    if (out == intensity || out == photon_prob)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_add_noise: out must not alias the inputs");
    if (!(photon_count > 0.0) || !std::isfinite(photon_count))
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_add_noise: photon_count must be positive and finite");
    if (n_views > 65535) return fail(DRR_ERR_UNSUPPORTED, "drr_add_noise: more than 65535 views in one call");
    const dim3 grid((width + kNoiseTileW - 1) / kNoiseTileW, (height + kNoiseTileH - 1) / kNoiseTileH, n_views);
    if (grid.y > 65535) return fail(DRR_ERR_UNSUPPORTED, "drr_add_noise: image too tall");
    add_noise_kernel<<<grid, dim3(kNoiseTileW, kNoiseTileH), 0, (cudaStream_t)stream>>>(
        intensity, photon_prob, out, height, width, (float)photon_count, seed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "drr_add_noise: launch");
    return DRR_OK;
}
