// drr_post.cu -- post-processing of rendered views on the GPU.
//
// drr_neglog restates deepdrr/utils/image_utils.py:18-58 (`_neglog`) for a stack of views:
//   image += min(image) + epsilon      (per view; note it ADDS the minimum, as the reference does)
//   image  = -log(image)
//   image  = (image - min) / (max - min)  per view; if any view is constant, every view becomes 0
// All arithmetic is float32 like the reference's numpy float32 arrays.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/drr_gb300.h"

namespace drr {
void set_last_error(const std::string &msg);  // drr_api.cu
}

namespace {

// Order-preserving map float -> uint32 so that atomicMin/atomicMax on the key order like floats.
__device__ __forceinline__ unsigned int fkey(float f) {
    unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float kfloat(unsigned int k) {
    unsigned int u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

constexpr int kThreads = 256;

__device__ __forceinline__ unsigned int warp_min(unsigned int v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ unsigned int warp_max(unsigned int v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// keys[view*3 + 0] = min(image), 1 = min(-log(.)), 2 = max(-log(.))
__global__ void neglog_init(unsigned int *keys, int n_views) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_views) {
        keys[i * 3 + 0] = 0xffffffffu;
        keys[i * 3 + 1] = 0xffffffffu;
        keys[i * 3 + 2] = 0u;
    }
}

__global__ void neglog_min(const float *__restrict__ img, int64_t npix, unsigned int *keys) {
    const int view = blockIdx.y;
    const float *x = img + (int64_t)view * npix;
    unsigned int m = 0xffffffffu;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x)
        m = min(m, fkey(x[i]));
    m = warp_min(m);
    if ((threadIdx.x & 31) == 0) atomicMin(&keys[view * 3 + 0], m);
}

__global__ void neglog_log(float *__restrict__ img, int64_t npix, float epsilon, unsigned int *keys) {
    const int view = blockIdx.y;
    float *x = img + (int64_t)view * npix;
    const float shift = __fadd_rn(kfloat(keys[view * 3 + 0]), epsilon);
    unsigned int lo = 0xffffffffu, hi = 0u;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
        float y = -logf(__fadd_rn(x[i], shift));
        x[i] = y;
        lo = min(lo, fkey(y));
        hi = max(hi, fkey(y));
    }
    lo = warp_min(lo);
    hi = warp_max(hi);
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&keys[view * 3 + 1], lo);
        atomicMax(&keys[view * 3 + 2], hi);
    }
}

// keys[3 * n_views] = 1 if any view is constant after the log (its min and max agree), else 0:
// one block, so the scaling pass reads one word instead of every view's keys.
__global__ void neglog_flag(unsigned int *keys, int n_views) {
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    int c = 0;
    for (int v = threadIdx.x; v < n_views; v += blockDim.x) c |= (keys[v * 3 + 1] == keys[v * 3 + 2]);
    if (c) atomicOr(&any, 1);
    __syncthreads();
    if (threadIdx.x == 0) keys[3 * n_views] = (unsigned int)any;
}

__global__ void neglog_scale(float *__restrict__ img, int64_t npix, int n_views, const unsigned int *keys) {
    const bool any_constant = keys[3 * n_views] != 0u;
    const int view = blockIdx.y;
    float *x = img + (int64_t)view * npix;
    const float lo = kfloat(keys[view * 3 + 1]);
    const float range = __fsub_rn(kfloat(keys[view * 3 + 2]), lo);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = any_constant ? 0.0f : __fdiv_rn(__fsub_rn(x[i], lo), range);
}

__global__ void clip_upper(float *__restrict__ img, int64_t n, float upper) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        img[i] = fminf(img[i], upper);
}

int blocks_for(int64_t npix) {
    int64_t b = (npix + kThreads * 4 - 1) / (kThreads * 4);
    if (b > 1216) b = 1216;  // 152 SMs x 8
    return b < 1 ? 1 : (int)b;
}

}  // namespace

extern "C" drr_status drr_neglog(float *images, int32_t n_views, int64_t pixels_per_view, float epsilon,
                                 void *stream) {
    if (n_views == 0 || pixels_per_view == 0) return DRR_OK;
    if (!images || n_views < 0 || pixels_per_view < 0 || n_views > 65535) {
        drr::set_last_error("drr_neglog: bad arguments");
        return DRR_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    unsigned int *keys = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&keys, sizeof(unsigned int) * (3 * (size_t)n_views + 1), s);
    if (e != cudaSuccess) {
        drr::set_last_error(std::string("drr_neglog: cudaMallocAsync: ") + cudaGetErrorString(e));
        return DRR_ERR_OUT_OF_MEMORY;
    }
    dim3 grid(blocks_for(pixels_per_view), n_views);
    neglog_init<<<(n_views + 255) / 256, 256, 0, s>>>(keys, n_views);
    neglog_min<<<grid, kThreads, 0, s>>>(images, pixels_per_view, keys);
    neglog_log<<<grid, kThreads, 0, s>>>(images, pixels_per_view, epsilon, keys);
    neglog_flag<<<1, kThreads, 0, s>>>(keys, n_views);
    neglog_scale<<<grid, kThreads, 0, s>>>(images, pixels_per_view, n_views, keys);
    e = cudaGetLastError();
    cudaFreeAsync(keys, s);
    if (e != cudaSuccess) {
        drr::set_last_error(std::string("drr_neglog: launch: ") + cudaGetErrorString(e));
        return DRR_ERR_CUDA;
    }
    return DRR_OK;
}

// ---- drr_neglog_noalloc: the same transform with library-owned scratch -----------------------
//
// Some hosts cannot let a library allocate device memory: a renderer or simulator that owns the
// allocator and pre-budgets every byte, a real-time loop where cudaMalloc/cudaFree would
// synchronise the device, or a CUDA-graph-based pipeline that forbids allocation calls while it
// records. For them this entry point keeps its 12 bytes per view of scratch (plus one flag word) in
// a fixed file-scope device array instead of allocating it. Every GPU that loads the library holds
// the array (kNoAllocMaxViews * 12 + 256 bytes, about 48 KiB) until the process exits.
namespace {

constexpr int kNoAllocMaxViews = 4096;
constexpr int kNoAllocCacheEntries = 64;

static __device__ __align__(256) unsigned int g_neglog_scratch[3 * kNoAllocMaxViews + 64];

// The array's device address differs per CUDA context (each context loads its own copy of the
// module), so it is cached per context, keyed by the driver's context ID, which no later context
// reuses: a cudaDeviceReset, or a caller that makes its own driver context current, gets a new
// lookup instead of a stale address. The driver's context queries are reached through the
// runtime's entry-point table, so the library does not link libcuda.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

std::mutex g_scratch_mutex;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
bool g_ctx_queries_resolved = false;
struct ScratchEntry {
    unsigned long long ctx_id;
    unsigned int *ptr;
};
ScratchEntry g_scratch_cache[kNoAllocCacheEntries];
int g_scratch_cached = 0;

drr_status scratch_fail(const char *what, cudaError_t e) {
    drr::set_last_error(std::string("drr_neglog_noalloc: ") + what + ": " + cudaGetErrorString(e));
    return DRR_ERR_CUDA;
}

// ID of the context current on this thread, or 0 if none is (or the driver cannot say).
unsigned long long current_context_id() {
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current && g_ctx_get_id && g_ctx_get_current(&ctx) == CUDA_SUCCESS && ctx &&
        g_ctx_get_id(ctx, &id) == CUDA_SUCCESS)
        return id;
    return 0;
}

// Device address of g_neglog_scratch in the current context. In host code the array's name is
// only a host-side stand-in, so the address is looked up with cudaGetSymbolAddress, once per
// context (the first call on each device, with that device current), and cached.
drr_status scratch_address(unsigned int **out) {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_ctx_queries_resolved) {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
        fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(fn);
        g_ctx_queries_resolved = true;
    }
    unsigned long long id = current_context_id();
    for (int i = 0; id != 0 && i < g_scratch_cached; i++)
        if (g_scratch_cache[i].ctx_id == id) {
            *out = g_scratch_cache[i].ptr;
            return DRR_OK;
        }
    unsigned int *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_neglog_scratch);  // makes the primary context current
    if (e != cudaSuccess || ptr == nullptr) return scratch_fail("cudaGetSymbolAddress", e);
    if (id == 0) id = current_context_id();
    if (id != 0 && g_scratch_cached < kNoAllocCacheEntries) g_scratch_cache[g_scratch_cached++] = {id, ptr};
    *out = ptr;
    return DRR_OK;
}

}  // namespace

extern "C" drr_status drr_neglog_noalloc(float *images, int32_t n_views, int64_t pixels_per_view, float epsilon,
                                         void *stream) {
    if (n_views == 0 || pixels_per_view == 0) return DRR_OK;
    if (!images || n_views < 0 || pixels_per_view < 0) {
        drr::set_last_error("drr_neglog_noalloc: bad arguments");
        return DRR_ERR_INVALID_ARGUMENT;
    }
    if (n_views > kNoAllocMaxViews) {
        drr::set_last_error("drr_neglog_noalloc: " + std::to_string(n_views) + " views exceed the fixed scratch of " +
                            std::to_string(kNoAllocMaxViews) + " views; split the call or use drr_neglog");
        return DRR_ERR_UNSUPPORTED;
    }
    unsigned int *keys = nullptr;
    drr_status st = scratch_address(&keys);
    if (st != DRR_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 grid(blocks_for(pixels_per_view), n_views);
    // neglog_init resets the per-view minimum / maximum words the previous call left behind
    neglog_init<<<(n_views + 255) / 256, 256, 0, s>>>(keys, n_views);
    neglog_min<<<grid, kThreads, 0, s>>>(images, pixels_per_view, keys);
    neglog_log<<<grid, kThreads, 0, s>>>(images, pixels_per_view, epsilon, keys);
    neglog_flag<<<1, kThreads, 0, s>>>(keys, n_views);
    neglog_scale<<<grid, kThreads, 0, s>>>(images, pixels_per_view, n_views, keys);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        drr::set_last_error(std::string("drr_neglog_noalloc: launch: ") + cudaGetErrorString(e));
        return DRR_ERR_CUDA;
    }
    return DRR_OK;
}

// ---- drr_collected_energy: Projector(collected_energy=True), projector.py:833-853 ----------------
//
// Per view: energy = intensity * solid_angle * photon_count / mean(solid_angle) / pixel_area, in
// float32 operations in the reference's order (numpy float32 arrays; the mean and the pixel area are
// scalars rounded to float32). The mean is summed in float64 per view and rounded once, so it is
// the correctly rounded mean of the view's float32 solid angles.
namespace {

__global__ void ce_sum(const float *__restrict__ sa, int64_t npix, double *sums) {
    const int view = blockIdx.y;
    const float *x = sa + (int64_t)view * npix;
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x)
        acc += (double)x[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&sums[view], acc);
}

// The pixel areas of up to kCeViews views, as kernel parameters (no host-to-device copy).
constexpr int kCeViews = 64;
struct CeAreas {
    float area[kCeViews];  // float32(pixel_size_x * pixel_size_y) per view of the launch
};

__global__ void ce_scale(const float *__restrict__ intensity, const float *__restrict__ sa, float *out, int64_t npix,
                         const double *sums, const __grid_constant__ CeAreas areas, float photons) {
    const int view = blockIdx.y;
    const float mean = (float)(sums[view] / (double)npix);
    const float area = areas.area[view];
    const int64_t off = (int64_t)view * npix;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
        const float e = __fmul_rn(__fmul_rn(intensity[off + i], sa[off + i]), photons);
        out[off + i] = __fdiv_rn(__fdiv_rn(e, mean), area);
    }
}

}  // namespace

extern "C" drr_status drr_collected_energy(const float *intensity, const float *solid_angle, float *out,
                                           int32_t n_views, int64_t pixels_per_view, double photon_count,
                                           const double *pixel_area, void *stream) {
    if (n_views == 0 || pixels_per_view == 0) return DRR_OK;
    if (!intensity || !solid_angle || !out || !pixel_area || n_views < 0 || pixels_per_view < 0 || n_views > 65535) {
        drr::set_last_error("drr_collected_energy: bad arguments");
        return DRR_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    double *sums = nullptr;  // per-view float64 sums of the solid angles
    cudaError_t e = cudaMallocAsync((void **)&sums, sizeof(double) * (size_t)n_views, s);
    if (e != cudaSuccess) {
        drr::set_last_error(std::string("drr_collected_energy: cudaMallocAsync: ") + cudaGetErrorString(e));
        return DRR_ERR_OUT_OF_MEMORY;
    }
    e = cudaMemsetAsync(sums, 0, sizeof(double) * (size_t)n_views, s);
    if (e == cudaSuccess) {
        ce_sum<<<dim3(blocks_for(pixels_per_view), n_views), kThreads, 0, s>>>(solid_angle, pixels_per_view, sums);
        e = cudaGetLastError();
    }
    for (int v0 = 0; v0 < n_views && e == cudaSuccess; v0 += kCeViews) {
        const int nv = n_views - v0 < kCeViews ? n_views - v0 : kCeViews;
        CeAreas a;
        for (int k = 0; k < kCeViews; k++) a.area[k] = k < nv ? (float)pixel_area[v0 + k] : 1.0f;  // a Python float meets float32
        const int64_t off = (int64_t)v0 * pixels_per_view;
        ce_scale<<<dim3(blocks_for(pixels_per_view), nv), kThreads, 0, s>>>(intensity + off, solid_angle + off, out + off,
                                                                          pixels_per_view, sums + v0, a,
                                                                          (float)photon_count);
        e = cudaGetLastError();
    }
    cudaFreeAsync(sums, s);
    if (e != cudaSuccess) {
        drr::set_last_error(std::string("drr_collected_energy: ") + cudaGetErrorString(e));
        return DRR_ERR_CUDA;
    }
    return DRR_OK;
}

extern "C" drr_status drr_clip_upper(float *images, int64_t n, float upper, void *stream) {
    if (n == 0) return DRR_OK;
    if (!images || n < 0) {
        drr::set_last_error("drr_clip_upper: bad arguments");
        return DRR_ERR_INVALID_ARGUMENT;
    }
    clip_upper<<<blocks_for(n), kThreads, 0, (cudaStream_t)stream>>>(images, n, upper);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        drr::set_last_error(std::string("drr_clip_upper: launch: ") + cudaGetErrorString(e));
        return DRR_ERR_CUDA;
    }
    return DRR_OK;
}
