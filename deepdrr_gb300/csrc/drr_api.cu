// drr_api.cu -- C ABI of libdrr_gb300.so: volume sets (textures, label codes), spectrum tables.
//
// Host-side replacement for deepdrr/projector/projector.py (deepdrr v1.2.2):
//   create_cuda_texture            projector.py:116-257   -> make_texture()
//   Projector.initialize (volumes) projector.py:1464-1546 -> drr_volset_create()
//   Projector.initialize (tables)  projector.py:1659-1686 -> drr_tables_create()
// Projection itself (_render_single, projector.py:709-800) is in drr_project.cu.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/drr_gb300.h"
#include "drr_forward.cuh"
#include "drr_internal.h"

namespace {

thread_local std::string g_last_error;

#define DRR_CUDA_TRY(expr, what)                                \
    do {                                                        \
        cudaError_t e_ = (expr);                                \
        if (e_ != cudaSuccess) return drr::cuda_fail(e_, what); \
    } while (0)

using drr::cuda_fail;
using drr::fail;
using drr::Volume;

// bfloat16 -> float16, exact for 0 and |x| in [2^-14, 65504]; anything else raises *bad.
__global__ void bf16_to_f16_kernel(const __nv_bfloat16 *__restrict__ in, size_t n, __half *out, unsigned int *bad) {
    unsigned int local_bad = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float x = __bfloat162float(in[i]);
        const float ax = fabsf(x);
        if (!(ax == 0.0f || (ax >= 6.103515625e-05f && ax <= 65504.0f))) local_bad = 1;
        out[i] = __float2half_rn(x);
    }
    if (local_bad) atomicOr(bad, 1u);
}

__global__ void max_label_kernel(const uint8_t *__restrict__ labels, size_t n, unsigned int *out) {
    unsigned int local = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        local = max(local, (unsigned int)labels[i]);
    for (int o = 16; o > 0; o >>= 1) local = max(local, __shfl_xor_sync(0xffffffffu, local, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, local);
}

// create_cuda_texture (projector.py:116-257): 1-channel cudaArray of extent (ni, nj, nk), clamp
// addressing on every axis, unnormalised coordinates, element-type reads.
drr_status make_texture(const void *src, int elem_bytes, cudaChannelFormatDesc fd, bool linear, int ni, int nj,
                        int nk, cudaStream_t stream, cudaArray_t *arr_out, cudaTextureObject_t *tex_out) {
    cudaExtent ext = make_cudaExtent((size_t)ni, (size_t)nj, (size_t)nk);
    cudaArray_t arr = nullptr;
    DRR_CUDA_TRY(cudaMalloc3DArray(&arr, &fd, ext, 0), "cudaMalloc3DArray");
    cudaMemcpy3DParms cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.srcPtr = make_cudaPitchedPtr(const_cast<void *>(src), (size_t)ni * elem_bytes, (size_t)ni, (size_t)nj);
    cp.dstArray = arr;
    cp.extent = ext;
    cp.kind = cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaMemcpy3DAsync(&cp, stream);
    if (e != cudaSuccess) {
        cudaFreeArray(arr);
        return cuda_fail(e, "cudaMemcpy3DAsync (volume to texture array)");
    }
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.filterMode = linear ? cudaFilterModeLinear : cudaFilterModePoint;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    cudaTextureObject_t tex = 0;
    e = cudaCreateTextureObject(&tex, &rd, &td, nullptr);
    if (e != cudaSuccess) {
        cudaFreeArray(arr);
        return cuda_fail(e, "cudaCreateTextureObject");
    }
    *arr_out = arr;
    *tex_out = tex;
    return DRR_OK;
}

void free_volume(Volume &v) {
    if (v.density_tex) cudaDestroyTextureObject(v.density_tex);
    if (v.density_point) cudaDestroyTextureObject(v.density_point);
    if (v.density_array) cudaFreeArray(v.density_array);
    if (v.coded) cudaFree(v.coded);
    if (v.gen_words) cudaFree(v.gen_words);
    if (v.gen_start) cudaFree(v.gen_start);
    v = Volume();
}

// Label codes of every base of a volume (see drr::pack_labels_kernel), owned by the volume set: 2
// bytes per base. The neighbourhoods of three or more labels (rare in CT) get their packed labels
// in a side table, numbered within segments of kGeneralSegment bases of a code-table row so that a
// number fits the codes' 11 free bits (drr::index_general_kernel): 4 bytes each, plus 4 bytes per
// segment for its first index.
drr_status make_label_tables(const uint8_t *src, int ni, int nj, int nk, cudaStream_t s, Volume &v) {
    const size_t row = (size_t)ni + 2, plane = row * (nj + 2), np = plane * (nk + 2);
    DRR_CUDA_TRY(cudaMalloc(&v.coded, np * sizeof(uint16_t)), "cudaMalloc (label codes)");
    const size_t blocks = (np + 255) / 256;
    drr::pack_labels_kernel<<<(unsigned)(blocks < 1048576 ? blocks : 1048576), 256, 0, s>>>(src, ni, nj, nk,
                                                                                           v.coded);
    DRR_CUDA_TRY(cudaGetLastError(), "pack_labels_kernel launch");
    const size_t segs = (size_t)(nk + 2) * (nj + 2) * drr::general_segments_per_row(ni);
    const unsigned seg_blocks = (unsigned)((segs + 7) / 8 < 1048576 ? (segs + 7) / 8 : 1048576);  // 8 warps each
    DRR_CUDA_TRY(cudaMalloc(&v.gen_start, sizeof(uint32_t) * (segs + 1)), "cudaMalloc (general index)");
    drr::count_general_kernel<<<seg_blocks, 256, 0, s>>>(v.coded, ni, nj, nk, v.gen_start);
    DRR_CUDA_TRY(cudaGetLastError(), "count_general_kernel launch");
    std::vector<uint32_t> start(segs + 1);
    DRR_CUDA_TRY(cudaMemcpyAsync(start.data(), v.gen_start, sizeof(uint32_t) * segs, cudaMemcpyDeviceToHost, s),
                 "general counts download");
    DRR_CUDA_TRY(cudaStreamSynchronize(s), "general counts download");
    uint64_t total = 0;  // counts to first indices (exclusive sums)
    for (size_t g = 0; g < segs; g++) {
        const uint64_t c = start[g];
        start[g] = (uint32_t)total;
        total += c;
    }
    if (total > 0xFFFFFFFFull) return drr::fail(DRR_ERR_UNSUPPORTED, "drr_volset_create: too many neighbourhoods of three or more labels");
    start[segs] = (uint32_t)total;
    DRR_CUDA_TRY(cudaMalloc(&v.gen_words, sizeof(uint32_t) * (total > 0 ? total : 1)), "cudaMalloc (general words)");
    DRR_CUDA_TRY(cudaMemcpyAsync(v.gen_start, start.data(), sizeof(uint32_t) * (segs + 1), cudaMemcpyHostToDevice, s),
                 "general index upload");
    drr::index_general_kernel<<<seg_blocks, 256, 0, s>>>(src, ni, nj, nk, v.coded, v.gen_start, v.gen_words);
    DRR_CUDA_TRY(cudaGetLastError(), "index_general_kernel launch");
    // rows of bases j = -2 and the plane of bases k = -2 hold the same neighbourhoods as those of -1:
    // copy their codes, numbers included, so that a lookup may clamp j and k to -1
    DRR_CUDA_TRY(cudaMemcpy2DAsync(v.coded, plane * sizeof(uint16_t), v.coded + row, plane * sizeof(uint16_t),
                                   row * sizeof(uint16_t), (size_t)nk + 2, cudaMemcpyDeviceToDevice, s),
                 "label codes of the base rows -2");
    DRR_CUDA_TRY(cudaMemcpyAsync(v.coded, v.coded + plane, plane * sizeof(uint16_t), cudaMemcpyDeviceToDevice, s),
                 "label codes of the base plane -2");
    DRR_CUDA_TRY(cudaStreamSynchronize(s), "general index upload");  // `start` is a host vector
    return DRR_OK;
}

}  // namespace

namespace drr {
__global__ void pack_labels_kernel(const uint8_t *__restrict__ labels, int ni, int nj, int nk, uint16_t *coded) {
    const size_t np = (size_t)(ni + 2) * (nj + 2) * (nk + 2);
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < np; e += (size_t)gridDim.x * blockDim.x) {
        const int bi = (int)(e % (ni + 2)) - 2;
        const int bj = (int)((e / (ni + 2)) % (nj + 2)) - 2;
        const int bk = (int)(e / ((size_t)(ni + 2) * (nj + 2))) - 2;
        uint32_t word = 0;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const int i = clampi(bi + (c & 1), 0, ni - 1);
            const int j = clampi(bj + ((c >> 1) & 1), 0, nj - 1);
            const int k = clampi(bk + (c >> 2), 0, nk - 1);
            word |= ((uint32_t)labels[((size_t)k * nj + j) * ni + i] & 15u) << (4 * c);
        }
        // A = corner 0's label, B = the first other label (A when there is none), the mask of the
        // corners labelled B (bit 0, corner 0's, is always clear); kCodeGeneral marks a neighbourhood
        // with three or more labels
        const uint32_t A = word & 15u;
        uint32_t B = A, mask = 0u;
        bool general = false;
#pragma unroll
        for (int c = 1; c < 8; c++) {
            const uint32_t L = (word >> (4 * c)) & 15u;
            if (L == A) continue;
            if (B == A) B = L;
            if (L == B)
                mask |= 1u << c;
            else
                general = true;
        }
        coded[e] = (uint16_t)(general ? (kCodeGeneral | A) : (A | (B << 4) | (mask << 8)));
    }
}

// Neighbourhoods of three or more labels in each segment of kGeneralSegment bases of a code-table
// row, one warp per segment (segment g: row g / segs_per_row, bases (g % segs_per_row) * kGeneralSegment
// onwards).
__global__ void count_general_kernel(const uint16_t *__restrict__ coded, int ni, int nj, int nk, uint32_t *counts) {
    const size_t row = (size_t)ni + 2;
    const size_t spr = general_segments_per_row(ni);
    const size_t segs = (size_t)(nk + 2) * (nj + 2) * spr;
    const int lane = threadIdx.x & 31;
    for (size_t g = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < segs;
         g += ((size_t)gridDim.x * blockDim.x) >> 5) {
        const size_t r = g / spr, i0 = (g % spr) * kGeneralSegment;
        const size_t i1 = i0 + kGeneralSegment < row ? i0 + kGeneralSegment : row;
        uint32_t c = 0;
        for (size_t i = i0 + lane; i < i1; i += 32) c += (coded[r * row + i] & kCodeGeneral) ? 1u : 0u;
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) counts[g] = c;
    }
}

// Numbers the neighbourhoods of three or more labels of each row segment in table order (one warp
// per segment), stores each one's packed labels (4 bits per corner: the eight labels the reference
// fetches, at clamp(b + d, 0, n - 1)) at words[start[g] + number] and the number (below
// kGeneralSegment) in its code's free bits: 4-7 the low four, 9-15 the high seven.
__global__ void index_general_kernel(const uint8_t *__restrict__ labels, int ni, int nj, int nk, uint16_t *coded,
                                     const uint32_t *__restrict__ start, uint32_t *words) {
    const size_t row = (size_t)ni + 2;
    const size_t spr = general_segments_per_row(ni);
    const size_t segs = (size_t)(nk + 2) * (nj + 2) * spr;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    for (size_t g = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < segs;
         g += ((size_t)gridDim.x * blockDim.x) >> 5) {
        const size_t r = g / spr, i0 = (g % spr) * kGeneralSegment;
        const size_t i1 = i0 + kGeneralSegment < row ? i0 + kGeneralSegment : row;
        const int bj = (int)(r % (size_t)(nj + 2)) - 2, bk = (int)(r / (size_t)(nj + 2)) - 2;
        uint32_t running = 0;
        for (size_t ib = i0; ib < i1; ib += 32) {
            const size_t i = ib + lane;
            uint16_t *pc = coded + r * row + i;
            const bool gen = i < i1 && (*pc & kCodeGeneral);
            const unsigned b = __ballot_sync(0xffffffffu, gen);
            if (gen) {
                const uint32_t number = running + __popc(b & lt);
                const int bi = (int)i - 2;
                uint32_t word = 0;
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    const int ii = clampi(bi + (c & 1), 0, ni - 1);
                    const int jj = clampi(bj + ((c >> 1) & 1), 0, nj - 1);
                    const int kk = clampi(bk + (c >> 2), 0, nk - 1);
                    word |= ((uint32_t)labels[((size_t)kk * nj + jj) * ni + ii] & 15u) << (4 * c);
                }
                words[start[g] + number] = word;
                *pc = (uint16_t)((*pc & (kCodeGeneral | 15u)) | ((number & 15u) << 4) | ((number >> 4) << 9));
            }
            running += __popc(b);
        }
    }
}
}  // namespace drr

namespace drr {
void set_last_error(const std::string &msg) { g_last_error = msg; }

drr_status fail(drr_status s, const std::string &msg) {
    g_last_error = msg;
    return s;
}

drr_status cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return e == cudaErrorMemoryAllocation ? DRR_ERR_OUT_OF_MEMORY : DRR_ERR_CUDA;
}

void free_staging(Staging &st) {
    if (st.uploaded) {
        cudaEventSynchronize(st.uploaded);
        cudaEventDestroy(st.uploaded);
    }
    if (st.host) cudaFreeHost(st.host);
    if (st.device) cudaFree(st.device);
    if (st.counter) cudaFree(st.counter);
    st = Staging();
}

drr_status ensure_staging(Staging &st, size_t bytes) {
    if (!st.counter) DRR_CUDA_TRY(cudaMalloc(&st.counter, sizeof(unsigned int)), "cudaMalloc (work counter)");
    if (!st.uploaded) DRR_CUDA_TRY(cudaEventCreateWithFlags(&st.uploaded, cudaEventDisableTiming), "cudaEventCreate");
    if (bytes <= st.capacity) return DRR_OK;
    if (st.pending) cudaEventSynchronize(st.uploaded);
    if (st.host) cudaFreeHost(st.host);
    if (st.device) cudaFree(st.device);
    st.host = st.device = nullptr;
    st.capacity = 0;
    DRR_CUDA_TRY(cudaMallocHost(&st.host, bytes), "cudaMallocHost (view staging)");
    DRR_CUDA_TRY(cudaMalloc(&st.device, bytes), "cudaMalloc (view records)");
    st.capacity = bytes;
    return DRR_OK;
}
}  // namespace drr

extern "C" {

const char *drr_last_error(void) { return g_last_error.c_str(); }

const char *drr_version(void) { return "deepdrr-gb300 0.1.0 (sm_103a)"; }

drr_status drr_volset_create(const drr_volume_desc *volumes, int32_t n_volumes, int32_t n_materials, void *stream,
                             drr_volset **out) {
    g_last_error.clear();
    if (!out) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_volset_create: out is NULL");
    *out = nullptr;
    if (n_volumes < 1 || n_volumes > DRR_MAX_VOLUMES)
        return fail(n_volumes < 1 ? DRR_ERR_INVALID_ARGUMENT : DRR_ERR_UNSUPPORTED,
                    "drr_volset_create: n_volumes must be in [1, " + std::to_string(DRR_MAX_VOLUMES) + "], got " +
                        std::to_string(n_volumes));
    if (n_materials < 1 || n_materials > DRR_MAX_MATERIALS)
        return fail(n_materials < 1 ? DRR_ERR_INVALID_ARGUMENT : DRR_ERR_UNSUPPORTED,
                    "drr_volset_create: n_materials must be in [1, " + std::to_string(DRR_MAX_MATERIALS) + "], got " +
                        std::to_string(n_materials));
    if (!volumes) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_volset_create: volumes is NULL");
    for (int i = 0; i < n_volumes; i++) {
        const drr_volume_desc &d = volumes[i];
        if (!d.density || !d.labels)
            return fail(DRR_ERR_INVALID_ARGUMENT, "drr_volset_create: volume " + std::to_string(i) + " has a NULL pointer");
        if (d.ni < 1 || d.nj < 1 || d.nk < 1)
            return fail(DRR_ERR_INVALID_ARGUMENT, "drr_volset_create: volume " + std::to_string(i) + " has an empty extent");
        if (d.ni > 16384 || d.nj > 16384 || d.nk > 16384)
            return fail(DRR_ERR_UNSUPPORTED, "drr_volset_create: 3D textures are limited to 16384 texels per axis");
        if (d.density_type != DRR_DENSITY_F32 && d.density_type != DRR_DENSITY_F16 &&
            d.density_type != DRR_DENSITY_BF16)
            return fail(DRR_ERR_UNSUPPORTED, "drr_volset_create: volume " + std::to_string(i) +
                                                 ": unknown density type " + std::to_string(d.density_type));
    }
    cudaStream_t s = (cudaStream_t)stream;
    drr_volset *set = new (std::nothrow) drr_volset();
    if (!set) return fail(DRR_ERR_OUT_OF_MEMORY, "drr_volset_create: host allocation failed");
    set->n_volumes = n_volumes;
    set->n_materials = n_materials;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&set->sm_count, cudaDevAttrMultiProcessorCount, dev);
    }
    unsigned int *d_max = nullptr;  // per-volume maximum label, then one range-violation flag
    cudaError_t e = cudaMalloc(&d_max, sizeof(unsigned int) * (DRR_MAX_VOLUMES + 1));
    if (e != cudaSuccess) {
        delete set;
        return cuda_fail(e, "cudaMalloc (label check)");
    }
    unsigned int *d_bad = d_max + DRR_MAX_VOLUMES;
    cudaMemsetAsync(d_max, 0, sizeof(unsigned int) * (DRR_MAX_VOLUMES + 1), s);
    drr_status st = DRR_OK;
    for (int i = 0; i < n_volumes && st == DRR_OK; i++) {
        const drr_volume_desc &d = volumes[i];
        Volume &v = set->vol[i];
        v.ni = d.ni;
        v.nj = d.nj;
        v.nk = d.nk;
        v.density_type = d.density_type;
        const size_t n = (size_t)d.ni * d.nj * d.nk;
        max_label_kernel<<<1216, 256, 0, s>>>(d.labels, n, d_max + i);
        const bool half = d.density_type != DRR_DENSITY_F32;
        const void *src = d.density;
        __half *converted = nullptr;
        if (d.density_type == DRR_DENSITY_BF16) {
            // bfloat16 has no texture format; its values are exact in float16 between 2^-14 and
            // 65504 (and 0), so the texture holds the same numbers in float16
            e = cudaMalloc(&converted, n * sizeof(__half));
            if (e != cudaSuccess) {
                st = cuda_fail(e, "cudaMalloc (bfloat16 conversion)");
                break;
            }
            cudaMemsetAsync(d_bad, 0, sizeof(unsigned int), s);
            bf16_to_f16_kernel<<<1216, 256, 0, s>>>((const __nv_bfloat16 *)d.density, n, converted, d_bad);
            unsigned int bad = 0;
            e = cudaMemcpyAsync(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                cudaFree(converted);
                st = cuda_fail(e, "bfloat16 conversion");
                break;
            }
            if (bad) {
                cudaFree(converted);
                st = fail(DRR_ERR_UNSUPPORTED, "drr_volset_create: volume " + std::to_string(i) +
                                                   " has bfloat16 densities outside float16's normal range "
                                                   "(|x| in [2^-14, 65504] or 0); store it as float32");
                break;
            }
            src = converted;
        }
        cudaChannelFormatDesc fd = half ? cudaCreateChannelDesc(16, 0, 0, 0, cudaChannelFormatKindFloat)
                                        : cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindFloat);
        st = make_texture(src, half ? 2 : 4, fd, true, d.ni, d.nj, d.nk, s, &v.density_array, &v.density_tex);
        if (converted) {
            cudaStreamSynchronize(s);
            cudaFree(converted);
        }
        if (st != DRR_OK) break;
        st = make_label_tables(d.labels, d.ni, d.nj, d.nk, s, v);
    }
    unsigned int hmax[DRR_MAX_VOLUMES] = {0};
    if (st == DRR_OK) {
        e = cudaMemcpyAsync(hmax, d_max, sizeof(hmax), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_fail(e, "drr_volset_create: label check");
    }
    cudaFree(d_max);
    if (st == DRR_OK) {
        for (int i = 0; i < n_volumes; i++)
            if ((int)hmax[i] >= n_materials) {
                st = fail(DRR_ERR_INVALID_ARGUMENT, "drr_volset_create: volume " + std::to_string(i) + " has label " +
                                                        std::to_string(hmax[i]) + " >= n_materials (" +
                                                        std::to_string(n_materials) + ")");
                break;
            }
    }
    if (st != DRR_OK) {
        for (int i = 0; i < n_volumes; i++) free_volume(set->vol[i]);
        delete set;
        return st;
    }
    *out = set;
    return DRR_OK;
}

drr_status drr_volset_destroy(drr_volset *set) {
    g_last_error.clear();
    if (!set) return DRR_OK;
    for (int i = 0; i < set->n_volumes; i++) free_volume(set->vol[i]);
    drr::free_staging(set->staging);
    delete set;
    return DRR_OK;
}

drr_status drr_volset_set_density(drr_volset *set, int32_t volume, const void *density, void *stream) {
    g_last_error.clear();
    if (!set || !density) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_volset_set_density: NULL argument");
    if (volume < 0 || volume >= set->n_volumes)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_volset_set_density: volume index out of range");
    Volume &v = set->vol[volume];
    if (v.density_type == DRR_DENSITY_BF16)
        return fail(DRR_ERR_UNSUPPORTED, "drr_volset_set_density: bfloat16 volumes are converted once at creation");
    const size_t elem = v.density_type == DRR_DENSITY_F32 ? 4 : 2;
    cudaMemcpy3DParms cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.srcPtr = make_cudaPitchedPtr(const_cast<void *>(density), (size_t)v.ni * elem, (size_t)v.ni, (size_t)v.nj);
    cp.dstArray = v.density_array;
    cp.extent = make_cudaExtent((size_t)v.ni, (size_t)v.nj, (size_t)v.nk);
    cp.kind = cudaMemcpyDeviceToDevice;
    DRR_CUDA_TRY(cudaMemcpy3DAsync(&cp, (cudaStream_t)stream), "drr_volset_set_density: cudaMemcpy3DAsync");
    return DRR_OK;
}

drr_status drr_tables_create(const float *energies_kev, const float *pdf, const float *mu_over_rho, int32_t n_bins,
                             int32_t n_materials, void *stream, drr_tables **out) {
    g_last_error.clear();
    if (!out) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_tables_create: out is NULL");
    *out = nullptr;
    if (!energies_kev || !pdf || !mu_over_rho)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_tables_create: NULL table pointer");
    if (n_bins < 1) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_tables_create: n_bins must be >= 1");
    if (n_materials < 1 || n_materials > DRR_MAX_MATERIALS)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_tables_create: n_materials out of range");
    drr_tables *t = new (std::nothrow) drr_tables();
    if (!t) return fail(DRR_ERR_OUT_OF_MEMORY, "drr_tables_create: host allocation failed");
    const size_t nfloat = (size_t)n_bins * (2 + n_materials);
    cudaError_t e = cudaMalloc(&t->d_buf, nfloat * sizeof(float));
    if (e != cudaSuccess) {
        delete t;
        return cuda_fail(e, "cudaMalloc (tables)");
    }
    cudaStream_t s = (cudaStream_t)stream;
    e = cudaMemcpyAsync(t->d_buf, energies_kev, n_bins * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(t->d_buf + n_bins, pdf, n_bins * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(t->d_buf + 2 * n_bins, mu_over_rho, (size_t)n_bins * n_materials * sizeof(float),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaFree(t->d_buf);
        delete t;
        return cuda_fail(e, "drr_tables_create: upload");
    }
    t->n_bins = n_bins;
    t->n_materials = n_materials;
    *out = t;
    return DRR_OK;
}

drr_status drr_tables_destroy(drr_tables *tables) {
    g_last_error.clear();
    if (!tables) return DRR_OK;
    cudaFree(tables->d_buf);
    delete tables;
    return DRR_OK;
}

}  // extern "C"

