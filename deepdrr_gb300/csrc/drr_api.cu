// drr_api.cu -- C ABI of libdrr_gb300.so: volume sets (textures), spectrum tables, projection.
//
// Host-side replacement for deepdrr/projector/projector.py (deepdrr v1.2.2):
//   create_cuda_texture            projector.py:116-257   -> make_texture()
//   Projector.initialize (volumes) projector.py:1464-1546 -> drr_volset_create()
//   Projector.initialize (tables)  projector.py:1659-1686 -> drr_tables_create()
//   _update_object_locations       projector.py:802-831   -> pack_view()
//   _render_single                 projector.py:709-800   -> drr_project()
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "../../include/drr_gb300.h"
#include "drr_forward.cuh"

namespace {

thread_local std::string g_last_error;

drr_status fail(drr_status s, const std::string &msg) {
    g_last_error = msg;
    return s;
}

drr_status cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return e == cudaErrorMemoryAllocation ? DRR_ERR_OUT_OF_MEMORY : DRR_ERR_CUDA;
}

#define DRR_CUDA_TRY(expr, what)                 \
    do {                                         \
        cudaError_t e_ = (expr);                 \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

struct Volume {
    cudaArray_t density_array = nullptr;
    cudaTextureObject_t density_tex = 0;
    uint32_t *packed = nullptr;   // [(nk+1)][(nj+1)][(ni+1)] 2x2x2 label words
    int ni = 0, nj = 0, nk = 0;
    int density_type = DRR_DENSITY_F32;
};

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
    if (v.density_array) cudaFreeArray(v.density_array);
    if (v.packed) cudaFree(v.packed);
    v = Volume();
}

// Label words of every base of a volume (see drr::pack_labels_kernel), owned by the volume set.
drr_status make_label_tables(const uint8_t *src, int ni, int nj, int nk, cudaStream_t s, Volume &v) {
    const size_t np = (size_t)(ni + 1) * (nj + 1) * (nk + 1);
    DRR_CUDA_TRY(cudaMalloc(&v.packed, np * sizeof(uint32_t)), "cudaMalloc (packed labels)");
    const size_t blocks = (np + 255) / 256;
    drr::pack_labels_kernel<<<(unsigned)(blocks < 1048576 ? blocks : 1048576), 256, 0, s>>>(src, ni, nj, nk,
                                                                                           v.packed);
    DRR_CUDA_TRY(cudaGetLastError(), "pack_labels_kernel launch");
    return DRR_OK;
}

}  // namespace

namespace drr {
__global__ void pack_labels_kernel(const uint8_t *__restrict__ labels, int ni, int nj, int nk, uint32_t *packed) {
    const size_t np = (size_t)(ni + 1) * (nj + 1) * (nk + 1);
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < np; e += (size_t)gridDim.x * blockDim.x) {
        const int bi = (int)(e % (ni + 1)) - 1;
        const int bj = (int)((e / (ni + 1)) % (nj + 1)) - 1;
        const int bk = (int)(e / ((size_t)(ni + 1) * (nj + 1))) - 1;
        uint32_t word = 0;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const int i = clampi(bi + (c & 1), 0, ni - 1);
            const int j = clampi(bj + ((c >> 1) & 1), 0, nj - 1);
            const int k = clampi(bk + (c >> 2), 0, nk - 1);
            word |= ((uint32_t)labels[((size_t)k * nj + j) * ni + i] & 15u) << (4 * c);
        }
        packed[e] = word;
    }
}
}  // namespace drr

namespace drr {
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace drr

struct drr_volset {
    int n_volumes = 0;
    int n_materials = 0;
    Volume vol[DRR_MAX_VOLUMES];
};

struct drr_tables {
    int n_bins = 0;
    int n_materials = 0;
    float *d_buf = nullptr;  // energies [n_bins] | pdf [n_bins] | mu [n_bins][n_materials]
};

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
    delete set;
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

namespace {

// _update_object_locations (projector.py:802-831): float64 host geometry cast to float32. The
// source position in IJK is computed in float64 in a fixed order, ((a0 s0 + a1 s1) + a2 s2) + a3.
template <int NV>
void pack_view(const drr_project_args &a, int nvol, int view, drr::ViewRec<NV> &rec) {
    const double *W = a.world_from_index + (size_t)view * 9;
    for (int j = 0; j < 9; j++) rec.w[j] = (float)W[j];
    rec.pad = 0.0f;
    const double *src = a.source_world + (size_t)view * 3;
    for (int i = 0; i < NV; i++) {
        drr::VolPose &vp = rec.vol[i];
        if (i >= nvol) {
            std::memset(&vp, 0, sizeof(vp));
            continue;
        }
        const double *A = a.ijk_from_world + ((size_t)view * nvol + i) * 12;
        for (int r = 0; r < 3; r++) {
            for (int c = 0; c < 3; c++) vp.a[r * 3 + c] = (float)A[r * 4 + c];
            volatile double acc = A[r * 4 + 0] * src[0];
            acc = acc + A[r * 4 + 1] * src[1];
            acc = acc + A[r * 4 + 2] * src[2];
            acc = acc + A[r * 4 + 3];
            vp.s[r] = (float)acc;
        }
    }
}

int material_bucket(int m) {
    if (m <= 2) return 2;
    if (m <= 3) return 3;
    if (m <= 4) return 4;
    if (m <= 6) return 6;
    if (m <= 8) return 8;
    return 16;
}

template <int NV>
cudaError_t dispatch_m(const drr::ForwardParams<NV> &p, int bucket, cudaStream_t s) {
    switch (bucket) {
        case 2: return drr::launch_forward<NV, 2>(p, s);
        case 3: return drr::launch_forward<NV, 3>(p, s);
        case 4: return drr::launch_forward<NV, 4>(p, s);
        case 6: return drr::launch_forward<NV, 6>(p, s);
        case 8: return drr::launch_forward<NV, 8>(p, s);
        default: return drr::launch_forward<NV, 16>(p, s);
    }
}

template <int NV>
drr_status project_nv(drr_volset *set, const drr_tables *tab, const drr_project_args &a, cudaStream_t s) {
    drr::ForwardParams<NV> *pp = new (std::nothrow) drr::ForwardParams<NV>();
    if (!pp) return fail(DRR_ERR_OUT_OF_MEMORY, "drr_project: host allocation failed");
    drr::ForwardParams<NV> &p = *pp;
    std::memset(&p, 0, sizeof(p));
    for (int i = 0; i < NV; i++) {
        const Volume &v = set->vol[i];
        p.vol[i].density = v.density_tex;
        p.vol[i].packed = v.packed;
        p.vol[i].n[0] = v.ni;
        p.vol[i].n[1] = v.nj;
        p.vol[i].n[2] = v.nk;
        p.vol[i].nm1[0] = (float)(v.ni - 1);
        p.vol[i].nm1[1] = (float)(v.nj - 1);
        p.vol[i].nm1[2] = (float)(v.nk - 1);
        p.vol[i].hi[0] = (float)(v.ni - 0.5);
        p.vol[i].hi[1] = (float)(v.nj - 0.5);
        p.vol[i].hi[2] = (float)(v.nk - 0.5);
        p.vol[i].priority = a.priority[i];
        p.vol[i].enabled = a.enabled[i] ? 1 : 0;
    }
    p.energies = tab->d_buf;
    p.pdf = tab->d_buf + tab->n_bins;
    p.mu = tab->d_buf + 2 * tab->n_bins;
    p.intensity = a.intensity;
    p.photon_prob = a.photon_prob;
    p.area_density = a.area_density;
    p.solid_angle = a.solid_angle;
    p.width = a.width;
    p.height = a.height;
    p.n_materials = set->n_materials;
    p.n_bins = tab->n_bins;
    p.step = a.step;
    p.max_ray_length = a.max_ray_length;
    p.attenuate = (a.flags & DRR_FLAG_ATTENUATE_OUTSIDE) ? 1 : 0;
    p.air_index = a.air_index;
    p.full_march = (a.flags & DRR_FLAG_FULL_MARCH) ? 1 : 0;
    const int bucket = material_bucket(set->n_materials);
    drr_status st = DRR_OK;
    for (int v0 = 0; v0 < a.n_views; v0 += drr::kViewsPerLaunch) {
        const int nv = a.n_views - v0 < drr::kViewsPerLaunch ? a.n_views - v0 : drr::kViewsPerLaunch;
        p.view0 = v0;
        p.n_views = nv;
        for (int k = 0; k < nv; k++) pack_view<NV>(a, set->n_volumes, v0 + k, p.views[k]);
        cudaError_t e = dispatch_m<NV>(p, bucket, s);
        if (e != cudaSuccess) {
            st = cuda_fail(e, "drr_project: kernel launch");
            break;
        }
    }
    delete pp;
    return st;
}

}  // namespace

extern "C" drr_status drr_project(drr_volset *set, const drr_tables *tables, const drr_project_args *args,
                                  void *stream) {
    g_last_error.clear();
    if (!set || !tables || !args) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: NULL handle or args");
    const drr_project_args &a = *args;
    if (a.width < 1 || a.height < 1) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: empty detector");
    if ((int64_t)a.width * a.height > (int64_t)1 << 28)
        return fail(DRR_ERR_UNSUPPORTED, "drr_project: detector larger than 2^28 pixels");
    if (a.height > 65535 * drr::kTileH) return fail(DRR_ERR_UNSUPPORTED, "drr_project: detector too tall");
    if (a.n_views < 0) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: n_views < 0");
    if (a.n_views == 0) return DRR_OK;
    if (!(a.step > 0.0f) || !std::isfinite(a.step))
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: step must be a positive finite number");
    if (!a.priority || !a.enabled || !a.world_from_index || !a.source_world || !a.ijk_from_world)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: NULL geometry pointer");
    if (!a.intensity || !a.photon_prob) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: NULL output pointer");
    if (tables->n_materials != set->n_materials)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: tables and volume set disagree on n_materials");
    for (int i = 0; i < set->n_volumes; i++)
        if (a.priority[i] < 0 || a.priority[i] >= set->n_volumes)
            return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: priority outside [0, n_volumes)");
    if ((a.flags & DRR_FLAG_ATTENUATE_OUTSIDE) && (a.air_index < 0 || a.air_index >= set->n_materials))
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: air_index outside [0, n_materials)");
    cudaStream_t s = (cudaStream_t)stream;
    switch (set->n_volumes) {
        case 1: return project_nv<1>(set, tables, a, s);
        case 2: return project_nv<2>(set, tables, a, s);
        case 3: return project_nv<3>(set, tables, a, s);
        default: return project_nv<4>(set, tables, a, s);
    }
}
