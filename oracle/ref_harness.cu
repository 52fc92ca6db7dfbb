// ref_harness.cu -- drives the reference projector kernel on the GPU (TEST INFRASTRUCTURE ONLY).
//
// The reference's `projectKernel` (deepdrr/projector/project_kernel.cu:135-650) is compiled from
// the reference sources into oracle/_ref/*.cubin by oracle/build_ref.py. This harness loads such a
// cubin with the CUDA driver API and reproduces what deepdrr's host does around it:
//   * textures exactly as create_cuda_texture makes them (projector.py:116-257): a 1-channel
//     cudaArray of extent (ni, nj, nk); float32 density with linear filtering; uint8 labels with
//     point filtering; clamp addressing; unnormalised coordinates; element-type reads;
//   * the argument list of _render_single (projector.py:718-756): IJK boxes [-0.5, n-0.5]
//     (projector.py:1626-1634), mesh buffers present but disabled (mesh_sub_layer_valid = 0);
//   * 8 x 8 thread blocks, one launch per view (projector.py:759-774);
//   * the column-major output (img_dx = u * H + v) transposed to [H][W] (projector.py:786-792).
// It also exposes a texture-filter probe used to pin the oracle's emulation of the texture unit.
// Only the tests and the CPU/GPU reference comparisons load this library.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;

int set_err(const std::string &s) {
    g_err = s;
    return -1;
}

#define RT(x)                                                                                       \
    do {                                                                                            \
        cudaError_t e_ = (x);                                                                       \
        if (e_ != cudaSuccess) return set_err(std::string(#x) + ": " + cudaGetErrorString(e_));     \
    } while (0)

#define DRV(x)                                                                                      \
    do {                                                                                            \
        CUresult r_ = (x);                                                                          \
        if (r_ != CUDA_SUCCESS) {                                                                   \
            const char *s_ = nullptr;                                                               \
            cuGetErrorString(r_, &s_);                                                              \
            return set_err(std::string(#x) + ": " + (s_ ? s_ : "?"));                               \
        }                                                                                           \
    } while (0)

struct Tex {
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
};

int make_tex(const void *host, int elem, cudaChannelFormatKind kind, bool linear, int ni, int nj, int nk, Tex *out) {
    cudaChannelFormatDesc fd = cudaCreateChannelDesc(elem * 8, 0, 0, 0, kind);
    cudaExtent ext = make_cudaExtent(ni, nj, nk);
    RT(cudaMalloc3DArray(&out->arr, &fd, ext, 0));
    cudaMemcpy3DParms cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.srcPtr = make_cudaPitchedPtr(const_cast<void *>(host), (size_t)ni * elem, ni, nj);
    cp.dstArray = out->arr;
    cp.extent = ext;
    cp.kind = cudaMemcpyHostToDevice;
    RT(cudaMemcpy3D(&cp));
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = out->arr;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.filterMode = linear ? cudaFilterModeLinear : cudaFilterModePoint;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    RT(cudaCreateTextureObject(&out->tex, &rd, &td, nullptr));
    return 0;
}

void free_tex(Tex &t) {
    if (t.tex) cudaDestroyTextureObject(t.tex);
    if (t.arr) cudaFreeArray(t.arr);
    t = Tex();
}

template <typename T>
int upload(const T *host, size_t n, T **dev, std::vector<void *> &owned) {
    RT(cudaMalloc((void **)dev, sizeof(T) * (n ? n : 1)));
    owned.push_back(*dev);
    if (n) RT(cudaMemcpy(*dev, host, sizeof(T) * n, cudaMemcpyHostToDevice));
    else RT(cudaMemset(*dev, 0, sizeof(T)));
    return 0;
}

__global__ void probe_linear(cudaTextureObject_t tex, const float *__restrict__ xyz, int n, float *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = tex3D<float>(tex, xyz[3 * i + 0], xyz[3 * i + 1], xyz[3 * i + 2]);
}

__global__ void probe_point(cudaTextureObject_t tex, const float *__restrict__ xyz, int n, float *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)tex3D<unsigned char>(tex, xyz[3 * i + 0], xyz[3 * i + 1], xyz[3 * i + 2]);
}

}  // namespace

extern "C" {

const char *ref_last_error(void) { return g_err.c_str(); }

// Run the reference kernel from `cubin_path` on one view. Host inputs; per-volume arrays are
// [nk][nj][ni]. Outputs are host [H][W]. `repeats` extra timed launches report the mean kernel
// time in *ms_out (CUDA events on the launch stream). Returns 0 or -1 (see ref_last_error).
int ref_project(const char *cubin_path, int n_volumes, int n_materials, const float *const *density,
                const uint8_t *const *labels, const int *dims, const int *priority, const int *enabled,
                const float *world_from_index, const float *ijk_from_world, const float *source_ijk,
                float max_ray_length, float step, int width, int height, int n_bins, const float *energies,
                const float *pdf, const float *mu, int want_solid_angle, float *intensity_out, float *photon_out,
                float *solid_angle_out, int repeats, float *ms_out) {
    RT(cudaFree(0));  // make the primary context current for the driver API
    CUmodule mod = nullptr;
    CUfunction fn = nullptr;
    DRV(cuModuleLoad(&mod, cubin_path));
    CUresult fr = cuModuleGetFunction(&fn, mod, "projectKernel");
    if (fr != CUDA_SUCCESS) {
        cuModuleUnload(mod);
        return set_err("projectKernel not found in cubin");
    }
    std::vector<Tex> dens(n_volumes), labs(n_volumes);
    std::vector<void *> owned;
    int rc = 0;
    auto cleanup = [&]() {
        for (auto &t : dens) free_tex(t);
        for (auto &t : labs) free_tex(t);
        for (void *p : owned) cudaFree(p);
        cuModuleUnload(mod);
    };
    std::vector<unsigned long long> dtex(n_volumes), ltex(n_volumes);
    std::vector<float> minp(n_volumes, -0.5f), maxx(n_volumes), maxy(n_volumes), maxz(n_volumes), vs(n_volumes, 1.0f);
    std::vector<float> sx(n_volumes), sy(n_volumes), sz(n_volumes);
    for (int i = 0; i < n_volumes && rc == 0; i++) {
        int ni = dims[3 * i], nj = dims[3 * i + 1], nk = dims[3 * i + 2];
        rc = make_tex(density[i], 4, cudaChannelFormatKindFloat, true, ni, nj, nk, &dens[i]);
        if (rc == 0) rc = make_tex(labels[i], 1, cudaChannelFormatKindUnsigned, false, ni, nj, nk, &labs[i]);
        dtex[i] = dens[i].tex;
        ltex[i] = labs[i].tex;
        maxx[i] = (float)(ni - 0.5);
        maxy[i] = (float)(nj - 0.5);
        maxz[i] = (float)(nk - 0.5);
        sx[i] = source_ijk[3 * i];
        sy[i] = source_ijk[3 * i + 1];
        sz[i] = source_ijk[3 * i + 2];
    }
    if (rc) {
        cleanup();
        return rc;
    }
    unsigned long long *d_dtex, *d_ltex;
    int *d_prio, *d_en, *d_umat;
    float *d_minx, *d_miny, *d_minz, *d_maxx, *d_maxy, *d_maxz, *d_vsx, *d_vsy, *d_vsz, *d_sx, *d_sy, *d_sz;
    float *d_w, *d_ijk, *d_e, *d_pdf, *d_mu, *d_int, *d_pp, *d_sa = nullptr, *d_alpha, *d_add;
    int8_t *d_facing, *d_valid;
    const size_t npix = (size_t)width * height;
    std::vector<int8_t> zeros8(2, 0);
    std::vector<float> zf(2, 0.f);
    std::vector<int8_t> zf8(2, 0);
    std::vector<int> zi(1, 0);
    if (upload(dtex.data(), n_volumes, &d_dtex, owned) || upload(ltex.data(), n_volumes, &d_ltex, owned) ||
        upload(priority, n_volumes, &d_prio, owned) || upload(enabled, n_volumes, &d_en, owned) ||
        upload(minp.data(), n_volumes, &d_minx, owned) || upload(minp.data(), n_volumes, &d_miny, owned) ||
        upload(minp.data(), n_volumes, &d_minz, owned) || upload(maxx.data(), n_volumes, &d_maxx, owned) ||
        upload(maxy.data(), n_volumes, &d_maxy, owned) || upload(maxz.data(), n_volumes, &d_maxz, owned) ||
        upload(vs.data(), n_volumes, &d_vsx, owned) || upload(vs.data(), n_volumes, &d_vsy, owned) ||
        upload(vs.data(), n_volumes, &d_vsz, owned) || upload(sx.data(), n_volumes, &d_sx, owned) ||
        upload(sy.data(), n_volumes, &d_sy, owned) || upload(sz.data(), n_volumes, &d_sz, owned) ||
        upload(world_from_index, 9, &d_w, owned) || upload(ijk_from_world, (size_t)12 * n_volumes, &d_ijk, owned) ||
        upload(energies, n_bins, &d_e, owned) || upload(pdf, n_bins, &d_pdf, owned) ||
        upload(mu, (size_t)n_bins * n_materials, &d_mu, owned) || upload(zf.data(), 2, &d_alpha, owned) ||
        upload(zf8.data(), 2, &d_facing, owned) || upload(zeros8.data(), 2, &d_valid, owned) ||
        upload(zf.data(), 2, &d_add, owned) || upload(zi.data(), 1, &d_umat, owned)) {
        cleanup();
        return -1;
    }
    if (cudaMalloc(&d_int, npix * 4) != cudaSuccess || (owned.push_back(d_int), false) ||
        cudaMalloc(&d_pp, npix * 4) != cudaSuccess || (owned.push_back(d_pp), false)) {
        cleanup();
        return set_err("cudaMalloc outputs");
    }
    if (want_solid_angle) {
        if (cudaMalloc(&d_sa, npix * 4) != cudaSuccess) {
            cleanup();
            return set_err("cudaMalloc solid angle");
        }
        owned.push_back(d_sa);
    }
    int W = width, H = height, nb = n_bins, nu = 0, offw = 0, offh = 0;
    float st = step, mrl = max_ray_length;
    void *args[] = {&d_dtex, &d_ltex, &W, &H, &st, &d_prio, &d_en, &d_minx, &d_miny, &d_minz, &d_maxx,
                    &d_maxy, &d_maxz, &d_vsx, &d_vsy, &d_vsz, &d_sx, &d_sy, &d_sz, &mrl, &d_w, &d_ijk,
                    &nb, &d_e, &d_pdf, &d_mu, &d_int, &d_pp, &d_sa, &d_alpha, &d_facing, &d_valid, &d_add,
                    &d_umat, &nu, &offw, &offh};
    const unsigned gx = (width + 7) / 8, gy = (height + 7) / 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    CUresult lr = cuLaunchKernel(fn, gx, gy, 1, 8, 8, 1, 0, nullptr, args, nullptr);
    if (lr == CUDA_SUCCESS && repeats > 0) {
        cudaEventRecord(e0, 0);
        for (int r = 0; r < repeats && lr == CUDA_SUCCESS; r++)
            lr = cuLaunchKernel(fn, gx, gy, 1, 8, 8, 1, 0, nullptr, args, nullptr);
        cudaEventRecord(e1, 0);
    }
    cudaError_t se = cudaDeviceSynchronize();
    if (lr != CUDA_SUCCESS || se != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cleanup();
        return set_err(std::string("reference kernel launch failed: ") + cudaGetErrorString(se));
    }
    if (repeats > 0 && ms_out) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        *ms_out = ms / repeats;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::vector<float> colmajor(npix);
    auto fetch = [&](float *dev, float *out) -> int {
        if (!out) return 0;
        RT(cudaMemcpy(colmajor.data(), dev, npix * 4, cudaMemcpyDeviceToHost));
        for (int u = 0; u < width; u++)
            for (int v = 0; v < height; v++) out[(size_t)v * width + u] = colmajor[(size_t)u * height + v];
        return 0;
    };
    rc = fetch(d_int, intensity_out);
    if (!rc) rc = fetch(d_pp, photon_out);
    if (!rc && d_sa) rc = fetch(d_sa, solid_angle_out);
    cleanup();
    return rc;
}

// Fetch a 3D texture built from `host` ([nk][nj][ni]) at n coordinates xyz[3n] (unnormalised).
// kind 0: float32 texture, linear filtering; 1: uint8 texture, point filtering; 2: float16 texture
// (host holds uint16 half bits), linear filtering.
int ref_probe_texture(int kind, const void *host, int ni, int nj, int nk, const float *xyz, int n, float *out) {
    RT(cudaFree(0));
    Tex t;
    int rc = kind == 1 ? make_tex(host, 1, cudaChannelFormatKindUnsigned, false, ni, nj, nk, &t)
                       : make_tex(host, kind == 2 ? 2 : 4, cudaChannelFormatKindFloat, true, ni, nj, nk, &t);
    if (rc) {
        free_tex(t);
        return rc;
    }
    float *d_xyz = nullptr, *d_out = nullptr;
    if (cudaMalloc(&d_xyz, sizeof(float) * 3 * (size_t)n) != cudaSuccess ||
        cudaMalloc(&d_out, sizeof(float) * (size_t)n) != cudaSuccess) {
        cudaFree(d_xyz);
        free_tex(t);
        return set_err("cudaMalloc probe");
    }
    cudaMemcpy(d_xyz, xyz, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice);
    if (kind == 1) probe_point<<<(n + 255) / 256, 256>>>(t.tex, d_xyz, n, d_out);
    else probe_linear<<<(n + 255) / 256, 256>>>(t.tex, d_xyz, n, d_out);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(out, d_out, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d_xyz);
    cudaFree(d_out);
    free_tex(t);
    if (e != cudaSuccess) return set_err(std::string("probe: ") + cudaGetErrorString(e));
    return 0;
}

}  // extern "C"
