// ref_harness.cu -- drives the reference projector kernel on the GPU (TEST AND BASELINE
// INFRASTRUCTURE ONLY).
//
// The reference's `projectKernel` (deepdrr/projector/project_kernel.cu:135-650) is compiled from
// the reference sources into oracle/_ref/*.cubin by oracle/build_ref.py. This harness loads such a
// cubin with the CUDA driver API and reproduces what deepdrr's host does around it:
//   * textures exactly as create_cuda_texture makes them (projector.py:116-257): a 1-channel
//     cudaArray of extent (ni, nj, nk); float32 density with linear filtering; uint8 labels with
//     point filtering; clamp addressing; unnormalised coordinates; element-type reads;
//   * the argument list of _render_single (projector.py:718-756): IJK boxes [-0.5, n-0.5]
//     (projector.py:1626-1634); mesh buffers either disabled (mesh_sub_layer_valid = 0, no additive
//     densities) or given by the caller in the reference's layouts;
//   * 8 x 8 thread blocks, one launch per view (projector.py:759-774);
//   * the column-major output (img_dx = u * H + v) transposed to [H][W] (projector.py:786-792).
// A scene (textures and tables) is created once and renders any number of views, as one
// Projector does after initialize(). Kernel time is measured with CUDA events on the launch
// stream; the host time of the whole per-view sequence (geometry upload, launch, both read-backs
// and the transposes, the work of _render_single) is measured with a steady clock.
// It also exposes a texture-filter probe used to pin the oracle's emulation of the texture unit.
// Only the tests and bench.py's reference-kernel baseline load this library.
#include <cuda.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

// MESH_LAYERS and MAX_MESH_HITS the cubins are compiled with (oracle/build_ref.py)
constexpr int kMeshLayers = 2;
constexpr int kMaxMeshHits = 32;

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

// A device buffer the scene owns, grown on demand.
struct DevBuf {
    void *ptr = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes) {
        if (bytes <= cap) return 0;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        RT(cudaMalloc(&ptr, bytes));
        cap = bytes;
        return 0;
    }
    int upload(const void *host, size_t bytes) {
        if (ensure(bytes ? bytes : 16)) return -1;
        if (bytes) RT(cudaMemcpy(ptr, host, bytes, cudaMemcpyHostToDevice));
        else RT(cudaMemset(ptr, 0, 16));
        return 0;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
    }
};

struct RefScene {
    CUmodule mod = nullptr;
    CUfunction fn = nullptr;
    int nv = 0, M = 0, n_bins = 0;
    std::vector<Tex> dens, labs;
    // per-scene constants (projector.py:1546-1686)
    DevBuf dtex, ltex, prio, en, minx, miny, minz, maxx, maxy, maxz, vsx, vsy, vsz, e, pdf, mu;
    // per-view inputs (_update_object_locations, projector.py:802-831) and outputs
    DevBuf sx, sy, sz, w, ijk, out_int, out_pp, out_sa;
    // mesh buffers (projector.py:1055-1330); 1-element dummies when no mesh is given
    DevBuf hit_alpha, hit_facing, layer_valid, additive, umat;
    std::vector<float> colmajor;

    void release() {
        for (auto &t : dens) free_tex(t);
        for (auto &t : labs) free_tex(t);
        DevBuf *all[] = {&dtex, &ltex, &prio, &en, &minx, &miny, &minz, &maxx, &maxy, &maxz, &vsx, &vsy, &vsz,
                         &e, &pdf, &mu, &sx, &sy, &sz, &w, &ijk, &out_int, &out_pp, &out_sa, &hit_alpha,
                         &hit_facing, &layer_valid, &additive, &umat};
        for (DevBuf *b : all) b->release();
        if (mod) cuModuleUnload(mod);
        mod = nullptr;
    }
};

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

// Load the reference kernel from `cubin_path` and build its textures and tables, as
// Projector.initialize does. Host inputs; per-volume arrays are [nk][nj][ni]. Returns 0 and a
// handle in *out, or -1 (see ref_last_error).
int ref_scene_create(const char *cubin_path, int n_volumes, int n_materials, const float *const *density,
                     const uint8_t *const *labels, const int *dims, const int *priority, const int *enabled,
                     int n_bins, const float *energies, const float *pdf, const float *mu, void **out) {
    *out = nullptr;
    RT(cudaFree(0));  // make the primary context current for the driver API
    RefScene *s = new RefScene();
    s->nv = n_volumes;
    s->M = n_materials;
    s->n_bins = n_bins;
    auto bail = [&](int rc) {
        s->release();
        delete s;
        return rc;
    };
    CUresult lr = cuModuleLoad(&s->mod, cubin_path);
    if (lr != CUDA_SUCCESS) {
        s->mod = nullptr;
        return bail(set_err(std::string("cuModuleLoad failed: ") + cubin_path));
    }
    if (cuModuleGetFunction(&s->fn, s->mod, "projectKernel") != CUDA_SUCCESS)
        return bail(set_err("projectKernel not found in cubin"));
    s->dens.resize(n_volumes);
    s->labs.resize(n_volumes);
    std::vector<unsigned long long> dtex(n_volumes), ltex(n_volumes);
    std::vector<float> minp(n_volumes, -0.5f), maxx(n_volumes), maxy(n_volumes), maxz(n_volumes), vs(n_volumes, 1.0f);
    for (int i = 0; i < n_volumes; i++) {
        int ni = dims[3 * i], nj = dims[3 * i + 1], nk = dims[3 * i + 2];
        if (make_tex(density[i], 4, cudaChannelFormatKindFloat, true, ni, nj, nk, &s->dens[i]) ||
            make_tex(labels[i], 1, cudaChannelFormatKindUnsigned, false, ni, nj, nk, &s->labs[i]))
            return bail(-1);
        dtex[i] = s->dens[i].tex;
        ltex[i] = s->labs[i].tex;
        maxx[i] = (float)(ni - 0.5);
        maxy[i] = (float)(nj - 0.5);
        maxz[i] = (float)(nk - 0.5);
    }
    const size_t fv = sizeof(float) * n_volumes;
    if (s->dtex.upload(dtex.data(), 8 * (size_t)n_volumes) || s->ltex.upload(ltex.data(), 8 * (size_t)n_volumes) ||
        s->prio.upload(priority, sizeof(int) * n_volumes) || s->en.upload(enabled, sizeof(int) * n_volumes) ||
        s->minx.upload(minp.data(), fv) || s->miny.upload(minp.data(), fv) || s->minz.upload(minp.data(), fv) ||
        s->maxx.upload(maxx.data(), fv) || s->maxy.upload(maxy.data(), fv) || s->maxz.upload(maxz.data(), fv) ||
        s->vsx.upload(vs.data(), fv) || s->vsy.upload(vs.data(), fv) || s->vsz.upload(vs.data(), fv) ||
        s->e.upload(energies, sizeof(float) * n_bins) || s->pdf.upload(pdf, sizeof(float) * n_bins) ||
        s->mu.upload(mu, sizeof(float) * (size_t)n_bins * n_materials))
        return bail(-1);
    *out = s;
    return 0;
}

void ref_scene_destroy(void *handle) {
    RefScene *s = static_cast<RefScene *>(handle);
    if (!s) return;
    s->release();
    delete s;
}

// Render one view. world_from_index [9], ijk_from_world [nv][12] and source_ijk [nv][3] are the
// float32 values _update_object_locations uploads. Optional subtractive-mesh hit lists
// (hit_alpha float / hit_facing int8, [2][H][W][32], with layer_valid int8 [2]) and additive
// densities (float [2][n_umat][H][W][2]: signed sum and crossing balance, with unique_materials
// int [n_umat]) are passed in the reference's layouts; NULL disables them. Outputs are host [H][W]
// (NULL: not read back). After one untimed launch, `repeats` more launches report their mean
// kernel time in *ms_out; *wall_ms_out (if non-NULL) receives the host time of one whole
// _render_single sequence: geometry upload, launch, synchronisation, read-back of intensity and
// photon_prob, and their transposes.
int ref_scene_project(void *handle, const float *world_from_index, const float *ijk_from_world,
                      const float *source_ijk, float max_ray_length, float step, int width, int height,
                      int want_solid_angle, const float *hit_alpha, const int8_t *hit_facing,
                      const int8_t *layer_valid, const float *additive, const int *unique_materials, int n_umat,
                      float *intensity_out, float *photon_out, float *solid_angle_out, int repeats, float *ms_out,
                      float *wall_ms_out) {
    RefScene *s = static_cast<RefScene *>(handle);
    if (!s) return set_err("null scene");
    const int nv = s->nv;
    const size_t npix = (size_t)width * height;
    std::vector<float> sx(nv), sy(nv), sz(nv);
    for (int i = 0; i < nv; i++) {
        sx[i] = source_ijk[3 * i];
        sy[i] = source_ijk[3 * i + 1];
        sz[i] = source_ijk[3 * i + 2];
    }
    auto upload_geometry = [&]() -> int {
        const size_t fv = sizeof(float) * nv;
        if (s->sx.upload(sx.data(), fv) || s->sy.upload(sy.data(), fv) || s->sz.upload(sz.data(), fv) ||
            s->w.upload(world_from_index, sizeof(float) * 9) || s->ijk.upload(ijk_from_world, fv * 12))
            return -1;
        return 0;
    };
    if (upload_geometry()) return -1;
    if (s->out_int.ensure(npix * 4) || s->out_pp.ensure(npix * 4)) return -1;
    if (want_solid_angle && s->out_sa.ensure(npix * 4)) return -1;
    const int8_t no_layers[kMeshLayers] = {0, 0};
    const size_t hits = (size_t)kMeshLayers * npix * kMaxMeshHits;
    if (hit_alpha && hit_facing && layer_valid) {
        if (s->hit_alpha.upload(hit_alpha, hits * 4) || s->hit_facing.upload(hit_facing, hits) ||
            s->layer_valid.upload(layer_valid, kMeshLayers))
            return -1;
    } else {
        const float zf[2] = {0.f, 0.f};
        const int8_t z8[2] = {0, 0};
        if (s->hit_alpha.upload(zf, 8) || s->hit_facing.upload(z8, 2) || s->layer_valid.upload(no_layers, kMeshLayers))
            return -1;
    }
    int nu = 0;
    if (additive && unique_materials && n_umat > 0) {
        if (s->additive.upload(additive, sizeof(float) * kMeshLayers * (size_t)n_umat * npix * 2) ||
            s->umat.upload(unique_materials, sizeof(int) * n_umat))
            return -1;
        nu = n_umat;
    } else {
        const float zf[2] = {0.f, 0.f};
        const int zi[1] = {0};
        if (s->additive.upload(zf, 8) || s->umat.upload(zi, 4)) return -1;
    }
    int W = width, H = height, nb = s->n_bins, offw = 0, offh = 0;
    float st = step, mrl = max_ray_length;
    void *d_sa = want_solid_angle ? s->out_sa.ptr : nullptr;
    void *args[] = {&s->dtex.ptr, &s->ltex.ptr, &W, &H, &st, &s->prio.ptr, &s->en.ptr, &s->minx.ptr,
                    &s->miny.ptr, &s->minz.ptr, &s->maxx.ptr, &s->maxy.ptr, &s->maxz.ptr, &s->vsx.ptr,
                    &s->vsy.ptr, &s->vsz.ptr, &s->sx.ptr, &s->sy.ptr, &s->sz.ptr, &mrl, &s->w.ptr, &s->ijk.ptr,
                    &nb, &s->e.ptr, &s->pdf.ptr, &s->mu.ptr, &s->out_int.ptr, &s->out_pp.ptr, &d_sa,
                    &s->hit_alpha.ptr, &s->hit_facing.ptr, &s->layer_valid.ptr, &s->additive.ptr, &s->umat.ptr,
                    &nu, &offw, &offh};
    const unsigned gx = (width + 7) / 8, gy = (height + 7) / 8;
    auto launch = [&]() { return cuLaunchKernel(s->fn, gx, gy, 1, 8, 8, 1, 0, nullptr, args, nullptr); };
    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0));
    RT(cudaEventCreate(&e1));
    CUresult lr = launch();
    if (lr == CUDA_SUCCESS && repeats > 0) {
        cudaEventRecord(e0, 0);
        for (int r = 0; r < repeats && lr == CUDA_SUCCESS; r++) lr = launch();
        cudaEventRecord(e1, 0);
    }
    cudaError_t se = cudaDeviceSynchronize();
    if (lr != CUDA_SUCCESS || se != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return set_err(std::string("reference kernel launch failed: ") + cudaGetErrorString(se));
    }
    if (repeats > 0 && ms_out) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        *ms_out = ms / repeats;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s->colmajor.resize(npix);
    auto fetch = [&](void *dev, float *out) -> int {
        if (!out) return 0;
        RT(cudaMemcpy(s->colmajor.data(), dev, npix * 4, cudaMemcpyDeviceToHost));
        for (int u = 0; u < width; u++)
            for (int v = 0; v < height; v++) out[(size_t)v * width + u] = s->colmajor[(size_t)u * height + v];
        return 0;
    };
    if (fetch(s->out_int.ptr, intensity_out) || fetch(s->out_pp.ptr, photon_out)) return -1;
    if (want_solid_angle && fetch(s->out_sa.ptr, solid_angle_out)) return -1;
    if (wall_ms_out) {
        // one more view the way _render_single runs it, timed on the host
        std::vector<float> a(npix), b(npix);
        const auto t0 = std::chrono::steady_clock::now();
        if (upload_geometry()) return -1;
        lr = launch();
        se = cudaDeviceSynchronize();
        if (lr != CUDA_SUCCESS || se != cudaSuccess)
            return set_err(std::string("reference kernel launch failed: ") + cudaGetErrorString(se));
        if (fetch(s->out_int.ptr, a.data()) || fetch(s->out_pp.ptr, b.data())) return -1;
        const auto t1 = std::chrono::steady_clock::now();
        *wall_ms_out = (float)std::chrono::duration<double, std::milli>(t1 - t0).count();
    }
    return 0;
}

// One scene, one view: ref_scene_create + ref_scene_project + ref_scene_destroy.
int ref_project(const char *cubin_path, int n_volumes, int n_materials, const float *const *density,
                const uint8_t *const *labels, const int *dims, const int *priority, const int *enabled,
                const float *world_from_index, const float *ijk_from_world, const float *source_ijk,
                float max_ray_length, float step, int width, int height, int n_bins, const float *energies,
                const float *pdf, const float *mu, int want_solid_angle, float *intensity_out, float *photon_out,
                float *solid_angle_out, int repeats, float *ms_out) {
    void *h = nullptr;
    if (ref_scene_create(cubin_path, n_volumes, n_materials, density, labels, dims, priority, enabled, n_bins,
                         energies, pdf, mu, &h))
        return -1;
    int rc = ref_scene_project(h, world_from_index, ijk_from_world, source_ijk, max_ray_length, step, width, height,
                               want_solid_angle, nullptr, nullptr, nullptr, nullptr, nullptr, 0, intensity_out,
                               photon_out, solid_angle_out, repeats, ms_out, nullptr);
    ref_scene_destroy(h);
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
