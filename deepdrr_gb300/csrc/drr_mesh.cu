// drr_mesh.cu -- additive triangle meshes: per-pixel path integrals by CUDA rasterisation.
//
// Replaces the additive part of the reference's OpenGL mesh path: the DRRMode.DENSITY pass of
// pyrenderdrr/renderer.py (shaders/density.frag:9-13 with additive blending, renderer.py:420-435),
// read back per layer and material (projector.py:1063-1088, 1302-1330) and added to the path
// lengths in project_kernel.cu:569-579. For each pixel and mesh material the shader pass sums over
// every triangle the pixel's centre ray crosses (distance from the source times the signed face
// orientation times the material's density, and the signed orientation alone); the kernel adds
// max(sum, 0) to the material's path length (mm g/cm^3, before the division by 10) where the
// orientations balance (a closed surface crossed in and out).
//
// Here each triangle is rasterised in the detector's index space, as a GPU rasteriser does it:
// vertices snapped to 1/256 pixel, coverage of pixel centres by exact 64-bit edge functions with a
// top-left rule for ties, so a ray through an edge or vertex shared by two triangles counts once
// and closed surfaces balance exactly. The distance is the float64 ray-plane intersection along the
// unit ray of the pixel (the projector's own ray), the orientation the sign of the ray against the
// triangle's right-handed normal (+1 leaving, -1 entering). Sums are float64 atomics.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/drr_gb300.h"
#include "drr_internal.h"

using drr::cuda_fail;
using drr::fail;

namespace {

struct RasterView {
    double winv[9];  // inverse of the ray matrix W: index-space homogeneous coordinates of x - source
    double w[9];     // W: ray(u, v) = W [u + 0.5, v + 0.5, 1]
    double src[3];
    int width, height;
};

// image coordinates farther than this from the detector are not rasterised (keeps the 64-bit edge
// functions exact: snapped coordinates stay below 2^28, products below 2^58)
constexpr double kMaxImageCoord = 1.0e6;

__device__ __forceinline__ bool top_left(long long dx, long long dy) { return dy > 0 || (dy == 0 && dx < 0); }

// Subtractive hit lists of one view: per layer and pixel up to max_hits (distance, facing) pairs,
// facing +1 entering and -1 leaving, sorted by distance, facing 0 after the last hit.
struct HitLists {
    float *alpha;          // [n_layers][H][W][max_hits]
    int8_t *facing;        // [n_layers][H][W][max_hits]
    unsigned int *count;   // [n_layers][H][W] (building only)
    int n_layers, max_hits;
};

enum { kModeAdditive = 1, kModeSubtractive = 2 };

// density_between.frag: an additive crossing at distance d (sign +1 leaving, -1 entering) against the
// subtractive pair [near, far] adds sign * rho * (far - max(d, near)) for d < far; summed over a
// closed additive surface this removes rho times the overlap of its interior with [near, far].
__device__ __forceinline__ double between(double d, double near, double far) {
    if (d < near) return far - near;
    if (d < far) return far - d;
    return 0.0;
}

// pass 0: additive integrals (with subtraction by the hit lists of higher layers when given);
// pass 1: append subtractive crossings to the hit lists
__global__ void rasterize_kernel(const float *__restrict__ tri, const int32_t *__restrict__ slot,
                                 const float *__restrict__ density, const int32_t *__restrict__ layer,
                                 const uint8_t *__restrict__ mode, int n_tri, RasterView view, double *R, double *G,
                                 int n_slots, HitLists hits, int pass) {
    const int lane = threadIdx.x & 31;
    const int warps_per_block = blockDim.x >> 5;
    const size_t plane = (size_t)view.width * view.height;
    for (int f = blockIdx.x * warps_per_block + (threadIdx.x >> 5); f < n_tri; f += gridDim.x * warps_per_block) {
        double P[3][3], S[3][2];
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const double x = tri[(size_t)f * 9 + 3 * k] - view.src[0];
            const double y = tri[(size_t)f * 9 + 3 * k + 1] - view.src[1];
            const double z = tri[(size_t)f * 9 + 3 * k + 2] - view.src[2];
            P[k][0] = x + view.src[0];
            P[k][1] = y + view.src[1];
            P[k][2] = z + view.src[2];
            const double qx = view.winv[0] * x + view.winv[1] * y + view.winv[2] * z;
            const double qy = view.winv[3] * x + view.winv[4] * y + view.winv[5] * z;
            const double qz = view.winv[6] * x + view.winv[7] * y + view.winv[8] * z;
            if (!(qz > 1e-9)) ok = false;  // at or behind the source plane: not rasterised
            S[k][0] = qx / qz;
            S[k][1] = qy / qz;
            if (!(fabs(S[k][0]) < kMaxImageCoord && fabs(S[k][1]) < kMaxImageCoord)) ok = false;
        }
        if (!ok) continue;
        long long X[3], Y[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            X[k] = llrint(S[k][0] * 256.0);
            Y[k] = llrint(S[k][1] * 256.0);
        }
        long long area = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0]);
        if (area == 0) continue;
        int o1 = 1, o2 = 2;  // vertex order with positive area for the coverage test
        if (area < 0) o1 = 2, o2 = 1;
        const long long ax = X[0], ay = Y[0], bx = X[o1], by = Y[o1], cx = X[o2], cy = Y[o2];
        // bounding box of pixel centres 256 u + 128
        const long long xmin = min(ax, min(bx, cx)), xmax = max(ax, max(bx, cx));
        const long long ymin = min(ay, min(by, cy)), ymax = max(ay, max(by, cy));
        long long u0 = (xmin - 128 + 255) >> 8, u1 = (xmax - 128) >> 8;
        long long v0 = (ymin - 128 + 255) >> 8, v1 = (ymax - 128) >> 8;
        u0 = max(u0, 0LL), v0 = max(v0, 0LL);
        u1 = min(u1, (long long)view.width - 1), v1 = min(v1, (long long)view.height - 1);
        if (u0 > u1 || v0 > v1) continue;
        // right-handed normal of the triangle as given (outward for a consistently wound surface)
        const double e1[3] = {P[1][0] - P[0][0], P[1][1] - P[0][1], P[1][2] - P[0][2]};
        const double e2[3] = {P[2][0] - P[0][0], P[2][1] - P[0][1], P[2][2] - P[0][2]};
        const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double np = n[0] * (P[0][0] - view.src[0]) + n[1] * (P[0][1] - view.src[1]) + n[2] * (P[0][2] - view.src[2]);
        const double rho = density[f];
        const int s = slot[f];
        const int lay = layer ? layer[f] : 0;
        const int md = mode ? mode[f] : kModeAdditive;
        if (pass == 0 && (!(md & kModeAdditive) || s < 0 || s >= n_slots)) continue;
        if (pass == 1 && (!(md & kModeSubtractive) || lay < 0 || lay >= hits.n_layers)) continue;
        const long long nu = u1 - u0 + 1, count = nu * (v1 - v0 + 1);
        for (long long idx = lane; idx < count; idx += 32) {
            const long long u = u0 + idx % nu, v = v0 + idx / nu;
            const long long px = 256 * u + 128, py = 256 * v + 128;
            const long long e_ab = (bx - ax) * (py - ay) - (by - ay) * (px - ax);
            const long long e_bc = (cx - bx) * (py - by) - (cy - by) * (px - bx);
            const long long e_ca = (ax - cx) * (py - cy) - (ay - cy) * (px - cx);
            const bool in = (e_ab > 0 || (e_ab == 0 && top_left(bx - ax, by - ay))) &&
                            (e_bc > 0 || (e_bc == 0 && top_left(cx - bx, cy - by))) &&
                            (e_ca > 0 || (e_ca == 0 && top_left(ax - cx, ay - cy)));
            if (!in) continue;
            const double fu = (double)u + 0.5, fv = (double)v + 0.5;
            double r[3];
#pragma unroll
            for (int k = 0; k < 3; k++) r[k] = view.w[3 * k] * fu + view.w[3 * k + 1] * fv + view.w[3 * k + 2];
            const double len = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            const double nr = (n[0] * r[0] + n[1] * r[1] + n[2] * r[2]) / len;
            if (nr == 0.0) continue;  // ray in the triangle's plane
            const double dist = np / nr;
            const double sign = nr > 0.0 ? 1.0 : -1.0;
            const size_t pix = (size_t)v * view.width + (size_t)u;
            if (pass == 1) {
                const size_t lp = (size_t)lay * plane + pix;
                const unsigned int k = atomicAdd(hits.count + lp, 1u);
                if ((int)k < hits.max_hits) {
                    hits.alpha[lp * hits.max_hits + k] = (float)dist;
                    hits.facing[lp * hits.max_hits + k] = sign > 0.0 ? (int8_t)-1 : (int8_t)1;
                }
                continue;
            }
            double r_add = sign * dist * rho;
            for (int L = lay + 1; L < hits.n_layers; L++) {
                const size_t base = ((size_t)L * plane + pix) * hits.max_hits;
                for (int i = 0; i + 1 < hits.max_hits; i += 2) {
                    if (hits.facing[base + i] == 0 || hits.facing[base + i + 1] == 0) break;
                    r_add += sign * rho * between(dist, hits.alpha[base + i], hits.alpha[base + i + 1]);
                }
            }
            const size_t o = (size_t)s * plane + pix;
            atomicAdd(R + o, r_add);
            atomicAdd(G + o, sign);
        }
    }
}

// order each pixel's subtractive crossings by distance (insertion sort of at most max_hits) and
// end the list with facing 0
__global__ void sort_hits_kernel(HitLists hits, size_t n_lists) {
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n_lists; l += (size_t)gridDim.x * blockDim.x) {
        float *a = hits.alpha + l * hits.max_hits;
        int8_t *f = hits.facing + l * hits.max_hits;
        const int n = min((int)hits.count[l], hits.max_hits);
        for (int i = 1; i < n; i++) {
            const float ai = a[i];
            const int8_t fi = f[i];
            int j = i - 1;
            while (j >= 0 && a[j] > ai) {
                a[j + 1] = a[j];
                f[j + 1] = f[j];
                --j;
            }
            a[j + 1] = ai;
            f[j + 1] = fi;
        }
        for (int i = n; i < hits.max_hits; i++) {
            a[i] = 0.0f;
            f[i] = 0;
        }
    }
}

// project_kernel.cu:573-577: the sum counts where the orientations balance, never below zero
__global__ void mesh_finalize_kernel(const double *R, const double *G, size_t n, float *out) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float r = (float)R[i], g = (float)G[i];
        out[i] = fabsf(g) < 0.00001f ? fmaxf(r, 0.0f) : 0.0f;
    }
}

bool invert3(const double *a, double *inv) {
    const double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                       a[2] * (a[3] * a[7] - a[4] * a[6]);
    if (!(det != 0.0) || !std::isfinite(det)) return false;
    const double id = 1.0 / det;
    inv[0] = (a[4] * a[8] - a[5] * a[7]) * id;
    inv[1] = (a[2] * a[7] - a[1] * a[8]) * id;
    inv[2] = (a[1] * a[5] - a[2] * a[4]) * id;
    inv[3] = (a[5] * a[6] - a[3] * a[8]) * id;
    inv[4] = (a[0] * a[8] - a[2] * a[6]) * id;
    inv[5] = (a[2] * a[3] - a[0] * a[5]) * id;
    inv[6] = (a[3] * a[7] - a[4] * a[6]) * id;
    inv[7] = (a[1] * a[6] - a[0] * a[7]) * id;
    inv[8] = (a[0] * a[4] - a[1] * a[3]) * id;
    return true;
}

}  // namespace

namespace {

drr_status check_mesh(const drr_mesh_desc *mesh, const char *who) {
    if (!mesh) return fail(DRR_ERR_INVALID_ARGUMENT, std::string(who) + ": NULL mesh");
    if (mesh->n_slots < 1 || mesh->n_slots > DRR_MAX_MATERIALS)
        return fail(DRR_ERR_INVALID_ARGUMENT, std::string(who) + ": n_slots outside [1, DRR_MAX_MATERIALS]");
    if (mesh->n_triangles < 0 || (mesh->n_triangles > 0 && (!mesh->triangles || !mesh->slot || !mesh->density)))
        return fail(DRR_ERR_INVALID_ARGUMENT, std::string(who) + ": bad triangle arrays");
    if (mesh->n_layers < 0 || mesh->n_layers > DRR_MAX_MESH_LAYERS)
        return fail(DRR_ERR_INVALID_ARGUMENT, std::string(who) + ": n_layers outside [0, DRR_MAX_MESH_LAYERS]");
    return DRR_OK;
}

bool make_view(const double *world_from_index, const double *source_world, int v, int width, int height,
               RasterView &rv) {
    std::memcpy(rv.w, world_from_index + (size_t)v * 9, sizeof(rv.w));
    std::memcpy(rv.src, source_world + (size_t)v * 3, sizeof(rv.src));
    rv.width = width;
    rv.height = height;
    return invert3(rv.w, rv.winv);
}

int raster_blocks(int n_tri) { return (int)std::min<long long>(((long long)n_tri + 7) / 8, 65535LL * 4); }

}  // namespace

extern "C" drr_status drr_mesh_hits(const drr_mesh_desc *mesh, int32_t width, int32_t height,
                                    const double *world_from_index, const double *source_world, int32_t max_hits,
                                    float *hit_alpha, int8_t *hit_facing, void *stream) {
    drr::set_last_error("");
    drr_status st = check_mesh(mesh, "drr_mesh_hits");
    if (st != DRR_OK) return st;
    if (!world_from_index || !source_world || !hit_alpha || !hit_facing)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_mesh_hits: NULL argument");
    if (width < 1 || height < 1) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_mesh_hits: bad size");
    if (max_hits < 2 || max_hits > 256 || (max_hits & 1))
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_mesh_hits: max_hits must be even, in [2, 256]");
    if (mesh->n_layers < 1) return DRR_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t plane = (size_t)width * height, lists = plane * mesh->n_layers;
    RasterView rv;
    if (!make_view(world_from_index, source_world, 0, width, height, rv))
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_mesh_hits: singular world_from_index");
    HitLists h{hit_alpha, hit_facing, nullptr, mesh->n_layers, max_hits};
    cudaError_t e = cudaMallocAsync((void **)&h.count, lists * sizeof(unsigned int), s);
    if (e != cudaSuccess) return cuda_fail(e, "drr_mesh_hits: scratch");
    e = cudaMemsetAsync(h.count, 0, lists * sizeof(unsigned int), s);
    if (e == cudaSuccess && mesh->n_triangles > 0) {
        rasterize_kernel<<<raster_blocks(mesh->n_triangles), 256, 0, s>>>(
            mesh->triangles, mesh->slot, mesh->density, mesh->layer, mesh->mode, mesh->n_triangles, rv, nullptr,
            nullptr, mesh->n_slots, h, 1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        const size_t nb = (lists + 255) / 256;
        sort_hits_kernel<<<(unsigned)(nb < 4864 ? nb : 4864), 256, 0, s>>>(h, lists);
        e = cudaGetLastError();
    }
    cudaFreeAsync(h.count, s);
    if (e != cudaSuccess) return cuda_fail(e, "drr_mesh_hits");
    return DRR_OK;
}

extern "C" drr_status drr_mesh_area_density(const drr_mesh_desc *mesh, int32_t width, int32_t height,
                                            int32_t n_views, const double *world_from_index,
                                            const double *source_world, const float *hit_alpha,
                                            const int8_t *hit_facing, int32_t max_hits, float *out, void *stream) {
    drr::set_last_error("");
    drr_status st = check_mesh(mesh, "drr_mesh_area_density");
    if (st != DRR_OK) return st;
    if (!world_from_index || !source_world || !out)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_mesh_area_density: NULL argument");
    if (width < 1 || height < 1 || n_views < 0) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_mesh_area_density: bad size");
    if (hit_alpha && (n_views != 1 || !hit_facing || max_hits < 2 || (max_hits & 1)))
        return fail(DRR_ERR_INVALID_ARGUMENT,
                    "drr_mesh_area_density: hit lists need one view, facings and an even max_hits >= 2");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t plane = (size_t)width * height, per_view = plane * mesh->n_slots;
    if (n_views == 0) return DRR_OK;
    double *R = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&R, 2 * per_view * sizeof(double), s);
    if (e != cudaSuccess) return cuda_fail(e, "drr_mesh_area_density: scratch");
    double *G = R + per_view;
    HitLists h{const_cast<float *>(hit_alpha), const_cast<int8_t *>(hit_facing), nullptr,
               hit_alpha ? mesh->n_layers : 0, hit_alpha ? max_hits : 0};
    for (int v = 0; v < n_views && e == cudaSuccess; v++) {
        RasterView rv;
        if (!make_view(world_from_index, source_world, v, width, height, rv)) {
            cudaFreeAsync(R, s);
            return fail(DRR_ERR_INVALID_ARGUMENT, "drr_mesh_area_density: singular world_from_index");
        }
        e = cudaMemsetAsync(R, 0, 2 * per_view * sizeof(double), s);
        if (e == cudaSuccess && mesh->n_triangles > 0) {
            rasterize_kernel<<<raster_blocks(mesh->n_triangles), 256, 0, s>>>(
                mesh->triangles, mesh->slot, mesh->density, mesh->layer, mesh->mode, mesh->n_triangles, rv, R, G,
                mesh->n_slots, h, 0);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            const size_t nb = (per_view + 255) / 256;
            mesh_finalize_kernel<<<(unsigned)(nb < 4864 ? nb : 4864), 256, 0, s>>>(R, G, per_view,
                                                                                 out + (size_t)v * per_view);
            e = cudaGetLastError();
        }
    }
    cudaFreeAsync(R, s);
    if (e != cudaSuccess) return cuda_fail(e, "drr_mesh_area_density");
    return DRR_OK;
}
