// drr_adjoint.cuh -- adjoint of the single-volume forward projection (density and pose gradients).
//
// The reference is not differentiable (README.md:47); this kernel adds the gradients of a loss L
// given dL/d(intensity) and dL/d(photon_prob) per pixel:
//
//   * dL/d(density): the exact adjoint of forward_kernel. A sample at p adds w_t * rho(p) * seg_m(p)
//     to the raw path length of material m, with rho(p) = sum_c W_c rho_c over the texture unit's
//     8-bit corner weights W_c at coordinate p + 0.5 (the staged rule the oracle's
//     hw_corner_weights states). So dL/d(rho_c) = sum over samples of w_t W_c sum_m gr_m seg_m,
//     gr_m = dL/d(raw path length m). Contributions are summed per ray in registers while the
//     sample stays in the same texel cell and added to the gradient volume when it leaves it
//     (adjoint_density_kernel).
//   * dL/d(pose): the derivative of a rigid motion of the volume, theta = (translation t,
//     rotation vector w about `center`, world frame), at theta = 0. Because the filtered density is
//     piecewise constant in p (8-bit weights), the position derivative uses the continuous
//     trilinear interpolation of the same texels and labels: h = w_t (grad rho Q + rho grad Q) with
//     Q the trilinear interpolation of gr over the eight corner labels. With q = A^T h (A the 3x3 of
//     IJK_from_world) and x_t = source + alpha_t r: dL/dt = -sum q, dL/dw = -sum (x_t - center) x q.
//     Changes of the step count and of the entry / exit samples with the pose are not differentiated
//     (adjoint_pose_kernel).
//
// The march reproduces the forward's samples exactly (same float32 alpha sequence, same live step
// range, same trapezoid half weights). Only single-volume projections without air attenuation
// outside the volume are differentiated.
#pragma once

#include "drr_forward.cuh"

namespace drr {

struct AdjointView {
    ViewRec<1> v;
    float source_world[3];
    float pad;
};

struct AdjointParams {
    SceneParams<1> s;                   // outputs of s are unused; tables and the volume are read
    cudaTextureObject_t density_point;  // point-filtered view of the density array
    const AdjointView *views;           // device [n_views]
    int32_t n_views;
    const float *area_density;          // [n][M][H][W] from the forward (g/cm^2)
    const float *grad_intensity;        // [n][H][W] or null
    const float *grad_photon_prob;      // [n][H][W] or null
    const float *grad_area_density;     // [n][M][H][W] or null
    float *grad_density;                // [nk][nj][ni], accumulated into
    float *grad_pose;                   // [n][6] (dL/dt xyz, dL/dw xyz), accumulated into; or null
    float center[3];                    // rotation centre, world
};

// Corner weights of the texture unit for the density coordinate x = p + 0.5 on one axis of n
// texels: texel i0 = fix >> 8, fraction a = fix & 255 (see the oracle's tex_linear). v = 256 x - 128
// is exact wherever it is >= 0 (256 x is exact and 128 a multiple of its ulp, so the fused form
// rounds nothing there); after the unit's own clamp to [0, (n - 1) 256], v is a multiple of 2^-16
// below 2^17, so v + 0.5 is exact and rounding half up is one round-down conversion.
__device__ __forceinline__ void hw_axis(float x, int n, int &i0, int &i1, int &a) {
    float v = __fmaf_rn(x, 256.0f, -128.0f);
    v = fminf(fmaxf(v, 0.0f), (float)(n - 1) * 256.0f);
    const int fix = __float2int_rd(__fadd_rn(v, 0.5f));
    i0 = fix >> 8;
    a = fix & 255;
    i1 = min(i0 + 1, n - 1);
}

__device__ __forceinline__ void hw_weights(int Ax, int Ay, int Az, int W[8]) {
#pragma unroll
    for (int dz = 0; dz <= 1; dz++) {
        const int vz = dz ? Az : 256 - Az;
        const int hx = (vz * Ax + 128) >> 8;
#pragma unroll
        for (int dx = 0; dx <= 1; dx++) {
            const int vx = dx ? hx : vz - hx;
            const int hy = dx ? (vx * Ay + 128) >> 8 : vx - ((vx * (256 - Ay) + 128) >> 8);
            W[dx | 2 | (dz << 2)] = hy;
            W[dx | (dz << 2)] = vx - hy;
        }
    }
}

// Material weight of label L: gr[L].
template <int M>
__device__ __forceinline__ float gr_of(const float gr[M], int L) {
    float v = 0.0f;
#pragma unroll
    for (int m = 0; m < M; m++)
        if (m == L) v = gr[m];
    return v;
}

// Trilinear gradient of eight corner values c = dx | dy << 1 | dz << 2 at fractions (fx, fy, fz).
__device__ __forceinline__ void trilinear_grad(const float v[8], float fx, float fy, float fz, float gx, float gy,
                                               float gz, float d[3]) {
    d[0] = gz * (gy * (v[1] - v[0]) + fy * (v[3] - v[2])) + fz * (gy * (v[5] - v[4]) + fy * (v[7] - v[6]));
    d[1] = gz * (gx * (v[2] - v[0]) + fx * (v[3] - v[1])) + fz * (gx * (v[6] - v[4]) + fx * (v[7] - v[5]));
    d[2] = gy * (gx * (v[4] - v[0]) + fx * (v[5] - v[1])) + fy * (gx * (v[6] - v[2]) + fx * (v[7] - v[3]));
}

__device__ __forceinline__ float trilinear(const float v[8], float fx, float fy, float fz, float gx, float gy,
                                           float gz) {
    return gz * (gy * (gx * v[0] + fx * v[1]) + fy * (gx * v[2] + fx * v[3])) +
           fz * (gy * (gx * v[4] + fx * v[5]) + fy * (gx * v[6] + fx * v[7]));
}

// Per-ray state of both adjoint kernels: the upstream material weights and the forward's march.
template <int M>
struct AdjointRay {
    float gr[M];  // dL/d(raw path length of material m), i.e. dL/d(area density) * step / 10
    float A[9];   // the view's IJK_from_world rotation
    float rx, ry, rz, rxi, ryi, rzi, sx, sy, sz;
    float alpha;
    int t, t_end, num_steps;
};

// Ray setup identical to render_ray's (single volume), done by all 32 lanes of a warp for the same
// ray; the spectral sum for the material weights is split over the lanes. Returns false (for the
// whole warp) when the ray samples nothing or carries no upstream gradient.
template <int M>
__device__ __forceinline__ bool adjoint_setup_warp(const AdjointParams &P, const AdjointView &av, int u, int v, int zv,
                                                   int lane, AdjointRay<M> &R) {
    const SceneParams<1> &p = P.s;
    const ViewRec<1> &view = av.v;
    const VolConst &V = p.vol[0];
    const size_t plane = (size_t)p.width * (size_t)p.height;
    const size_t pix = (size_t)v * p.width + u;
    const int nmat = p.n_materials;
    float ad[M];
#pragma unroll
    for (int m = 0; m < M; m++) {
        const size_t at = ((size_t)zv * nmat + m) * plane + pix;
        ad[m] = m < nmat ? P.area_density[at] : 0.0f;
        R.gr[m] = 0.0f;
    }
    const float gI = P.grad_intensity ? P.grad_intensity[zv * plane + pix] : 0.0f;
    const float gP = P.grad_photon_prob ? P.grad_photon_prob[zv * plane + pix] : 0.0f;
    if (gI != 0.0f || gP != 0.0f) {
        for (int bin = lane; bin < p.n_bins; bin += 32) {
            float x = 0.0f;
#pragma unroll
            for (int m = 0; m < M; m++)
                if (m < nmat) x = __fmaf_rn(ad[m], __ldg(p.mu + bin * nmat + m), x);
            const float e = expf(-x) * __ldg(p.pdf + bin);
            const float d = -(gI * __ldg(p.energies + bin) + gP) * e;  // dL/dx_bin
#pragma unroll
            for (int m = 0; m < M; m++)
                if (m < nmat) R.gr[m] = __fmaf_rn(d, __ldg(p.mu + bin * nmat + m), R.gr[m]);
        }
    }
    const float scale = p.step / 10.0f;  // AD = raw * step / 10
    bool any = false;
#pragma unroll
    for (int m = 0; m < M; m++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) R.gr[m] += __shfl_xor_sync(0xffffffffu, R.gr[m], o);
        const float up = m < nmat && P.grad_area_density != nullptr
                             ? P.grad_area_density[((size_t)zv * nmat + m) * plane + pix]
                             : 0.0f;
        R.gr[m] = (R.gr[m] + up) * scale;
        any |= R.gr[m] != 0.0f;
    }
    if (!any || !V.enabled) return false;
    const float uf = (float)u + 0.5f, vf = (float)v + 0.5f;
    float rx = ray_component(uf, view.w[0], vf, view.w[1], view.w[2]);
    float ry = ray_component(uf, view.w[3], vf, view.w[4], view.w[5]);
    float rz = ray_component(uf, view.w[6], vf, view.w[7], view.w[8]);
    const float ray_length = __fsqrt_rn(__fmaf_rn(rz, rz, __fmaf_rn(rx, rx, __fmul_rn(ry, ry))));
    const float inv_norm = __fdiv_rn(1.0f, ray_length);
    R.rx = __fmul_rn(rx, inv_norm);
    R.ry = __fmul_rn(ry, inv_norm);
    R.rz = __fmul_rn(rz, inv_norm);
#pragma unroll
    for (int k = 0; k < 9; k++) R.A[k] = view.vol[0].a[k];
    R.rxi = dot3(R.A[0], R.rx, R.A[1], R.ry, R.A[2], R.rz);
    R.ryi = dot3(R.A[3], R.rx, R.A[4], R.ry, R.A[5], R.rz);
    R.rzi = dot3(R.A[6], R.rx, R.A[7], R.ry, R.A[8], R.rz);
    R.sx = view.vol[0].s[0];
    R.sy = view.vol[0].s[1];
    R.sz = view.vol[0].s[2];
    const float r3[3] = {R.rxi, R.ryi, R.rzi};
    const float s3[3] = {R.sx, R.sy, R.sz};
    float mn = 0.0f, mx = p.max_ray_length > 0.0f ? p.max_ray_length : __int_as_float(0x7f800000);
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        if (0.0f != r3[ax]) {
            const float reci = __fdiv_rn(1.0f, r3[ax]);
            const float a0 = __fmul_rn(__fsub_rn(-0.5f, s3[ax]), reci);
            const float a1 = __fmul_rn(__fsub_rn(V.hi[ax], s3[ax]), reci);
            mn = fmaxf(mn, fminf(a0, a1));
            mx = fminf(mx, fmaxf(a0, a1));
        } else if (-0.5f > s3[ax] || s3[ax] > V.hi[ax]) {
            return false;
        }
    }
    const float minA = fminf(ray_length, mn);
    const float maxA = fmaxf(0.0f, mx);
    const float span_steps = ceilf(__fdiv_rn(__fsub_rn(maxA, minA), p.step));
    if (!(mn <= mx) || !(span_steps <= (float)kMaxSteps)) return false;
    R.num_steps = (int)span_steps;
    R.alpha = minA;
    R.t = advance_alpha(&R.alpha, p.step, mn, R.num_steps, false);
    float a_end = R.alpha;
    R.t_end = R.t + advance_alpha(&a_end, p.step, mx, R.num_steps - R.t, true);
    return R.t < R.t_end;
}

// First lane of each run of equal keys at or before this lane (keys of a straight ray's cells form
// contiguous runs: a ray never re-enters a cell it has left).
__device__ __forceinline__ int run_start(bool head, int lane) {
    int s = head ? lane : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s = max(s, x);
    }
    return s;
}

// q = sum_m gr_m seg_m(p) for the sample's label word: the derivative of its contribution by its
// filtered density (the material weights need only float32 accuracy here, not the forward's
// rounding order).
template <int M>
__device__ __forceinline__ float material_weight(uint32_t word, const float gr[M], float fx, float fy, float fz) {
    if (uniform_word(word)) return gr_of<M>(gr, (int)(word & 15u));
    const float gx = 1.0f - fx, gy = 1.0f - fy, gz = 1.0f - fz;
    const float xy[4] = {gx * gy, fx * gy, gx * fy, fx * fy};
    float q = 0.0f;
#pragma unroll
    for (int c = 0; c < 8; c++) q += xy[c & 3] * (c >> 2 ? fz : gz) * gr_of<M>(gr, (int)((word >> (4 * c)) & 15u));
    return q;
}

// Density gradient, one warp per ray, lane l on sample t0 + l of each 32-sample chunk: the exact
// transpose of the forward's samples. Each sample adds w_t q_t W_c / 256 to texel c of its
// hardware-filter cell; lanes in the same cell sum their eight values by a segmented warp scan and
// the last lane of each run adds the sums to the gradient volume.
template <int M>
__global__ void __launch_bounds__(256) adjoint_density_kernel(const __grid_constant__ AdjointParams P) {
    const SceneParams<1> &p = P.s;
    const int lane = threadIdx.x & 31;
    const int ray = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int zv = blockIdx.y;
    if (ray >= p.width * p.height || zv >= P.n_views) return;  // whole warps
    const int u = ray % p.width, v = ray / p.width;
    AdjointRay<M> R;
    if (!adjoint_setup_warp<M>(P, P.views[zv], u, v, zv, lane, R)) return;
    const VolConst &V = p.vol[0];
    const int n0 = V.n[0], n1 = V.n[1], n2 = V.n[2];
    const float step = p.step;
    float *const grad = P.grad_density;
    float chunk_alpha = R.alpha;
    for (int t0 = R.t; t0 < R.t_end; t0 += 32) {
        const int t = t0 + lane;
        const float alpha = alpha_after(chunk_alpha, step, lane);
        const float wt = t >= R.t_end ? 0.0f : ((0 == t || R.num_steps - 1 == t) ? 0.5f : 1.0f);
        const float px = __fsub_rn(__fmaf_rn(alpha, R.rxi, R.sx), 1.0f);
        const float py = __fsub_rn(__fmaf_rn(alpha, R.ryi, R.sy), 1.0f);
        const float pz = __fsub_rn(__fmaf_rn(alpha, R.rzi, R.sz), 1.0f);
        const float bx = floorf(px), by = floorf(py), bz = floorf(pz);
        const uint32_t word = fetch_label_word(V, bx, by, bz);
        const float q = material_weight<M>(word, R.gr, px - bx, py - by, pz - bz);
        int i0, i1, ax_, j0, j1, ay_, k0, k1, az_;
        hw_axis(__fadd_rn(px, 0.5f), n0, i0, i1, ax_);
        hw_axis(__fadd_rn(py, 0.5f), n1, j0, j1, ay_);
        hw_axis(__fadd_rn(pz, 0.5f), n2, k0, k1, az_);
        int W[8];
        hw_weights(ax_, ay_, az_, W);
        const float r = wt * q * (1.0f / 256.0f);
        float c8[8];
#pragma unroll
        for (int c = 0; c < 8; c++) c8[c] = r * (float)W[c];
        // runs of lanes in the same filter cell
        const int pi = __shfl_up_sync(0xffffffffu, i0, 1), pj = __shfl_up_sync(0xffffffffu, j0, 1),
                  pk = __shfl_up_sync(0xffffffffu, k0, 1);
        const bool head = lane == 0 || pi != i0 || pj != j0 || pk != k0;
        const int s = run_start(head, lane);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const float x = __shfl_up_sync(0xffffffffu, c8[c], o);
                if (lane - o >= s) c8[c] += x;
            }
        }
        const bool next_head = __shfl_down_sync(0xffffffffu, head ? 1 : 0, 1) != 0;
        if (lane == 31 || next_head) {
            const int is[2] = {i0, i1}, js[2] = {j0, j1}, ks[2] = {k0, k1};
#pragma unroll
            for (int c = 0; c < 8; c++)
                if (c8[c] != 0.0f) atomicAdd(grad + ((size_t)ks[c >> 2] * n1 + js[(c >> 1) & 1]) * n0 + is[c & 1], c8[c]);
        }
        chunk_alpha = __fadd_rn(__shfl_sync(0xffffffffu, alpha, 31), step);
    }
}

// Pose gradient, one warp per ray as above: h = d/dp of w_t rho(p) Q(p) with rho and Q the
// continuous trilinear interpolants of the label cell's texels and per-corner material weights.
// The first lane of each run of lanes in one label cell fetches the cell's eight texels; shuffles
// hand them to the run. h and alpha h are summed in IJK space and rotated to the world once.
template <int M>
__global__ void __launch_bounds__(256) adjoint_pose_kernel(const __grid_constant__ AdjointParams P) {
    __shared__ float s_pose[8][6];
    const SceneParams<1> &p = P.s;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int ray = blockIdx.x * 8 + wib;
    const int zv = blockIdx.y;
    float pose[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    AdjointRay<M> R;
    if (ray < p.width * p.height && zv < P.n_views &&
        adjoint_setup_warp<M>(P, P.views[zv], ray % p.width, ray / p.width, zv, lane, R)) {
        const VolConst &V = p.vol[0];
        const float step = p.step;
        float Hi[3] = {0.f, 0.f, 0.f}, Ki[3] = {0.f, 0.f, 0.f};
        float chunk_alpha = R.alpha;
        for (int t0 = R.t; t0 < R.t_end; t0 += 32) {
            const int t = t0 + lane;
            const float alpha = alpha_after(chunk_alpha, step, lane);
            const float wt = t >= R.t_end ? 0.0f : ((0 == t || R.num_steps - 1 == t) ? 0.5f : 1.0f);
            const float px = __fsub_rn(__fmaf_rn(alpha, R.rxi, R.sx), 1.0f);
            const float py = __fsub_rn(__fmaf_rn(alpha, R.ryi, R.sy), 1.0f);
            const float pz = __fsub_rn(__fmaf_rn(alpha, R.rzi, R.sz), 1.0f);
            const float bx = floorf(px), by = floorf(py), bz = floorf(pz);
            const float fx = px - bx, fy = py - by, fz = pz - bz;
            const float gx = 1.0f - fx, gy = 1.0f - fy, gz = 1.0f - fz;
            const float qx = __shfl_up_sync(0xffffffffu, bx, 1), qy = __shfl_up_sync(0xffffffffu, by, 1),
                        qz = __shfl_up_sync(0xffffffffu, bz, 1);
            const bool head = lane == 0 || qx != bx || qy != by || qz != bz;
            const int s = run_start(head, lane);
            float rho8[8];
#pragma unroll
            for (int c = 0; c < 8; c++) {
                float r = 0.0f;
                if (head)
                    r = tex3D<float>(P.density_point, bx + (float)(c & 1) + 0.5f, by + (float)((c >> 1) & 1) + 0.5f,
                                     bz + (float)(c >> 2) + 0.5f);
                rho8[c] = __shfl_sync(0xffffffffu, r, s);
            }
            const uint32_t word = fetch_label_word(V, bx, by, bz);
            float dr[3];
            trilinear_grad(rho8, fx, fy, fz, gx, gy, gz, dr);
            float h[3];
            if (uniform_word(word)) {
                const float wQ = wt * gr_of<M>(R.gr, (int)(word & 15u));
                h[0] = wQ * dr[0], h[1] = wQ * dr[1], h[2] = wQ * dr[2];
            } else {
                float g8[8];
#pragma unroll
                for (int c = 0; c < 8; c++) g8[c] = gr_of<M>(R.gr, (int)((word >> (4 * c)) & 15u));
                float dQ[3];
                trilinear_grad(g8, fx, fy, fz, gx, gy, gz, dQ);
                const float rho = trilinear(rho8, fx, fy, fz, gx, gy, gz);
                const float Q = trilinear(g8, fx, fy, fz, gx, gy, gz);
                h[0] = wt * (dr[0] * Q + rho * dQ[0]);
                h[1] = wt * (dr[1] * Q + rho * dQ[1]);
                h[2] = wt * (dr[2] * Q + rho * dQ[2]);
            }
#pragma unroll
            for (int k = 0; k < 3; k++) {
                Hi[k] += h[k];
                Ki[k] = __fmaf_rn(alpha, h[k], Ki[k]);
            }
            chunk_alpha = __fadd_rn(__shfl_sync(0xffffffffu, alpha, 31), step);
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                Hi[k] += __shfl_xor_sync(0xffffffffu, Hi[k], o);
                Ki[k] += __shfl_xor_sync(0xffffffffu, Ki[k], o);
            }
        }
        float Hw[3], K[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            Hw[k] = R.A[k] * Hi[0] + R.A[3 + k] * Hi[1] + R.A[6 + k] * Hi[2];
            K[k] = R.A[k] * Ki[0] + R.A[3 + k] * Ki[1] + R.A[6 + k] * Ki[2];
        }
        const float d[3] = {P.views[zv].source_world[0] - P.center[0], P.views[zv].source_world[1] - P.center[1],
                            P.views[zv].source_world[2] - P.center[2]};
        const float rr[3] = {R.rx, R.ry, R.rz};
        pose[0] = -Hw[0];
        pose[1] = -Hw[1];
        pose[2] = -Hw[2];
        pose[3] = -((d[1] * Hw[2] - d[2] * Hw[1]) + (rr[1] * K[2] - rr[2] * K[1]));
        pose[4] = -((d[2] * Hw[0] - d[0] * Hw[2]) + (rr[2] * K[0] - rr[0] * K[2]));
        pose[5] = -((d[0] * Hw[1] - d[1] * Hw[0]) + (rr[0] * K[1] - rr[1] * K[0]));
    }
    // one ray per warp: lane 0 holds its ray's terms; sum the block's eight rays, one atomic each
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 6; k++) s_pose[wib][k] = pose[k];
    }
    __syncthreads();
    if (threadIdx.x < 6 && zv < P.n_views) {
        float x = 0.0f;
        for (int w = 0; w < 8; w++) x += s_pose[w][threadIdx.x];
        if (x != 0.0f) atomicAdd(P.grad_pose + (size_t)zv * 6 + threadIdx.x, x);
    }
}

template <int M>
cudaError_t launch_adjoint(const AdjointParams &p, cudaStream_t stream);

}  // namespace drr
