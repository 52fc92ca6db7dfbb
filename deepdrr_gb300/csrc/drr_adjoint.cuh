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

// Ray setup identical to render_ray's (single volume): returns false when the ray samples nothing
// or carries no upstream gradient.
template <int M>
__device__ __forceinline__ bool adjoint_setup(const AdjointParams &P, const AdjointView &av, int u, int v, int zv,
                                              AdjointRay<M> &R) {
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
        R.gr[m] = m < nmat && P.grad_area_density != nullptr ? P.grad_area_density[at] : 0.0f;
    }
    const float gI = P.grad_intensity ? P.grad_intensity[zv * plane + pix] : 0.0f;
    const float gP = P.grad_photon_prob ? P.grad_photon_prob[zv * plane + pix] : 0.0f;
    if (gI != 0.0f || gP != 0.0f) {
        for (int bin = 0; bin < p.n_bins; bin++) {
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
        R.gr[m] *= scale;
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
    // the rotation in registers: the kernels' atomics could alias the view records as far as the
    // compiler knows, so reads through the pointer would repeat per sample
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

// Density gradient: the exact transpose of the forward's samples. Each sample adds
// w_t q_t W_c / 256 to texel c of its hardware-filter cell (q_t = sum_m gr_m seg_m). While the cell
// and w_t q_t stay the same the integer weights W_c are summed and converted once; the cell's eight
// sums are added to the gradient volume when the ray leaves it.
template <int M>
__global__ void __launch_bounds__(kBlockThreads) adjoint_density_kernel(const __grid_constant__ AdjointParams P) {
    const SceneParams<1> &p = P.s;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int u = blockIdx.x * kTileW + ((warp & 1) << 3) + (lane & 7);
    const int v = blockIdx.y * kTileH + ((warp >> 1) << 2) + (lane >> 3);
    const int zv = blockIdx.z;
    if (u >= p.width || v >= p.height || zv >= P.n_views) return;
    AdjointRay<M> R;
    if (!adjoint_setup<M>(P, P.views[zv], u, v, zv, R)) return;
    const VolConst &V = p.vol[0];
    const int n0 = V.n[0], n1 = V.n[1], n2 = V.n[2];
    const float step = p.step;
    float *const grad = P.grad_density;
    float alpha = R.alpha;
    // label words are loaded one step ahead (as in the forward) so no lane branches to fetch them;
    // the material weight of a uniform cell is cached while the label stays the same
    int cur_label = -1;
    float cur_g = 0.0f;
    // hardware-filter cell and its sums
    int ci = -1, cj = 0, ck = 0, ci1 = 0, cj1 = 0, ck1 = 0;
    float acc[8];
    int iw[8];
#pragma unroll
    for (int c = 0; c < 8; c++) acc[c] = 0.0f, iw[c] = 0;
    float run = 0.0f;  // w_t q_t / 256 of the integer sums in iw
    auto fold = [&]() {
#pragma unroll
        for (int c = 0; c < 8; c++) {
            acc[c] = __fmaf_rn(run, (float)iw[c], acc[c]);
            iw[c] = 0;
        }
    };
    auto flush = [&]() {
        fold();
        const int is[2] = {ci, ci1}, js[2] = {cj, cj1}, ks[2] = {ck, ck1};
#pragma unroll
        for (int c = 0; c < 8; c++) {
            if (acc[c] != 0.0f) atomicAdd(grad + ((size_t)ks[c >> 2] * n1 + js[(c >> 1) & 1]) * n0 + is[c & 1], acc[c]);
            acc[c] = 0.0f;
        }
    };
    float cx = __fsub_rn(__fmaf_rn(alpha, R.rxi, R.sx), 1.0f);
    float cy = __fsub_rn(__fmaf_rn(alpha, R.ryi, R.sy), 1.0f);
    float cz = __fsub_rn(__fmaf_rn(alpha, R.rzi, R.sz), 1.0f);
    float cbx = floorf(cx), cby = floorf(cy), cbz = floorf(cz);
    uint32_t w_cur = fetch_label_word(V, cbx, cby, cbz);
    for (int t = R.t; t < R.t_end; ++t) {
        const float wt = (0 == t || R.num_steps - 1 == t) ? 0.5f : 1.0f;
        const float an = __fadd_rn(alpha, step);
        const float nx = __fsub_rn(__fmaf_rn(an, R.rxi, R.sx), 1.0f);
        const float ny = __fsub_rn(__fmaf_rn(an, R.ryi, R.sy), 1.0f);
        const float nz = __fsub_rn(__fmaf_rn(an, R.rzi, R.sz), 1.0f);
        const float nbx = floorf(nx), nby = floorf(ny), nbz = floorf(nz);
        const uint32_t w_next = fetch_label_word(V, nbx, nby, nbz);
        const float px = cx, py = cy, pz = cz;
        const uint32_t word = w_cur;
        float q;
        if (uniform_word(word)) {
            const int L = (int)(word & 15u);
            if (L != cur_label) {
                cur_label = L;
                cur_g = gr_of<M>(R.gr, L);
            }
            q = cur_g;
        } else {
            const CornerWeights cw = corner_weights(__fsub_rn(px, cbx), __fsub_rn(py, cby), __fsub_rn(pz, cbz));
            const uint32_t A = word & 15u;
            const uint32_t xa = word ^ (A * 0x11111111u);
            const uint32_t B = (word >> ((__ffs(xa) - 1) & ~3)) & 15u;
            const uint32_t xb = word ^ (B * 0x11111111u);
            const uint32_t za = ~(((xa & 0x77777777u) + 0x77777777u) | xa) & 0x88888888u;
            const uint32_t zb = ~(((xb & 0x77777777u) + 0x77777777u) | xb) & 0x88888888u;
            if ((za | zb) == 0x88888888u) {
                float sA = 0.0f, sB = 0.0f;
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    const float w = __fmul_rn(cw.xy[c & 3], cw.z[c >> 2]);
                    if ((za >> (4 * c + 3)) & 1u)
                        sA += w;
                    else
                        sB += w;
                }
                q = __fmaf_rn(sA, gr_of<M>(R.gr, (int)A), sB * gr_of<M>(R.gr, (int)B));
            } else {
                q = 0.0f;
#pragma unroll
                for (int c = 0; c < 8; c++)
                    q = __fmaf_rn(__fmul_rn(cw.xy[c & 3], cw.z[c >> 2]), gr_of<M>(R.gr, (int)((word >> (4 * c)) & 15u)),
                                  q);
            }
        }
        int i0, i1, ax_, j0, j1, ay_, k0, k1, az_;
        hw_axis(__fadd_rn(px, 0.5f), n0, i0, i1, ax_);
        hw_axis(__fadd_rn(py, 0.5f), n1, j0, j1, ay_);
        hw_axis(__fadd_rn(pz, 0.5f), n2, k0, k1, az_);
        if (i0 != ci || j0 != cj || k0 != ck) {
            if (ci >= 0) flush();
            ci = i0, cj = j0, ck = k0, ci1 = i1, cj1 = j1, ck1 = k1;
        }
        const float r = wt * q * (1.0f / 256.0f);
        if (r != run) {
            fold();
            run = r;
        }
        int W[8];
        hw_weights(ax_, ay_, az_, W);
#pragma unroll
        for (int c = 0; c < 8; c++) iw[c] += W[c];
        alpha = an;
        cx = nx, cy = ny, cz = nz, cbx = nbx, cby = nby, cbz = nbz;
        w_cur = w_next;
    }
    if (ci >= 0) flush();
}

// Pose gradient: d/dp of w_t rho(p) Q(p) with rho and Q the continuous trilinear interpolants of the
// label cell's texels and per-corner material weights, summed as q_w = A^T h (Hw) and alpha q_w (K).
// In a cell whose eight labels agree Q is constant and grad rho is bilinear in the fractions, so the
// cell's samples are summed as weighted moments of the fractions and turned into h when the ray
// leaves the cell; mixed cells are evaluated per sample.
template <int M>
__global__ void __launch_bounds__(kBlockThreads) adjoint_pose_kernel(const __grid_constant__ AdjointParams P) {
    const SceneParams<1> &p = P.s;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int u = blockIdx.x * kTileW + ((warp & 1) << 3) + (lane & 7);
    const int v = blockIdx.y * kTileH + ((warp >> 1) << 2) + (lane >> 3);
    const int zv = blockIdx.z;
    const bool active = u < p.width && v < p.height && zv < P.n_views;
    float pose[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    AdjointRay<M> R;
    if (active && adjoint_setup<M>(P, P.views[zv], u, v, zv, R)) {
        const VolConst &V = p.vol[0];
        const float step = p.step;
        float alpha = R.alpha;
        float pb0 = __int_as_float(0x7fc00000), pb1 = pb0, pb2 = pb0;
        bool uni = false;
        float gu = 0.0f, g8[8], rho8[8];
#pragma unroll
        for (int c = 0; c < 8; c++) g8[c] = rho8[c] = 0.0f;
        // moments of the current uniform cell: sum w, w f_x, w f_y, w f_z, w f_x f_y, w f_x f_z,
        // w f_y f_z, and the same weighted by alpha
        float m[7], n[7];
#pragma unroll
        for (int k = 0; k < 7; k++) m[k] = n[k] = 0.0f;
        // sums of h and alpha h in IJK space; the world-space q = A^T h is applied once per ray
        float Hi[3] = {0.f, 0.f, 0.f}, Ki[3] = {0.f, 0.f, 0.f};
        auto add_world = [&](float hx, float hy, float hz, float kx, float ky, float kz) {
            Hi[0] += hx, Hi[1] += hy, Hi[2] += hz;
            Ki[0] += kx, Ki[1] += ky, Ki[2] += kz;
        };
        auto flush_moments = [&]() {
            if (m[0] == 0.0f) return;
            const float *r = rho8;
            const float dx0 = r[1] - r[0], dx1 = r[3] - r[2], dx2 = r[5] - r[4], dx3 = r[7] - r[6];
            const float dy0 = r[2] - r[0], dy1 = r[3] - r[1], dy2 = r[6] - r[4], dy3 = r[7] - r[5];
            const float dz0 = r[4] - r[0], dz1 = r[5] - r[1], dz2 = r[6] - r[2], dz3 = r[7] - r[3];
            // d rho / d f_x = dx0 + (dx1 - dx0) f_y + (dx2 - dx0) f_z + (dx0 - dx1 - dx2 + dx3) f_y f_z, etc.
            auto gsum = [&](const float *s) {
                float g[3];
                g[0] = dx0 * s[0] + (dx1 - dx0) * s[2] + (dx2 - dx0) * s[3] + (dx0 - dx1 - dx2 + dx3) * s[6];
                g[1] = dy0 * s[0] + (dy1 - dy0) * s[1] + (dy2 - dy0) * s[3] + (dy0 - dy1 - dy2 + dy3) * s[5];
                g[2] = dz0 * s[0] + (dz1 - dz0) * s[1] + (dz2 - dz0) * s[2] + (dz0 - dz1 - dz2 + dz3) * s[4];
                return make_float3(g[0] * gu, g[1] * gu, g[2] * gu);
            };
            const float3 h = gsum(m), hk = gsum(n);
            add_world(h.x, h.y, h.z, hk.x, hk.y, hk.z);
#pragma unroll
            for (int k = 0; k < 7; k++) m[k] = n[k] = 0.0f;
        };
        for (int t = R.t; t < R.t_end; ++t) {
            const float wt = (0 == t || R.num_steps - 1 == t) ? 0.5f : 1.0f;
            const float px = __fsub_rn(__fmaf_rn(alpha, R.rxi, R.sx), 1.0f);
            const float py = __fsub_rn(__fmaf_rn(alpha, R.ryi, R.sy), 1.0f);
            const float pz = __fsub_rn(__fmaf_rn(alpha, R.rzi, R.sz), 1.0f);
            const float bx = floorf(px), by = floorf(py), bz = floorf(pz);
            const float fx = __fsub_rn(px, bx), fy = __fsub_rn(py, by), fz = __fsub_rn(pz, bz);
            if (bx != pb0 || by != pb1 || bz != pb2) {
                if (uni) flush_moments();
                const uint32_t word = fetch_label_word(V, bx, by, bz);
                uni = uniform_word(word);
                gu = gr_of<M>(R.gr, (int)(word & 15u));
                if (!uni) {
#pragma unroll
                    for (int c = 0; c < 8; c++) g8[c] = gr_of<M>(R.gr, (int)((word >> (4 * c)) & 15u));
                }
#pragma unroll
                for (int c = 0; c < 8; c++)
                    rho8[c] = tex3D<float>(P.density_point, bx + (float)(c & 1) + 0.5f,
                                           by + (float)((c >> 1) & 1) + 0.5f, bz + (float)(c >> 2) + 0.5f);
                pb0 = bx, pb1 = by, pb2 = bz;
            }
            if (uni) {
                if (gu != 0.0f) {
                    const float wa = wt * alpha;
                    const float fxy = fx * fy, fxz = fx * fz, fyz = fy * fz;
                    m[0] += wt, m[1] += wt * fx, m[2] += wt * fy, m[3] += wt * fz;
                    m[4] += wt * fxy, m[5] += wt * fxz, m[6] += wt * fyz;
                    n[0] += wa, n[1] += wa * fx, n[2] += wa * fy, n[3] += wa * fz;
                    n[4] += wa * fxy, n[5] += wa * fxz, n[6] += wa * fyz;
                }
            } else {
                const float gx = 1.0f - fx, gy = 1.0f - fy, gz = 1.0f - fz;
                float dr[3], dQ[3];
                trilinear_grad(rho8, fx, fy, fz, gx, gy, gz, dr);
                trilinear_grad(g8, fx, fy, fz, gx, gy, gz, dQ);
                const float rho = trilinear(rho8, fx, fy, fz, gx, gy, gz);
                const float Q = trilinear(g8, fx, fy, fz, gx, gy, gz);
                const float hx = wt * (dr[0] * Q + rho * dQ[0]);
                const float hy = wt * (dr[1] * Q + rho * dQ[1]);
                const float hz = wt * (dr[2] * Q + rho * dQ[2]);
                add_world(hx, hy, hz, alpha * hx, alpha * hy, alpha * hz);
            }
            alpha = __fadd_rn(alpha, step);
        }
        if (uni) flush_moments();
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
    if (zv < P.n_views) {
        // one view per block: reduce over the warp, then one atomic per warp and component
#pragma unroll
        for (int k = 0; k < 6; k++) {
            float x = pose[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0 && x != 0.0f) atomicAdd(P.grad_pose + (size_t)zv * 6 + k, x);
        }
    }
}

template <int M>
cudaError_t launch_adjoint(const AdjointParams &p, cudaStream_t stream);

}  // namespace drr
