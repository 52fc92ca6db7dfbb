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
//     sample stays in the same texel cell and added to the gradient volume when it leaves it.
//   * dL/d(pose): the derivative of a rigid motion of the volume, theta = (translation t,
//     rotation vector w about `center`, world frame), at theta = 0. Because the filtered density is
//     piecewise constant in p (8-bit weights), the position derivative uses the continuous
//     trilinear interpolation of the same texels and labels: h = w_t (grad rho Q + rho grad Q) with
//     Q the trilinear interpolation of gr over the eight corner labels. With q = A^T h (A the 3x3 of
//     IJK_from_world) and x_t = source + alpha_t r: dL/dt = -sum q, dL/dw = -sum (x_t - center) x q.
//     Changes of the step count and of the entry / exit samples with the pose are not differentiated.
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
// texels: texel i0 = fix >> 8, fraction a = fix & 255 (see the oracle's tex_linear).
__device__ __forceinline__ void hw_axis(float x, int n, int &i0, int &i1, int &a) {
    // (x - 0.5) * 256 is exact wherever it is >= 0 (x * 256 is exact and 128 a multiple of its ulp,
    // so the fused form rounds nothing there);
    // the clamp to [0, (n - 1) * 256] is the unit's own, and round-half-up is done without a
    // rounding addition.
    float v = __fmaf_rn(x, 256.0f, -128.0f);
    v = fminf(fmaxf(v, 0.0f), (float)(n - 1) * 256.0f);
    const float fl = floorf(v);
    const int fix = (int)fl + (__fsub_rn(v, fl) >= 0.5f ? 1 : 0);
    i0 = fix >> 8;
    a = fix & 255;
    i1 = i0 + 1 < n ? i0 + 1 : n - 1;
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

// Material weight of each of the eight corners of a label word: gr[label of corner c].
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

template <int M, bool POSE>
__global__ void __launch_bounds__(kBlockThreads) adjoint_kernel(const __grid_constant__ AdjointParams P) {
    const SceneParams<1> &p = P.s;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int u = blockIdx.x * kTileW + ((warp & 1) << 3) + (lane & 7);
    const int v = blockIdx.y * kTileH + ((warp >> 1) << 2) + (lane >> 3);
    const int zv = blockIdx.z;
    const bool active = u < p.width && v < p.height && zv < P.n_views;
    float pose[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (active) {
        const AdjointView &av = P.views[zv];
        const ViewRec<1> &view = av.v;
        const VolConst &V = p.vol[0];
        const size_t plane = (size_t)p.width * (size_t)p.height;
        const size_t pix = (size_t)v * p.width + u;
        const int nmat = p.n_materials;
        const float step = p.step;

        // dL/d(raw path length) per material from the forward's area densities
        float ad[M], gr[M];
#pragma unroll
        for (int m = 0; m < M; m++) {
            const size_t at = ((size_t)zv * nmat + m) * plane + pix;
            ad[m] = m < nmat ? P.area_density[at] : 0.0f;
            gr[m] = m < nmat && P.grad_area_density != nullptr ? P.grad_area_density[at] : 0.0f;
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
                    if (m < nmat) gr[m] = __fmaf_rn(d, __ldg(p.mu + bin * nmat + m), gr[m]);
            }
        }
        const float scale = step / 10.0f;  // AD = raw * step / 10
        bool any = false;
#pragma unroll
        for (int m = 0; m < M; m++) {
            gr[m] *= scale;
            any |= gr[m] != 0.0f;
        }

        // ray setup and live step range: identical to render_ray
        const float uf = (float)u + 0.5f, vf = (float)v + 0.5f;
        float rx = ray_component(uf, view.w[0], vf, view.w[1], view.w[2]);
        float ry = ray_component(uf, view.w[3], vf, view.w[4], view.w[5]);
        float rz = ray_component(uf, view.w[6], vf, view.w[7], view.w[8]);
        const float ray_length = __fsqrt_rn(__fmaf_rn(rz, rz, __fmaf_rn(rx, rx, __fmul_rn(ry, ry))));
        const float inv_norm = __fdiv_rn(1.0f, ray_length);
        rx = __fmul_rn(rx, inv_norm);
        ry = __fmul_rn(ry, inv_norm);
        rz = __fmul_rn(rz, inv_norm);
        // the view's IJK_from_world rotation in registers: the loop's atomics could alias the view
        // records as far as the compiler knows, so reads through the pointer would repeat per sample
        float A[9];
#pragma unroll
        for (int k = 0; k < 9; k++) A[k] = view.vol[0].a[k];
        const float rxi = dot3(A[0], rx, A[1], ry, A[2], rz);
        const float ryi = dot3(A[3], rx, A[4], ry, A[5], rz);
        const float rzi = dot3(A[6], rx, A[7], ry, A[8], rz);
        const float r3[3] = {rxi, ryi, rzi};
        float mn = 0.0f, mx = p.max_ray_length > 0.0f ? p.max_ray_length : __int_as_float(0x7f800000);
        bool ok = V.enabled != 0 && any;
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            const float s = view.vol[0].s[ax];
            if (!ok) break;
            if (0.0f != r3[ax]) {
                const float reci = __fdiv_rn(1.0f, r3[ax]);
                const float a0 = __fmul_rn(__fsub_rn(-0.5f, s), reci);
                const float a1 = __fmul_rn(__fsub_rn(V.hi[ax], s), reci);
                mn = fmaxf(mn, fminf(a0, a1));
                mx = fminf(mx, fmaxf(a0, a1));
            } else if (-0.5f > s || s > V.hi[ax]) {
                ok = false;
            }
        }
        const float minA = ok ? fminf(ray_length, mn) : ray_length;
        const float maxA = ok ? fmaxf(0.0f, mx) : 0.0f;
        const float span_steps = ceilf(__fdiv_rn(__fsub_rn(maxA, minA), step));
        if (ok && mn <= mx && span_steps <= (float)kMaxSteps) {
            const int num_steps = (int)span_steps;
            float alpha = minA;
            int t = advance_alpha(&alpha, step, mn, num_steps, false);
            float a_end = alpha;
            const int t_end = t + advance_alpha(&a_end, step, mx, num_steps - t, true);
            const float sx = view.vol[0].s[0], sy = view.vol[0].s[1], sz = view.vol[0].s[2];
            const int n0 = V.n[0], n1 = V.n[1], n2 = V.n[2];
            const bool want_density = P.grad_density != nullptr;
            float *const grad_density = P.grad_density;
            // density-gradient run: texel cell of the hardware filter and its eight contributions
            int ci = -1, cj = -1, ck = -1, ci1 = 0, cj1 = 0, ck1 = 0;
            float acc[8];
#pragma unroll
            for (int c = 0; c < 8; c++) acc[c] = 0.0f;
            auto flush = [&]() {
                if (ci < 0) return;
                const int is[2] = {ci, ci1}, js[2] = {cj, cj1}, ks[2] = {ck, ck1};
#pragma unroll
                for (int c = 0; c < 8; c++)
                    if (acc[c] != 0.0f)
                        atomicAdd(grad_density + ((size_t)ks[c >> 2] * n1 + js[(c >> 1) & 1]) * n0 + is[c & 1], acc[c]);
            };
            // cache of the label cell floor(p): its word, per-corner material weights and texels
            float pb0 = __int_as_float(0x7fc00000), pb1 = pb0, pb2 = pb0;
            bool uni = false;
            float gu = 0.0f, g8[8], rho8[8];
#pragma unroll
            for (int c = 0; c < 8; c++) g8[c] = rho8[c] = 0.0f;
            float Hw[3] = {0.f, 0.f, 0.f}, K[3] = {0.f, 0.f, 0.f};
            for (; t < t_end; ++t) {
                const float wt = (0 == t || num_steps - 1 == t) ? 0.5f : 1.0f;
                const float px = __fsub_rn(__fmaf_rn(alpha, rxi, sx), 1.0f);
                const float py = __fsub_rn(__fmaf_rn(alpha, ryi, sy), 1.0f);
                const float pz = __fsub_rn(__fmaf_rn(alpha, rzi, sz), 1.0f);
                const float bx = floorf(px), by = floorf(py), bz = floorf(pz);
                const float fx = __fsub_rn(px, bx), fy = __fsub_rn(py, by), fz = __fsub_rn(pz, bz);
                if (bx != pb0 || by != pb1 || bz != pb2) {
                    const uint32_t word = fetch_label_word(V, bx, by, bz);
                    uni = uniform_word(word);
                    gu = gr_of<M>(gr, (int)(word & 15u));
#pragma unroll
                    for (int c = 0; c < 8; c++) g8[c] = uni ? gu : gr_of<M>(gr, (int)((word >> (4 * c)) & 15u));
                    if (POSE) {
#pragma unroll
                        for (int c = 0; c < 8; c++)
                            rho8[c] = tex3D<float>(P.density_point, bx + (float)(c & 1) + 0.5f,
                                                   by + (float)((c >> 1) & 1) + 0.5f, bz + (float)(c >> 2) + 0.5f);
                    }
                    pb0 = bx;
                    pb1 = by;
                    pb2 = bz;
                }
                const float gx = 1.0f - fx, gy = 1.0f - fy, gz = 1.0f - fz;
                // q = sum_m gr_m seg_m: the derivative of this sample's contribution by its density
                float q = gu;
                if (!uni) {
                    const CornerWeights cw = corner_weights(fx, fy, fz);
                    q = 0.0f;
#pragma unroll
                    for (int c = 0; c < 8; c++) q = __fmaf_rn(__fmul_rn(cw.xy[c & 3], cw.z[c >> 2]), g8[c], q);
                }
                if (want_density) {
                    // density gradient with the texture unit's corner weights at x = p + 0.5
                    int i0, i1, ax_, j0, j1, ay_, k0, k1, az_;
                    hw_axis(__fadd_rn(px, 0.5f), n0, i0, i1, ax_);
                    hw_axis(__fadd_rn(py, 0.5f), n1, j0, j1, ay_);
                    hw_axis(__fadd_rn(pz, 0.5f), n2, k0, k1, az_);
                    if (i0 != ci || j0 != cj || k0 != ck) {
                        flush();
                        ci = i0, cj = j0, ck = k0, ci1 = i1, cj1 = j1, ck1 = k1;
#pragma unroll
                        for (int c = 0; c < 8; c++) acc[c] = 0.0f;
                    }
                    int W[8];
                    hw_weights(ax_, ay_, az_, W);
                    const float wq = wt * q * (1.0f / 256.0f);
#pragma unroll
                    for (int c = 0; c < 8; c++) acc[c] = __fmaf_rn(wq, (float)W[c], acc[c]);
                }
                if (POSE) {
                    // h = d/dp of w_t rho(p) Q(p), rho and Q the continuous trilinear interpolants of
                    // the cell's texels and per-corner material weights
                    float dr[3];
                    trilinear_grad(rho8, fx, fy, fz, gx, gy, gz, dr);
                    float h[3];
                    if (uni) {
                        const float wQ = wt * gu;
                        h[0] = wQ * dr[0];
                        h[1] = wQ * dr[1];
                        h[2] = wQ * dr[2];
                    } else {
                        float dQ[3];
                        trilinear_grad(g8, fx, fy, fz, gx, gy, gz, dQ);
                        const float rho = trilinear(rho8, fx, fy, fz, gx, gy, gz);
                        const float Q = trilinear(g8, fx, fy, fz, gx, gy, gz);
                        h[0] = wt * (dr[0] * Q + rho * dQ[0]);
                        h[1] = wt * (dr[1] * Q + rho * dQ[1]);
                        h[2] = wt * (dr[2] * Q + rho * dQ[2]);
                    }
                    // q_w = A^T h (world-space derivative), accumulated plain and weighted by alpha
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        const float qw = A[k] * h[0] + A[3 + k] * h[1] + A[6 + k] * h[2];
                        Hw[k] += qw;
                        K[k] = __fmaf_rn(alpha, qw, K[k]);
                    }
                }
                alpha = __fadd_rn(alpha, step);
            }
            if (want_density) flush();
            if (POSE) {
                const float d[3] = {av.source_world[0] - P.center[0], av.source_world[1] - P.center[1],
                                    av.source_world[2] - P.center[2]};
                const float r[3] = {rx, ry, rz};
                pose[0] = -Hw[0];
                pose[1] = -Hw[1];
                pose[2] = -Hw[2];
                pose[3] = -((d[1] * Hw[2] - d[2] * Hw[1]) + (r[1] * K[2] - r[2] * K[1]));
                pose[4] = -((d[2] * Hw[0] - d[0] * Hw[2]) + (r[2] * K[0] - r[0] * K[2]));
                pose[5] = -((d[0] * Hw[1] - d[1] * Hw[0]) + (r[0] * K[1] - r[1] * K[0]));
            }
        }
    }
    if (POSE && zv < P.n_views) {
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
