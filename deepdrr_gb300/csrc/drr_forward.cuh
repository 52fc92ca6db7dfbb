// drr_forward.cuh -- forward DRR kernel (one thread per detector ray), sm_103a.
//
// Restates projectKernel of deepdrr/projector/project_kernel.cu:135-650 (deepdrr v1.2.2) with the
// same float32 arithmetic, operation by operation, so that results match the reference kernel:
//   * ray setup and normalisation                       project_kernel.cu:218-234
//   * per-volume slab test in IJK, boxes [-0.5, n-0.5]  project_kernel.cu:265-323
//   * num_steps = ceil((maxAlpha - minAlpha) / step)    project_kernel.cu:334
//   * float32 `alpha += step`, sample p = s + alpha r - 1 (the -1 voxel offset of both fields)
//                                                       project_kernel.cu:398-404, 552
//   * label fetches on voxel change, one cache shared by all volumes   project_kernel.cu:394-431
//   * trilinear label fractions, priority resolution, trapezoid half weights, hardware-filtered
//     density, per-material accumulation                project_kernel.cu:433-551
//   * air tails, * step, / 10 (mm -> cm)                project_kernel.cu:358-361, 557-584
//   * polychromatic Beer-Lambert                        project_kernel.cu:637-646
// Every multiply-add is an explicit __fmaf_rn / __fmul_rn / __fadd_rn so the compiler cannot
// re-associate or contract differently from the CPU oracle.
//
// Differences from the reference, none of which changes a result:
//   * per-volume state lives in registers (NV, M are template parameters) instead of the
//     reference's 528-byte local-memory stack frame;
//   * steps before the first volume interval opens do no sampling (their float32 alpha sequence is
//     still accumulated step by step, so every later sample position is bit-identical), and the
//     march stops once alpha has passed the last interval. With more than one volume the last
//     skipped step is replayed in full so the shared label cache enters the first live step in the
//     reference's state. DRR_FLAG_FULL_MARCH disables both shortcuts;
//   * a 2x2x2 label block whose eight labels agree takes a one-material path (adding +0.0f to the
//     other materials, as the reference does, leaves them unchanged);
//   * disabled volumes are ignored (the reference samples them with uninitialised directions);
//     the label cache starts as label 0 (the reference leaves it uninitialised).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace drr {

constexpr int kViewsPerLaunch = 32;
constexpr int kBlockThreads = 128;  // 4 warps; each warp covers an 8 x 4 pixel tile
constexpr int kTileW = 16;          // block tile: 16 x 8 pixels
constexpr int kTileH = 8;
constexpr double kAirDensity = 0.1129;  // project_kernel.cu:5-7 (a double literal)
constexpr int kMaxSteps = 1 << 26;      // longest march per ray; longer rays are reported as NaN

struct VolConst {
    cudaTextureObject_t density;  // linear filter, clamp, unnormalised coordinates
    cudaTextureObject_t labels;   // point filter, clamp, unnormalised coordinates, uint8
    float hi[3];                  // n - 0.5 per axis (projector.py:1626-1634)
    int32_t priority;
    int32_t enabled;
    int32_t pad;
};

struct VolPose {
    float a[9];  // 3x3 part of IJK_from_world (row-major), float32 as the reference host casts it
    float s[3];  // source position in IJK, float64 product cast to float32 (projector.py:812-820)
};

template <int NV>
struct ViewRec {
    float w[9];  // world_from_index[:-1, :] in float32 (projector.py:803)
    float pad;
    VolPose vol[NV];
};

template <int NV>
struct ForwardParams {
    VolConst vol[NV];
    const float *energies;  // [n_bins] keV
    const float *pdf;       // [n_bins]
    const float *mu;        // [n_bins][n_materials]
    float *intensity;       // [views][H][W]
    float *photon_prob;     // [views][H][W]
    float *area_density;    // [views][n_materials][H][W] or null
    float *solid_angle;     // [views][H][W] or null
    int32_t width, height, n_materials, n_bins;
    float step, max_ray_length;
    int32_t attenuate, air_index;
    int32_t full_march;
    int32_t view0;    // output index of views[0]
    int32_t n_views;  // views in this launch
    ViewRec<NV> views[kViewsPerLaunch];
};

// Pixel solid angle from two tetrahedra, project_kernel.cu:14-133 (Van Oosterom-Strackee formula).
__device__ __forceinline__ float pixel_solid_angle(const float *w, int udx, int vdx) {
    float cx[4], cy[4], cz[4], cm[4];
    const float cu_off[4] = {0.f, 1.f, 1.f, 0.f};
    const float cv_off[4] = {0.f, 0.f, 1.f, 1.f};
#pragma unroll
    for (int c = 0; c < 4; c++) {
        float cu = (float)udx + cu_off[c];
        float cv = (float)vdx + cv_off[c];
        cx[c] = __fmaf_rn(cu, w[0], __fmaf_rn(cv, w[1], w[2]));
        cy[c] = __fmaf_rn(cu, w[3], __fmaf_rn(cv, w[4], w[5]));
        cz[c] = __fmaf_rn(cu, w[6], __fmaf_rn(cv, w[7], w[8]));
        cm[c] = sqrtf(cx[c] * cx[c] + cy[c] * cy[c] + cz[c] * cz[c]);
    }
    float kx = cy[0] * cz[2] - cz[0] * cy[2];
    float ky = cz[0] * cx[2] - cx[0] * cz[2];
    float kz = cx[0] * cy[2] - cy[0] * cx[2];
    float d01 = cx[0] * cx[1] + cy[0] * cy[1] + cz[0] * cz[1];
    float d02 = cx[0] * cx[2] + cy[0] * cy[2] + cz[0] * cz[2];
    float d03 = cx[0] * cx[3] + cy[0] * cy[3] + cz[0] * cz[3];
    float d12 = cx[1] * cx[2] + cy[1] * cy[2] + cz[1] * cz[2];
    float d23 = cx[2] * cx[3] + cy[2] * cy[3] + cz[2] * cz[3];
    float n012 = fabsf(cx[1] * kx + cy[1] * ky + cz[1] * kz);
    float n023 = fabsf(cx[3] * kx + cy[3] * ky + cz[3] * kz);
    float den012 = cm[0] * cm[1] * cm[2] + d01 * cm[2] + d02 * cm[1] + d12 * cm[0];
    float den023 = cm[0] * cm[2] * cm[3] + d02 * cm[3] + d03 * cm[2] + d23 * cm[0];
    float sa012 = 2.f * atan2f(n012, den012);
    if (sa012 < 0.0f) sa012 += 3.14159265358979f;
    float sa023 = 2.f * atan2f(n023, den023);
    if (sa023 < 0.0f) sa023 += 3.14159265358979f;
    return sa012 + sa023;
}

__device__ __forceinline__ float add_air(float x) {
    // area_density[AIR_INDEX] += AIR_DENSITY: a float32 accumulator plus a double literal
    return (float)((double)x + kAirDensity);
}

template <int NV, int M>
__global__ void __launch_bounds__(kBlockThreads) forward_kernel(const __grid_constant__ ForwardParams<NV> p) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int u = blockIdx.x * kTileW + ((warp & 1) << 3) + (lane & 7);
    const int v = blockIdx.y * kTileH + ((warp >> 1) << 2) + (lane >> 3);
    const int zv = blockIdx.z;
    if (u >= p.width || v >= p.height || zv >= p.n_views) return;
    const ViewRec<NV> &view = p.views[zv];
    const float step = p.step;
    const int nmat = p.n_materials;

    // ---- ray setup (project_kernel.cu:218-234) ----
    const float uf = (float)u + 0.5f;
    const float vf = (float)v + 0.5f;
    float rx = __fmaf_rn(uf, view.w[0], __fmaf_rn(vf, view.w[1], view.w[2]));
    float ry = __fmaf_rn(uf, view.w[3], __fmaf_rn(vf, view.w[4], view.w[5]));
    float rz = __fmaf_rn(uf, view.w[6], __fmaf_rn(vf, view.w[7], view.w[8]));
    const float ray_length = __fsqrt_rn(__fmaf_rn(rx, rx, __fmaf_rn(ry, ry, __fmul_rn(rz, rz))));
    const float inv_norm = __fdiv_rn(1.0f, ray_length);
    rx = __fmul_rn(rx, inv_norm);
    ry = __fmul_rn(ry, inv_norm);
    rz = __fmul_rn(rz, inv_norm);

    // ---- per-volume slab test (project_kernel.cu:265-323) ----
    float minA = ray_length, maxA = 0.0f;
    float rxi[NV], ryi[NV], rzi[NV], minv[NV], maxv[NV];
    bool trace[NV];
#pragma unroll
    for (int i = 0; i < NV; i++) {
        trace[i] = false;
        minv[i] = 0.0f;
        maxv[i] = 0.0f;
        rxi[i] = ryi[i] = rzi[i] = 0.0f;
        if (!p.vol[i].enabled) continue;
        const float *A = view.vol[i].a;
        rxi[i] = __fmaf_rn(A[0], rx, __fmaf_rn(A[1], ry, __fmul_rn(A[2], rz)));
        ryi[i] = __fmaf_rn(A[3], rx, __fmaf_rn(A[4], ry, __fmul_rn(A[5], rz)));
        rzi[i] = __fmaf_rn(A[6], rx, __fmaf_rn(A[7], ry, __fmul_rn(A[8], rz)));
        const float r3[3] = {rxi[i], ryi[i], rzi[i]};
        float mn = 0.0f;
        float mx = p.max_ray_length > 0.0f ? p.max_ray_length : __int_as_float(0x7f800000);
        bool ok = true;
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            if (!ok) break;
            const float s = view.vol[i].s[ax];
            const float hi = p.vol[i].hi[ax];
            if (0.0f != r3[ax]) {
                const float reci = __fdiv_rn(1.0f, r3[ax]);
                const float a0 = __fmul_rn(__fsub_rn(-0.5f, s), reci);
                const float a1 = __fmul_rn(__fsub_rn(hi, s), reci);
                mn = fmaxf(mn, fminf(a0, a1));
                mx = fminf(mx, fmaxf(a0, a1));
            } else if (-0.5f > s || s > hi) {
                ok = false;
            }
        }
        minv[i] = mn;
        maxv[i] = mx;
        if (!ok) continue;
        trace[i] = true;
        minA = fminf(minA, mn);
        maxA = fmaxf(maxA, mx);
    }
    const float span_steps = ceilf(__fdiv_rn(__fsub_rn(maxA, minA), step));
    const size_t plane = (size_t)p.width * (size_t)p.height;
    const size_t vout = (size_t)(p.view0 + zv);
    const size_t pix = (size_t)v * (size_t)p.width + (size_t)u;
    if (span_steps > (float)kMaxSteps || span_steps != span_steps) {
        // Only non-finite or absurd geometry gets here; report NaN rather than march for ever.
        const float nan = __int_as_float(0x7fc00000);
        p.intensity[vout * plane + pix] = nan;
        p.photon_prob[vout * plane + pix] = nan;
        if (p.area_density != nullptr)
            for (int m = 0; m < nmat; m++) p.area_density[(vout * nmat + m) * plane + pix] = nan;
        if (p.solid_angle != nullptr) p.solid_angle[vout * plane + pix] = nan;
        return;
    }
    const int num_steps = (int)span_steps;

    // live interval: union of the non-empty volume intervals
    float amin = __int_as_float(0x7f800000), amax = -__int_as_float(0x7f800000);
#pragma unroll
    for (int i = 0; i < NV; i++) {
        if (trace[i] && minv[i] <= maxv[i]) {
            amin = fminf(amin, minv[i]);
            amax = fmaxf(amax, maxv[i]);
        }
    }

    float ad[M];
#pragma unroll
    for (int m = 0; m < M; m++) ad[m] = 0.0f;
    const bool attenuate = p.attenuate != 0;
    const int air = p.air_index;
    if (attenuate) {
        const double pre = (double)__fdiv_rn(minA, step) * kAirDensity;
#pragma unroll
        for (int m = 0; m < M; m++)
            if (m == air) ad[m] = (float)((double)ad[m] + pre);
    }

    float alpha = minA;
    int t = 0;
    if (!p.full_march) {
        // Skip the steps before any interval opens, keeping the float32 alpha sequence exact.
        float prev_alpha = alpha;
        while (t < num_steps && alpha < amin) {
            prev_alpha = alpha;
            alpha = __fadd_rn(alpha, step);
            ++t;
        }
        if (NV > 1 && t > 0) {  // replay one skipped step to seed the shared label cache
            alpha = prev_alpha;
            --t;
        }
        if (attenuate) {
            for (int k = 0; k < t; k++) {
#pragma unroll
                for (int m = 0; m < M; m++)
                    if (m == air) ad[m] = add_air(ad[m]);
            }
        }
    }

    // ---- the march (project_kernel.cu:398-553) ----
    float pb0 = -1.0f, pb1 = -1.0f, pb2 = -1.0f;  // previous_coordinates
    int vox[8];
#pragma unroll
    for (int c = 0; c < 8; c++) vox[c] = 0;
    bool uni = true;  // all eight cached labels equal
    int uni_label = 0;

    for (; t < num_steps; ++t) {
        if (!p.full_march && alpha > amax) break;
        float px[NV], py[NV], pz[NV];
        float seg[NV][M];
#pragma unroll
        for (int vol = 0; vol < NV; vol++) {
#pragma unroll
            for (int m = 0; m < M; m++) seg[vol][m] = 0.0f;
            px[vol] = py[vol] = pz[vol] = 0.0f;
            if (!p.vol[vol].enabled) continue;
            const float *s = view.vol[vol].s;
            px[vol] = __fsub_rn(__fmaf_rn(alpha, rxi[vol], s[0]), 1.0f);
            py[vol] = __fsub_rn(__fmaf_rn(alpha, ryi[vol], s[1]), 1.0f);
            pz[vol] = __fsub_rn(__fmaf_rn(alpha, rzi[vol], s[2]), 1.0f);
            const float bx = floorf(px[vol]), by = floorf(py[vol]), bz = floorf(pz[vol]);
            if (bx != pb0 || by != pb1 || bz != pb2) {
                const cudaTextureObject_t lt = p.vol[vol].labels;
#pragma unroll
                for (int dz = 0; dz <= 1; dz++)
#pragma unroll
                    for (int dy = 0; dy <= 1; dy++)
#pragma unroll
                        for (int dx = 0; dx <= 1; dx++)
                            vox[dz * 4 + dy * 2 + dx] =
                                (int)tex3D<unsigned char>(lt, __fadd_rn(px[vol], (float)dx),
                                                          __fadd_rn(py[vol], (float)dy),
                                                          __fadd_rn(pz[vol], (float)dz));
                pb0 = bx;
                pb1 = by;
                pb2 = bz;
                uni_label = vox[0];
                uni = true;
#pragma unroll
                for (int c = 1; c < 8; c++) uni = uni && (vox[c] == vox[0]);
            }
            const float fx = __fsub_rn(px[vol], bx), fy = __fsub_rn(py[vol], by), fz = __fsub_rn(pz[vol], bz);
            const float gx = __fsub_rn(1.0f, fx), gy = __fsub_rn(1.0f, fy), gz = __fsub_rn(1.0f, fz);
            float w[8];
            w[0] = __fmul_rn(__fmul_rn(gx, gy), gz);
            w[1] = __fmul_rn(__fmul_rn(fx, gy), gz);
            w[2] = __fmul_rn(__fmul_rn(gx, fy), gz);
            w[3] = __fmul_rn(__fmul_rn(fx, fy), gz);
            w[4] = __fmul_rn(__fmul_rn(gx, gy), fz);
            w[5] = __fmul_rn(__fmul_rn(fx, gy), fz);
            w[6] = __fmul_rn(__fmul_rn(gx, fy), fz);
            w[7] = __fmul_rn(__fmul_rn(fx, fy), fz);
            if (uni) {
                float sum = w[0];
#pragma unroll
                for (int c = 1; c < 8; c++) sum = __fadd_rn(sum, w[c]);
#pragma unroll
                for (int m = 0; m < M; m++)
                    if (m == uni_label) seg[vol][m] = sum;
            } else {
#pragma unroll
                for (int m = 0; m < M; m++) {
                    float acc = 0.0f;
#pragma unroll
                    for (int c = 0; c < 8; c++) acc = __fadd_rn(acc, vox[c] == m ? w[c] : 0.0f);
                    seg[vol][m] = acc;
                }
            }
        }

        // priority resolution (project_kernel.cu:458-496)
        int cur = NV, n = 0;
#pragma unroll
        for (int i = 0; i < NV; i++) {
            if (!trace[i]) continue;
            if (alpha < minv[i] || alpha > maxv[i]) continue;
            bool allzero = true;
#pragma unroll
            for (int m = 0; m < M; m++) allzero = allzero && (seg[i][m] == 0.0f);
            if (allzero) continue;
            const int pr = p.vol[i].priority;
            if (pr < cur) {
                cur = pr;
                n = 1;
            } else if (pr == cur) {
                n += 1;
            }
        }

        if (n == 0) {
            if (attenuate) {
#pragma unroll
                for (int m = 0; m < M; m++)
                    if (m == air) ad[m] = add_air(ad[m]);
            }
        } else {
            float weight = __fdiv_rn(1.0f, (float)n);
            weight = __fmul_rn(weight, (0 == t || num_steps - 1 == t) ? 0.5f : 1.0f);
#pragma unroll
            for (int vol = 0; vol < NV; vol++) {
                // no range re-check, as in project_kernel.cu:541
                if (trace[vol] && p.vol[vol].priority == cur) {
                    const float rho = tex3D<float>(p.vol[vol].density, __fadd_rn(px[vol], 0.5f),
                                                   __fadd_rn(py[vol], 0.5f), __fadd_rn(pz[vol], 0.5f));
                    const float wr = __fmul_rn(weight, rho);
#pragma unroll
                    for (int m = 0; m < M; m++) ad[m] = __fmaf_rn(wr, seg[vol][m], ad[m]);
                }
            }
        }
        alpha = __fadd_rn(alpha, step);
    }
    if (attenuate) {
        for (; t < num_steps; ++t) {
#pragma unroll
            for (int m = 0; m < M; m++)
                if (m == air) ad[m] = add_air(ad[m]);
        }
        const double post = (double)__fdiv_rn(__fsub_rn(ray_length, maxA), step) * kAirDensity;
#pragma unroll
        for (int m = 0; m < M; m++)
            if (m == air) ad[m] = (float)((double)ad[m] + post);
    }
#pragma unroll
    for (int m = 0; m < M; m++) ad[m] = __fdiv_rn(__fmul_rn(ad[m], step), 10.0f);

    // ---- polychromatic attenuation (project_kernel.cu:637-646) ----
    float inten = 0.0f, prob = 0.0f;
    const float *__restrict__ mu = p.mu;
    for (int bin = 0; bin < p.n_bins; bin++) {
        float x = 0.0f;
#pragma unroll
        for (int m = 0; m < M; m++)
            if (m < nmat) x = __fmaf_rn(ad[m], __ldg(mu + bin * nmat + m), x);
        const float pb = __fmul_rn(expf(-x), __ldg(p.pdf + bin));
        prob = __fadd_rn(prob, pb);
        inten = __fmaf_rn(__ldg(p.energies + bin), pb, inten);
    }

    p.intensity[vout * plane + pix] = inten;
    p.photon_prob[vout * plane + pix] = prob;
    if (p.area_density != nullptr) {
#pragma unroll
        for (int m = 0; m < M; m++)
            if (m < nmat) p.area_density[(vout * nmat + m) * plane + pix] = ad[m];
    }
    if (p.solid_angle != nullptr) p.solid_angle[vout * plane + pix] = pixel_solid_angle(view.w, u, v);
}

// Host-side launcher, explicitly instantiated per (NV, M) in drr_inst_nv*.cu.
template <int NV, int M>
cudaError_t launch_forward(const ForwardParams<NV> &p, cudaStream_t stream);

}  // namespace drr
