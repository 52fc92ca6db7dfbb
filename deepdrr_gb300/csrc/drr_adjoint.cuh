// drr_adjoint.cuh -- adjoint of the single-volume forward projection (density and pose gradients).
//
// The reference is not differentiable (README.md:47); this kernel adds the gradients of a loss L
// given dL/d(intensity) and dL/d(photon_prob) per pixel:
//
//   * dL/d(density): the exact adjoint of forward_kernel. A sample at p adds w_t * rho(p) * seg_m(p)
//     to the raw path length of material m, with rho(p) = sum_c W_c rho_c over the texture unit's
//     8-bit corner weights W_c at coordinate p + 0.5 (drr_texweights.h). So dL/d(rho_c) = sum over
//     samples of w_t W_c q_t, q_t = sum_m gr_m seg_m(p_t) and gr_m = dL/d(raw path length m).
//   * dL/d(pose): the derivative of a rigid motion of the volume, theta = (translation t,
//     rotation vector w about `center`, world frame), at theta = 0. Because the filtered density is
//     piecewise constant in p (8-bit weights), the position derivative uses the continuous
//     trilinear interpolation of the same texels and labels: h = w_t (grad rho Q + rho grad Q) with
//     Q the trilinear interpolation of gr over the eight corner labels. With q = A^T h (A the 3x3 of
//     IJK_from_world) and x_t = source + alpha_t r: dL/dt = -sum q, dL/dw = -sum (x_t - center) x q.
//     Changes of the step count and of the entry / exit samples with the pose are not differentiated.
//
// One kernel computes both. Each thread marches one ray over exactly the forward's samples (same
// float32 alpha sequence, same live step range, same trapezoid half weights); the 32 rays of a warp
// step together. A ray's full-weight samples fall into runs: stretches with one label cell and one
// texture-filter cell (the two half-weight samples are runs of their own). Within a run the
// per-sample work is small and identical across the warp: the three staged terms of the eight
// integer corner weights, two 16-bit lanes to a register, are summed, and the run's summed corner
// weights are formed from them once (drr_texweights.h). A run ends where a sample's cells differ
// from the previous sample's. When a run ends, the ray appends its first alpha,
// length and sums to a per-warp ring in shared memory; once 32 runs wait, the warp drains them,
// one run per lane, so the per-cell work -- the label word, eight texel additions to the gradient
// volume, eight texel fetches and the pose sums -- runs with all lanes busy instead of once per
// lane that happens to change cell. The drain re-derives a run's positions from its first alpha
// with the march's own float32 operations. A run in a cell whose eight labels agree is summed in
// closed form: q and Q are constant there and grad rho is bilinear in the fractions, so the pose
// sums over the run's evenly spaced samples are polynomials in the run length; in a cell whose
// eight texels are equal they are zero, and a drain whose 32 runs all lie in such cells (air of
// constant density, which a warp's neighbouring rays often cross together) skips them. Runs in
// cells with mixed labels wait in a second ring and are then split into their samples, 32
// evaluated at once.
// Only single-volume projections without air attenuation outside the volume are differentiated.
#pragma once

#include "drr_forward.cuh"
#include "drr_texweights.h"

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

// Per-ray state of the adjoint: the upstream material weights and the forward's march.
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

// Per-warp run queues of adjoint_kernel: rings the warp drains 32 runs at a time (runs: kRunQueue
// entries; runs set aside in mixed-label cells: kAdjQueue). A run entry is one 16-byte and one
// 8-byte word group: alpha0, count | lane << 8 | half << 13, and the run's sums of the staged
// weight terms (SX, S0 | S1, SZ, drr_texweights.h). Past the run ring, one slot per lane takes the
// stores of lanes that close no run, so a push needs no branch.
constexpr int kAdjQueue = 64;
constexpr int kRunQueue = 128;  // run ring: up to 31 waiting + 64 pushed in two steps
constexpr int kMixWords = 3;  // alpha0, count | lane << 8 | half << 13, label word

template <int M>
struct AdjointWarpSmem {
    uint4 runa[kRunQueue + 32];  // alpha0, count | lane << 8 | half << 13, SX, S0
    uint2 runb[kRunQueue + 32];  // S1, SZ
    uint32_t mix[kMixWords][kAdjQueue];  // runs in cells with mixed labels, set aside by the drain
    float gr[M][32];   // each lane's material weights gr_m
    float ray[6][32];  // each lane's unit ray in IJK (0-2) and source in IJK (3-5)
    float pose[6][32];  // each lane's share of the drained sums: h (IJK, 0-2) and the moments m (3-5)
    float A[9];        // the view's IJK_from_world rotation
    float G[6];        // A A^T: xx, xy, xz, yy, yz, zz
};

__device__ __forceinline__ void red_add_pair(float *a, float x, float y) {
    if ((reinterpret_cast<uintptr_t>(a) & 7u) == 0) {
        asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(a), "f"(x), "f"(y) : "memory");
    } else {
        atomicAdd(a, x);
        atomicAdd(a + 1, y);
    }
}

// rv * W for the eight corner weights packed two to a word (P[dx * 2 + dy] = W(dz = 0) | W(dz = 1) << 16,
// drr_texweights.h), ordered for scatter_cell (v[2 row + dx] with row = dy | dz << 1). A 16-bit count
// becomes a float through the exponent field (2^23 + count is exact below 2^23), and one fused
// multiply-add gives rv * count rounded once, as rv * (float)count would: no integer-to-float
// conversions.
__device__ __forceinline__ void weighted_corners(const uint32_t P[4], float rv, float v[8]) {
    const float bias = __fmul_rn(rv, 8388608.0f);  // rv * 2^23, exact
#pragma unroll
    for (int row = 0; row < 4; row++) {
        const int dy = row & 1, dz = row >> 1;
#pragma unroll
        for (int dx = 0; dx < 2; dx++) {
            const uint32_t cnt = (P[dx * 2 + dy] >> (16 * dz)) & 0xFFFFu;
            v[2 * row + dx] = __fmaf_rn(rv, __uint_as_float(0x4B000000u | cnt), -bias);
        }
    }
}

// Adds v[c] to texel c = dx | dy << 1 | dz << 2 of the filter cell with lower corner (i0, j0, k0):
// texel (min(i0 + dx, n0 - 1), ...) of the [n2][n1][n0] gradient volume, as the texture's clamp
// addressing reads it. The two texels of a row are adjacent and go out as one vector reduction.
// Zero values are added too: a weight is zero only for a fraction of exactly 0, and testing for
// it costs the warp more than the few extra reductions. Volumes of at most 32767 texels per axis
// (drr_project_adjoint's limit) keep a plane's offsets below 2^31, so the rows are addressed as a
// plane pointer (one widening multiply) plus 32-bit offsets.
__device__ __forceinline__ void scatter_cell(float *grad, int i0, int j0, int k0, int n0, int n1, int n2,
                                             const float v[8]) {
    const int j1 = min(j0 + 1, n1 - 1), k1 = min(k0 + 1, n2 - 1);
    const int plane = n0 * n1;
    float *const p0 = grad + (long long)k0 * plane, *const p1 = grad + (long long)k1 * plane;
    const int o0 = j0 * n0 + i0, o1 = j1 * n0 + i0;
#pragma unroll
    for (int row = 0; row < 4; row++) {
        const float x = v[2 * row], y = v[2 * row + 1];
        float *a = (row & 2 ? p1 : p0) + (row & 1 ? o1 : o0);
        if (i0 + 1 >= n0) {  // clamped edge: both corners are the same texel
            atomicAdd(a, x + y);
        } else {
            red_add_pair(a, x, y);
        }
    }
}

// Fixed point of the texture unit for density coordinate p + 0.5 on an axis of n texels
// (drr_texweights.h). `hw_fix_live` omits the upper clamp, which no marched sample reaches: live
// samples satisfy p <= n - 1.5 (up to rounding), so 256 (p + 0.5) - 127.5 stays 128 below 256 (n - 1).
__device__ __forceinline__ int hw_fix(float p, int n) {
    return hw_fix_from_floor(__float2int_rd(__fmaf_rn(__fadd_rn(p, 0.5f), 256.0f, -127.5f)), n);
}
__device__ __forceinline__ int hw_fix_live(float p) {
    // the conversion to unsigned saturates: a negative value (a coordinate below the first texel
    // centre) becomes 0, the texture's lower clamp
    return (int)__float2uint_rd(__fmaf_rn(__fadd_rn(p, 0.5f), 256.0f, -127.5f));
}

// Pose sums of one run or sample, into lane `lane`'s own share: the IJK sum h, and the moment of
// the alpha-weighted sum hk about the source, r x (A^T hk) in world coordinates (r the owner ray's
// unit direction). With r_ijk = A r and any invertible A, (A^-1 a) x (A^-1 b) = A^T (a x b) / det A
// gives r x (A^T hk) = A^T (r_ijk x (A A^T hk)) / det A: the lane sums m = r_ijk x (G hk), G = A A^T,
// and A^T / det A is applied once per warp at the end. No lane writes another lane's share, so no
// atomics are needed (shared-memory float atomics cost more than the twelve multiply-adds).
template <int M>
__device__ __forceinline__ void add_pose_sums(AdjointWarpSmem<M> &sh, int lane, const float h[3], const float hk[3],
                                              int owner) {
    sh.pose[0][lane] += h[0], sh.pose[1][lane] += h[1], sh.pose[2][lane] += h[2];
    const float u0 = sh.G[0] * hk[0] + sh.G[1] * hk[1] + sh.G[2] * hk[2];
    const float u1 = sh.G[1] * hk[0] + sh.G[3] * hk[1] + sh.G[4] * hk[2];
    const float u2 = sh.G[2] * hk[0] + sh.G[4] * hk[1] + sh.G[5] * hk[2];
    const float r0 = sh.ray[0][owner], r1 = sh.ray[1][owner], r2 = sh.ray[2][owner];
    sh.pose[3][lane] += r1 * u2 - r2 * u1;
    sh.pose[4][lane] += r2 * u0 - r0 * u2;
    sh.pose[5][lane] += r0 * u1 - r1 * u0;
}

// One sample of a mixed-label cell at float32 alpha `al` of ray `owner` (label word `word`): the
// forward's label weights q_t with the texture unit's corner weights for the density, the
// trilinear gradient of rho Q for the pose. Written corner by corner so that few registers stay
// live: it runs rarely, inside the march's register budget.
template <int M>
__device__ __forceinline__ void mixed_sample(const AdjointParams &P, AdjointWarpSmem<M> &sh, int lane, float al,
                                             int owner, float wrun, uint32_t word) {
    const VolConst &V = P.s.vol[0];
    const int n0 = V.n[0], n1 = V.n[1], n2 = V.n[2];
    const float px = __fsub_rn(__fmaf_rn(al, sh.ray[0][owner], sh.ray[3][owner]), 1.0f);
    const float py = __fsub_rn(__fmaf_rn(al, sh.ray[1][owner], sh.ray[4][owner]), 1.0f);
    const float pz = __fsub_rn(__fmaf_rn(al, sh.ray[2][owner], sh.ray[5][owner]), 1.0f);
    const float bx = floorf(px), by = floorf(py), bz = floorf(pz);
    const float fx = __fsub_rn(px, bx), fy = __fsub_rn(py, by), fz = __fsub_rn(pz, bz);
    if (P.grad_density != nullptr) {
        const CornerWeights cw = corner_weights(fx, fy, fz);
        float q = 0.0f;
#pragma unroll
        for (int c = 0; c < 8; c++)
            q = __fmaf_rn(__fmul_rn(cw.xy[c & 3], cw.z[c >> 2]), sh.gr[(word >> (4 * c)) & 15u][owner], q);
        const float rv = __fmul_rn(__fmul_rn(wrun, q), 1.0f / 256.0f);
        const int fxi = hw_fix(px, n0), fyi = hw_fix(py, n1), fzi = hw_fix(pz, n2);
        uint32_t Wp[4];
        packed_corner_weights((uint32_t)fxi & 255u, (uint32_t)fyi & 255u, (uint32_t)fzi & 255u, Wp);
        if (rv != 0.0f) {
            float vals[8];
            weighted_corners(Wp, rv, vals);
            scatter_cell(P.grad_density, fxi >> 8, fyi >> 8, fzi >> 8, n0, n1, n2, vals);
        }
    }
    if (P.grad_pose != nullptr) {
        // rho, Q and their gradients, corner by corner
        float rho = 0.0f, Q = 0.0f, dr0 = 0.0f, dr1 = 0.0f, dr2 = 0.0f, dq0 = 0.0f, dq1 = 0.0f, dq2 = 0.0f;
#pragma unroll 1
        for (int c = 0; c < 8; c++) {
            const float ox = (float)(c & 1), oy = (float)((c >> 1) & 1), oz = (float)(c >> 2);
            const float rc = tex3D<float>(P.density_point, bx + ox + 0.5f, by + oy + 0.5f, bz + oz + 0.5f);
            const float gc = sh.gr[(word >> (4 * c)) & 15u][owner];
            const float wx = c & 1 ? fx : 1.0f - fx, wy = c & 2 ? fy : 1.0f - fy, wz = c & 4 ? fz : 1.0f - fz;
            const float sx = c & 1 ? 1.0f : -1.0f, sy = c & 2 ? 1.0f : -1.0f, sz = c & 4 ? 1.0f : -1.0f;
            const float bxy = wx * wy, bxz = wx * wz, byz = wy * wz, bc = bxy * wz;
            rho += rc * bc, Q += gc * bc;
            dr0 += rc * sx * byz, dr1 += rc * sy * bxz, dr2 += rc * sz * bxy;
            dq0 += gc * sx * byz, dq1 += gc * sy * bxz, dq2 += gc * sz * bxy;
        }
        float h[3], hk[3];
        h[0] = wrun * (dr0 * Q + rho * dq0), h[1] = wrun * (dr1 * Q + rho * dq1), h[2] = wrun * (dr2 * Q + rho * dq2);
#pragma unroll
        for (int c = 0; c < 3; c++) hk[c] = al * h[c];
        add_pose_sums<M>(sh, lane, h, hk, owner);
    }
}

// Drains `count` (<= 32) queued mixed-label runs starting at mixed-ring slot `first`: their
// samples, numbered across the warp, are evaluated 32 at a time. Called by the whole warp.
template <int M>
__device__ __forceinline__ void drain_mixed(const AdjointParams &P, AdjointWarpSmem<M> &sh, int lane, int first,
                                         int count) {
    const unsigned kAll = 0xffffffffu;
    const float step = P.s.step;
    float al = 0.0f, wrun = 1.0f;
    int kn = 0, owner = 0;
    uint32_t word = 0;
    if (lane < count) {
        const int e = (first + lane) & (kAdjQueue - 1);
        al = __uint_as_float(sh.mix[0][e]);
        const uint32_t w1 = sh.mix[1][e];
        kn = (int)(w1 & 255u), owner = (int)((w1 >> 8) & 31u);
        wrun = (w1 >> 13) & 1u ? 0.5f : 1.0f;
        word = sh.mix[2][e];
    }
    int off = kn;  // inclusive prefix sum over the lanes
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(kAll, off, o);
        if (lane >= o) off += x;
    }
    const int total = __shfl_sync(kAll, off, 31);
    for (int base = 0; base < total; base += 32) {
        const int g = base + lane;
        // the run holding sample g: the first lane whose inclusive prefix exceeds g
        int src = 0;
#pragma unroll
        for (int b = 16; b > 0; b >>= 1) {
            const int cand = src + b;
            const int o_c = __shfl_sync(kAll, off, cand - 1);
            if (o_c <= g) src = cand;
        }
        // every lane takes part in every shuffle (lane src - 1 wraps to 31 for src = 0)
        const int o_before = __shfl_sync(kAll, off, (src + 31) & 31);
        const int o_prev = src > 0 ? o_before : 0;
        const float s_al = __shfl_sync(kAll, al, src);
        const int s_owner = __shfl_sync(kAll, owner, src) & 31;
        const float s_w = __shfl_sync(kAll, wrun, src);
        const uint32_t s_word = __shfl_sync(kAll, word, src);
        if (g < total) {
            // the march's float32 alpha sequence: k = g - o_prev (< 255) additions from the run's
            // first. After the first addition every addition adds the same number of ulps while
            // alpha stays in one binade (drr_alpha.h), so a_k = a_1 + (k - 1) (a_2 - a_1) in ulps
            // when a_k's exponent is a_1's; otherwise the additions are done one by one.
            const int k = min(max(g - o_prev, 0), 254);
            float a = s_al;
            if (k > 0) {
                const float a1 = __fadd_rn(s_al, step), a2 = __fadd_rn(a1, step);
                const uint32_t b1 = __float_as_uint(a1);
                const uint32_t cand = b1 + (uint32_t)(k - 1) * (__float_as_uint(a2) - b1);
                if ((cand >> 23) == (b1 >> 23) && (b1 >> 23) != 0u && (b1 >> 31) == 0u) {
                    a = __uint_as_float(cand);
                } else {
                    for (int j = k; j > 0; --j) a = __fadd_rn(a, step);
                }
            }
            mixed_sample<M>(P, sh, lane, a, s_owner, s_w, s_word);
        }
    }
}

// Density and pose gradients of one view per blockIdx.z, one ray per thread (16 x 8 pixel tiles,
// each warp 8 x 4 pixels). A run is a stretch of a ray's full-weight samples with one label cell
// and one texture-filter cell; the trapezoid half-weight samples (t = 0 and t = num_steps - 1) are
// runs of their own. See the file comment. Resident blocks per SM balance occupancy against the
// registers the drain needs: with 3 materials and the drain's texel fetches issued before its
// label-code load, 6 blocks (80 registers, no spills) measured 0.780 ms/view on the 256^3 / 64 x
// 256^2 workload, against 0.912 at 7 blocks (72 registers, spilling) and 0.813 at 7 blocks with the
// fetches after the code. More materials keep 5.
template <int M>
__global__ void __launch_bounds__(kBlockThreads, M <= 4 ? 6 : 5) adjoint_kernel(const __grid_constant__ AdjointParams P) {
    __shared__ AdjointWarpSmem<M> smem[kBlockThreads / 32];
    const SceneParams<1> &p = P.s;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    AdjointWarpSmem<M> &sh = smem[warp];
    const int u = blockIdx.x * kTileW + ((warp & 1) << 3) + (lane & 7);
    const int v = blockIdx.y * kTileH + ((warp >> 1) << 2) + (lane >> 3);
    const int zv = blockIdx.z;  // the grid has one z per view
    const AdjointView &av = P.views[zv];
    const VolConst &V = p.vol[0];
    const bool do_dens = P.grad_density != nullptr;
    const bool do_pose = P.grad_pose != nullptr;
    const unsigned kAll = 0xffffffffu;

    AdjointRay<M> R{};
    const bool ray_live = u < p.width && v < p.height && adjoint_setup<M>(P, av, u, v, zv, R);
#pragma unroll
    for (int m = 0; m < M; m++) sh.gr[m][lane] = ray_live ? R.gr[m] : 0.0f;
    sh.ray[0][lane] = R.rxi;
    sh.ray[1][lane] = R.ryi;
    sh.ray[2][lane] = R.rzi;
    sh.ray[3][lane] = R.sx;
    sh.ray[4][lane] = R.sy;
    sh.ray[5][lane] = R.sz;
    if (lane < 9) sh.A[lane] = av.v.vol[0].a[lane];
    __syncwarp();
    if (lane < 6) {  // G = A A^T, entry (gi, gj)
        const int gi = lane < 3 ? 0 : (lane < 5 ? 1 : 2), gj = lane < 3 ? lane : (lane < 5 ? lane - 2 : 2);
        sh.G[lane] = sh.A[3 * gi] * sh.A[3 * gj] + sh.A[3 * gi + 1] * sh.A[3 * gj + 1] +
                     sh.A[3 * gi + 2] * sh.A[3 * gj + 2];
    }
    __syncwarp();

    const int n0 = V.n[0], n1 = V.n[1], n2 = V.n[2];
    const float step = p.step;
    float *const grad = P.grad_density;
#pragma unroll
    for (int k = 0; k < 6; k++) sh.pose[k][lane] = 0.0f;

    int head = 0, queued = 0;    // warp-uniform state of the run ring
    int mhead = 0, mqueued = 0;  // and of the mixed-label ring
    const unsigned lt = (1u << lane) - 1u;

    auto add_pose = [&](const float h[3], const float hk[3], int owner) { add_pose_sums<M>(sh, lane, h, hk, owner); };

    // Drains `count` (<= 32) queued runs starting at ring slot `first`, one run per lane. Each run is
    // re-derived from its first alpha with the march's own float32 operations, so its positions,
    // label cell and filter cell are the march's. Runs in cells with mixed labels are then split
    // into their samples, which the warp evaluates 32 at a time.
    auto drain = [&](int first, int count) {
        const bool mine = lane < count;
        const int e = (first + lane) & (kRunQueue - 1);
        float al = 0.0f, wrun = 1.0f;
        int kn = 0, owner = 0;
        uint32_t word = 0, w1 = 0;
        bool mixed = false;
        if (mine) {
            const uint4 ra = sh.runa[e];
            const uint2 rb = sh.runb[e];
            al = __uint_as_float(ra.x);
            w1 = ra.y;
            kn = (int)(w1 & 255u), owner = (int)((w1 >> 8) & 31u);
            wrun = (w1 >> 13) & 1u ? 0.5f : 1.0f;
            const float rxi = sh.ray[0][owner], ryi = sh.ray[1][owner], rzi = sh.ray[2][owner];
            const float px = __fsub_rn(__fmaf_rn(al, rxi, sh.ray[3][owner]), 1.0f);
            const float py = __fsub_rn(__fmaf_rn(al, ryi, sh.ray[4][owner]), 1.0f);
            const float pz = __fsub_rn(__fmaf_rn(al, rzi, sh.ray[5][owner]), 1.0f);
            const float bx = floorf(px), by = floorf(py), bz = floorf(pz);
            // the cell's eight texels (pose), fetched before the label code so that both loads are
            // in flight together
            float r8[8];
            if (do_pose) {
#pragma unroll
                for (int c = 0; c < 8; c++)
                    r8[c] = tex3D<float>(P.density_point, bx + (float)(c & 1) + 0.5f,
                                         by + (float)((c >> 1) & 1) + 0.5f, bz + (float)(c >> 2) + 0.5f);
            }
            // the cell's label code; the packed word only for a run in a mixed cell
            const float cbx = fminf(fmaxf(bx, -1.0f), V.nm1[0]), cby = fminf(fmaxf(by, -1.0f), V.nm1[1]);
            const float cbz = fminf(fmaxf(bz, -1.0f), V.nm1[2]);
            const uint32_t code = label_entry(V.coded, V, (int)cbx, (int)cby, (int)cbz);
            mixed = (code >> 8) != 0u;
            if (mixed) word = code_word(V, code, cbx, cby, cbz);
            if (!mixed) {
                const float gu = sh.gr[code & 15u][owner];
                if (do_dens) {
                    // every sample adds w_t gu W_c / 256 to texel c: the packed sums hold sum W_c
                    const float rv = __fmul_rn(__fmul_rn(wrun, gu), 1.0f / 256.0f);
                    uint32_t sums[4];
                    packed_weight_sums((uint32_t)kn, ra.z, ra.w, rb.x, rb.y, sums);
                    float vals[8];
                    weighted_corners(sums, rv, vals);
                    scatter_cell(grad, hw_fix(px, n0) >> 8, hw_fix(py, n1) >> 8, hw_fix(pz, n2) >> 8, n0, n1, n2,
                                 vals);
                }
                if (do_pose) {
                    // a cell whose eight texels are equal (and finite) has grad rho = 0: its pose
                    // terms are exactly zero, and a warp whose runs all lie in such cells skips them
                    bool flat = fabsf(r8[0]) < __int_as_float(0x7f800000);
#pragma unroll
                    for (int c = 1; c < 8; c++) flat = flat && r8[c] == r8[0];
                    if (!flat) {
                        // grad rho = c0 + c1 f_a + c2 f_b + c3 f_a f_b per axis (f_a, f_b the other two
                        // fractions), summed over the run's samples f0 + k d, alpha0 + k delta in closed form
                        const float ax = __fsub_rn(px, bx), ay = __fsub_rn(py, by), az = __fsub_rn(pz, bz);
                        const float delta = __fsub_rn(__fadd_rn(al, step), al);  // the float32 step at alpha0
                        const float bxs = delta * rxi, bys = delta * ryi, bzs = delta * rzi;
                        const float ex = r8[1] - r8[0], ey = r8[2] - r8[0], ez = r8[4] - r8[0];
                        const float x1 = (r8[3] - r8[2]) - ex, x2 = (r8[5] - r8[4]) - ex;
                        const float x3 = (r8[7] - r8[6]) - (r8[5] - r8[4]) - (r8[3] - r8[2]) + ex;
                        const float y1 = (r8[3] - r8[1]) - ey, y2 = (r8[6] - r8[4]) - ey;
                        const float y3 = (r8[7] - r8[5]) - (r8[6] - r8[4]) - (r8[3] - r8[1]) + ey;
                        const float z1 = (r8[5] - r8[1]) - ez, z2 = (r8[6] - r8[2]) - ez;
                        const float z3 = (r8[7] - r8[3]) - (r8[6] - r8[2]) - (r8[5] - r8[1]) + ez;
                        // about the run's middle sample k_c = (K - 1) / 2 the odd sums of k - k_c vanish:
                        // sum g(f_k) and sum alpha_k g(f_k) need only S2 = sum (k - k_c)^2 = K (K^2 - 1) / 12
                        const float kf = (float)kn;
                        const float kc = 0.5f * kf - 0.5f;
                        const float cx = ax + kc * bxs, cy = ay + kc * bys, cz = az + kc * bzs;
                        const float ac = al + kc * delta;
                        const float S2 = kf * (kf * kf - 1.0f) * (1.0f / 12.0f);
                        const float dS2 = delta * S2;
                        float h[3], hk[3];
                        float m = kf, n = ac * kf;  // g = 1
                        h[0] = ex * m, h[1] = ey * m, h[2] = ez * m;
                        hk[0] = ex * n, hk[1] = ey * n, hk[2] = ez * n;
                        m = kf * cx, n = ac * m + dS2 * bxs;  // g = f_x
                        h[1] += y1 * m, h[2] += z1 * m, hk[1] += y1 * n, hk[2] += z1 * n;
                        m = kf * cy, n = ac * m + dS2 * bys;  // g = f_y
                        h[0] += x1 * m, h[2] += z2 * m, hk[0] += x1 * n, hk[2] += z2 * n;
                        m = kf * cz, n = ac * m + dS2 * bzs;  // g = f_z
                        h[0] += x2 * m, h[1] += y2 * m, hk[0] += x2 * n, hk[1] += y2 * n;
                        m = kf * cx * cy + bxs * bys * S2, n = ac * m + dS2 * (cx * bys + cy * bxs);  // g = f_x f_y
                        h[2] += z3 * m, hk[2] += z3 * n;
                        m = kf * cx * cz + bxs * bzs * S2, n = ac * m + dS2 * (cx * bzs + cz * bxs);  // g = f_x f_z
                        h[1] += y3 * m, hk[1] += y3 * n;
                        m = kf * cy * cz + bys * bzs * S2, n = ac * m + dS2 * (cy * bzs + cz * bys);  // g = f_y f_z
                        h[0] += x3 * m, hk[0] += x3 * n;
                        const float gw = gu * wrun;
    #pragma unroll
                        for (int c = 0; c < 3; c++) h[c] *= gw, hk[c] *= gw;
                        add_pose(h, hk, owner);
                    }
                }
            }
        }
        // runs in mixed-label cells wait in their own ring until 32 of them can go at once
        const unsigned mm = __ballot_sync(kAll, mixed);
        if (mixed) {
            const int s = (mhead + mqueued + __popc(mm & lt)) & (kAdjQueue - 1);
            sh.mix[0][s] = __float_as_uint(al);
            sh.mix[1][s] = w1;
            sh.mix[2][s] = word;
        }
        mqueued += __popc(mm);
        if (mqueued >= 32) {
            __syncwarp();
            drain_mixed<M>(P, sh, lane, mhead, 32);
            __syncwarp();
            mhead = (mhead + 32) & (kAdjQueue - 1);
            mqueued -= 32;
        }
    };

    // Phases of each ray: [a half-weight sample at t = 0] [full-weight samples] [a half-weight
    // sample at t = num_steps - 1], each phase for the whole warp at once.
    float alpha = R.alpha;
    int t = R.t;
    const bool first_half = ray_live && R.t == 0;
    const bool last_half = ray_live && R.t_end == R.num_steps && R.num_steps > 1;
    const int t_stop = last_half ? R.num_steps - 1 : R.t_end;  // end of the full-weight samples

    // the open run: sample count, first alpha, sums of the staged weight terms hx, hy0, hy1 and of
    // Az (drr_texweights.h); the label cell and filter fixed point of the previous sample
    int K = 0;
    float a0 = 0.0f, rbx = 0.0f, rby = 0.0f, rbz = 0.0f;
    int rfx = 0, rfy = 0, rfz = 0;
    uint32_t SX = 0, S0 = 0, S1 = 0, SZ = 0;

    auto enqueue = [&](bool push, bool half) {
        const unsigned pm = __ballot_sync(kAll, push);
        {
            // a lane that closes no run stores into its own slot past the ring
            const int s = push ? (head + queued + __popc(pm & lt)) & (kRunQueue - 1) : kRunQueue + lane;
            sh.runa[s] = make_uint4(__float_as_uint(a0), (uint32_t)K | ((uint32_t)lane << 8) | (half ? 1u << 13 : 0u),
                                    SX, S0);
            sh.runb[s] = make_uint2(S1, SZ);
            K = push ? 0 : K;
        }
        queued += __popc(pm);
    };
    auto settle = [&]() {  // drain while 32 runs wait (warp-uniform); one call site per loop iteration
        while (queued >= 32) {
            __syncwarp();
            drain(head, 32);
            __syncwarp();
            head = (head + 32) & (kRunQueue - 1);
            queued -= 32;
        }
    };
    // a single-sample run at the current alpha (the half-weight samples)
    auto single = [&](bool here) {
        if (here) {
            const float cx = __fsub_rn(__fmaf_rn(alpha, R.rxi, R.sx), 1.0f);
            const float cy = __fsub_rn(__fmaf_rn(alpha, R.ryi, R.sy), 1.0f);
            const float cz = __fsub_rn(__fmaf_rn(alpha, R.rzi, R.sz), 1.0f);
            SX = S0 = S1 = SZ = 0u;
            if (do_dens) {
                const int fxi = hw_fix(cx, n0), fyi = hw_fix(cy, n1), fzi = hw_fix(cz, n2);
                SZ = (uint32_t)fzi & 255u;
                weight_terms((uint32_t)fxi & 255u, (uint32_t)fyi & 255u, SZ, SX, S0, S1);
            }
            a0 = alpha;
            K = 1;
        }
        enqueue(here, true);
        settle();
    };

    single(first_half);
    if (first_half) {
        alpha = __fadd_rn(alpha, step);
        ++t;
    }
    // The warp runs its longest ray's full-weight samples plus one step that closes the last runs,
    // a bound known up front (one reduction), so the loop needs no vote per step. A lane past its
    // own samples marches on through positions it does not use: it closes its last run, opens no
    // other, and its sums are never queued again. Its alpha after its own samples, where the last
    // half-weight sample lies, comes from the exact fast-forward (drr_alpha.h).
    const int my_steps = t < t_stop ? t_stop - t : 0;
    const int warp_steps = __reduce_max_sync(kAll, my_steps) + 1;
    float alpha_end = alpha;
    advance_alpha(&alpha_end, step, __int_as_float(0x7f800000), my_steps, false);
    // x and y travel as f32x2 pairs (the same roundings as the scalar operations)
    const float2 r2 = make_float2(R.rxi, R.ryi), s2 = make_float2(R.sx, R.sy);
    const float2 one2 = make_float2(1.0f, 1.0f), half2v = make_float2(0.5f, 0.5f);
    const float2 f256 = make_float2(256.0f, 256.0f), fofs = make_float2(-127.5f, -127.5f);
    const float2 step2 = make_float2(step, step);
    float2 a2 = make_float2(alpha, alpha);
    float2 c2 = sub2_rn(fma2_rn(a2, r2, s2), one2);
    float cz = __fsub_rn(__fmaf_rn(alpha, R.rzi, R.sz), 1.0f);
    auto march_step = [&](int it) {
        const bool live = it < my_steps;
        const float bx = floorf(c2.x), by = floorf(c2.y), bz = floorf(cz);
        int fxi = 0, fyi = 0, fzi = 0;
        // Each axis's position, label cell and fixed point are monotone in alpha (every operation
        // producing them is a monotone rounding), so a sample whose cells equal the previous
        // sample's has the cells of the whole open run: comparing with the previous sample suffices.
        bool fresh = K == 255 || bx != rbx || by != rby || bz != rbz;
        if (do_dens) {
            // hw_fix_live of x and y as one pair
            const float2 q2 = fma2_rn(add2_rn(c2, half2v), f256, fofs);
            fxi = (int)__float2uint_rd(q2.x), fyi = (int)__float2uint_rd(q2.y), fzi = hw_fix_live(cz);
            fresh = fresh || ((fxi ^ rfx) | (fyi ^ rfy) | (fzi ^ rfz)) >= 256;
        }
        // a run ends when this sample starts a new one or the ray has no full-weight samples left
        enqueue(K > 0 && (!live || fresh), false);
        const bool open = live && K == 0;  // this sample starts a run
        a0 = open ? a2.x : a0;
        if (do_dens) {
            uint32_t hx, hy0, hy1;
            const uint32_t Az = (uint32_t)fzi & 255u;
            weight_terms((uint32_t)fxi & 255u, (uint32_t)fyi & 255u, Az, hx, hy0, hy1);
            // a lane past its samples adds to sums that are never queued again (its run is closed)
            SX = (open ? 0u : SX) + hx;
            S0 = (open ? 0u : S0) + hy0;
            S1 = (open ? 0u : S1) + hy1;
            SZ = (open ? 0u : SZ) + Az;
        }
        rbx = bx, rby = by, rbz = bz;
        rfx = fxi, rfy = fyi, rfz = fzi;
        K += live ? 1 : 0;
        a2 = add2_rn(a2, step2);
        c2 = sub2_rn(fma2_rn(a2, r2, s2), one2);
        cz = __fsub_rn(__fmaf_rn(a2.x, R.rzi, R.sz), 1.0f);
    };
    // two steps per iteration and one drain site: at most 64 runs are pushed before the ring is
    // settled, so it holds 128. A step past warp_steps closes and opens nothing (every lane has
    // closed its last run by then).
    for (int it = 0; it < warp_steps; it += 2) {
        march_step(it);
        march_step(it + 1);
        settle();
    }
    alpha = alpha_end;
    single(last_half);
    __syncwarp();
    drain(head, queued);
    __syncwarp();
    drain_mixed<M>(P, sh, lane, mhead, mqueued);

    if (do_pose) {
        // the warp's pose sums: each ray's moment r x (A^T hk), then one atomic per component
        __syncwarp();
        float Hs0 = sh.pose[0][lane], Hs1 = sh.pose[1][lane], Hs2 = sh.pose[2][lane];
        float Cs0 = sh.pose[3][lane], Cs1 = sh.pose[4][lane], Cs2 = sh.pose[5][lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            Hs0 += __shfl_xor_sync(kAll, Hs0, o);
            Hs1 += __shfl_xor_sync(kAll, Hs1, o);
            Hs2 += __shfl_xor_sync(kAll, Hs2, o);
            Cs0 += __shfl_xor_sync(kAll, Cs0, o);
            Cs1 += __shfl_xor_sync(kAll, Cs1, o);
            Cs2 += __shfl_xor_sync(kAll, Cs2, o);
        }
        if (lane == 0) {
            const float *A = sh.A;
            {  // the rays' moments in world coordinates: A^T (sum of m) / det A
                const float det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                                  A[2] * (A[3] * A[7] - A[4] * A[6]);
                const float id = 1.0f / det;
                const float m0 = Cs0, m1 = Cs1, m2 = Cs2;
                Cs0 = id * (A[0] * m0 + A[3] * m1 + A[6] * m2);
                Cs1 = id * (A[1] * m0 + A[4] * m1 + A[7] * m2);
                Cs2 = id * (A[2] * m0 + A[5] * m1 + A[8] * m2);
            }
            const float Hw[3] = {A[0] * Hs0 + A[3] * Hs1 + A[6] * Hs2, A[1] * Hs0 + A[4] * Hs1 + A[7] * Hs2,
                                 A[2] * Hs0 + A[5] * Hs1 + A[8] * Hs2};
            const float d[3] = {av.source_world[0] - P.center[0], av.source_world[1] - P.center[1],
                                av.source_world[2] - P.center[2]};
            const float pose[6] = {-Hw[0], -Hw[1], -Hw[2], -((d[1] * Hw[2] - d[2] * Hw[1]) + Cs0),
                                   -((d[2] * Hw[0] - d[0] * Hw[2]) + Cs1), -((d[0] * Hw[1] - d[1] * Hw[0]) + Cs2)};
#pragma unroll
            for (int k = 0; k < 6; k++)
                if (pose[k] != 0.0f) atomicAdd(P.grad_pose + (size_t)zv * 6 + k, pose[k]);
        }
    }
}

template <int M>
cudaError_t launch_adjoint(const AdjointParams &p, cudaStream_t stream);

}  // namespace drr
