/*
 * drr_oracle.c -- CPU restatement of the DeepDRR volume projector.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle that the GPU kernels are checked against. Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it; the product library
 * never links, loads or calls it.
 *
 * It restates `projectKernel` of deepdrr v1.2.2, deepdrr/projector/project_kernel.cu:
 *   ray setup                 project_kernel.cu:195-234
 *   per-volume slab test      project_kernel.cu:265-323
 *   step count                project_kernel.cu:334
 *   march (labels, priority,  project_kernel.cu:398-553
 *          density, weights)
 *   air tails, step, mm->cm   project_kernel.cu:358-361, 557-584
 *   polychromatic attenuation project_kernel.cu:637-646
 * with the host preparation of deepdrr/projector/projector.py:802-831 (float64 host math cast to
 * float32, done by the caller of this file) and projector.py:1626-1634 (IJK boxes [-0.5, n-0.5]).
 *
 * Modes:
 *   ORC_MODE_F32  the reference's float32 arithmetic step by step: float32 `alpha += step`, the -1
 *                 voxel offset of both fields, the label cache shared by all volumes, the trapezoid
 *                 half weights at t = 0 and t = num_steps-1, fetch-then-range-check order, the
 *                 float64 air-density additions, and the texture unit's filtering emulated by
 *                 tex_linear() with `frac_bits` fractional bits in the filter weights (8 on NVIDIA
 *                 hardware; 0 = exact weights). Multiply-adds are written as fmaf() at the same
 *                 places as the GPU kernel of this project writes __fmaf_rn().
 *   ORC_MODE_F64  the same algorithm in double precision with exact trilinear weights and
 *                 alpha_t = minAlpha + t*step (no accumulation drift): the ideal value of the
 *                 reference's stepping rule, used for error statements.
 *
 * Deviation, stated: the reference samples disabled volumes with uninitialised ray directions
 * (project_kernel.cu:265-270 skip their setup, :398-456 still sample them). Disabled volumes are
 * ignored here entirely, and the label cache starts as label 0 where the reference leaves it
 * uninitialised (project_kernel.cu:394).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_VOL 8
#define ORC_MAX_MAT 16
#define ORC_AIR_DENSITY 0.1129 /* project_kernel.cu:5-7, a double literal */
#define ORC_MAX_STEPS (1 << 26) /* longer rays are reported as NaN instead of marched */

enum { ORC_MODE_F32 = 0, ORC_MODE_F64 = 1 };

typedef struct {
    int ni, nj, nk;            /* texture extent: x = i (fastest), y = j, z = k */
    const float *density;      /* [nk][nj][ni] */
    const uint8_t *labels;     /* [nk][nj][ni], values are material indices */
    int priority;
    int enabled;
    /* float32 per-view geometry exactly as the reference host passes it (projector.py:802-831) */
    float ijk_from_world[12];  /* 3x4 row-major */
    float source_ijk[3];
    /* float64 per-view geometry for ORC_MODE_F64 */
    double ijk_from_world_d[12];
    double source_ijk_d[3];
    int half_filter;           /* density held in a float16 texture: the filtered sample is a float16 */
} orc_volume;

/* IEEE binary16 round-to-nearest-even of x (what a float16 texture returns after filtering). */
static double round_to_half(double x) {
    if (x == 0.0 || !isfinite(x)) return x;
    double ax = fabs(x);
    int e;
    frexp(ax, &e); /* ax in [2^(e-1), 2^e) */
    int ex = e - 1;
    if (ex < -14) ex = -14; /* subnormal spacing 2^-24 */
    double ulp = ldexp(1.0, ex - 10);
    double r = nearbyint(ax / ulp) * ulp;
    if (r > 65504.0) r = INFINITY;
    return x < 0 ? -r : r;
}

typedef struct {
    int n_volumes;
    int n_materials;
    orc_volume vol[ORC_MAX_VOL];
    float world_from_index[9];     /* 3x3 row-major, float32 */
    double world_from_index_d[9];  /* float64 */
    float max_ray_length;          /* <= 0: unlimited (project_kernel.cu:285) */
    float step;                    /* world units (mm) */
    int width, height;
    int n_bins;
    const float *energies;         /* [n_bins], keV */
    const float *pdf;              /* [n_bins] */
    const float *mu;               /* [n_bins][n_materials], cm^2/g */
    int attenuate_outside;
    int air_index;
    int frac_bits;                 /* linear-filter weight precision in ORC_MODE_F32 (0 = exact) */
    int fp_profile;                /* multiply-add grouping of ORC_MODE_F32, see dot3_* below */
} orc_scene;

/* Multiply-add groupings of the float32 dot products of the ray setup. The reference kernel's
 * arithmetic is whatever grouping nvcc chose when it contracted a*b + c*d + e into FMAs; the
 * grouping is selected by `fp_profile` (bits 0-1: pixel ray, 2-3: squared norm, 4-5: IJK
 * direction, 6: sample position, 7: label-weight accumulation seg += xy * z as one fma) and
 * pinned against the reference kernel by the GPU tests. */
static inline float ray3(int mode, float u, float w0, float v, float w1, float w2) {
    switch (mode) {
        case 0: return fmaf(u, w0, fmaf(v, w1, w2));
        case 1: return fmaf(u, w0, v * w1) + w2;
        case 2: return fmaf(v, w1, u * w0) + w2;
        default: return (u * w0 + v * w1) + w2;
    }
}
static inline float norm2(int mode, float x, float y, float z) {
    switch (mode) {
        case 0: return fmaf(x, x, fmaf(y, y, z * z));
        case 1: return fmaf(z, z, fmaf(x, x, y * y));
        case 2: return fmaf(x, x, y * y) + z * z;
        default: return fmaf(z, z, fmaf(y, y, x * x));
    }
}
static inline float dot3(int mode, float a0, float x, float a1, float y, float a2, float z) {
    switch (mode) {
        case 0: return fmaf(a0, x, fmaf(a1, y, a2 * z));
        case 1: return fmaf(a2, z, fmaf(a0, x, a1 * y));
        case 2: return fmaf(a0, x, a1 * y) + a2 * z;
        default: return fmaf(a2, z, fmaf(a1, y, a0 * x));
    }
}
static inline float sample_pos(int mode, float alpha, float r, float s) {
    return mode == 0 ? fmaf(alpha, r, s) - 1.0f : (s + alpha * r) - 1.0f;
}

static inline int clamp_index(double f, int n) {
    /* clamp addressing of an unnormalised texture coordinate already floored */
    if (!(f >= 0.0)) return 0; /* also NaN */
    if (f > (double)(n - 1)) return n - 1;
    return (int)f;
}

static inline size_t vidx(const orc_volume *v, int i, int j, int k) {
    return ((size_t)k * (size_t)v->nj + (size_t)j) * (size_t)v->ni + (size_t)i;
}

/* cudaFilterModePoint, clamp, unnormalised coordinates: texel floor(x). */
static inline int tex_point(const orc_volume *v, double x, double y, double z) {
    int i = clamp_index(floor(x), v->ni);
    int j = clamp_index(floor(y), v->nj);
    int k = clamp_index(floor(z), v->nk);
    return (int)v->labels[vidx(v, i, j, k)];
}

static inline double quantize_weight(double a, int frac_bits) {
    if (frac_bits <= 0) return a;
    double s = ldexp(1.0, frac_bits);
    return floor(a * s + 0.5) / s;
}

/* Corner weights of the texture unit's 3D linear filter, in units of 1/256, from the per-axis
 * fractions Ax, Ay, Az in [0, 256] (each frac(x - 0.5) rounded to the nearest 1/256). Measured on
 * the GPU with one-hot 2x2x2 textures (tests/test_gpu_parity.py pins it): the z split is exact,
 * the x split rounds the upper branch half-up, and the y split rounds half-up the upper branch of
 * the dx = 1 columns and the lower branch of the dx = 0 columns. Corner c = dx | dy << 1 | dz << 2;
 * the eight weights always sum to 256. */
static void hw_corner_weights(int Ax, int Ay, int Az, int W[8]) {
    for (int dz = 0; dz <= 1; dz++) {
        int vz = dz ? Az : 256 - Az;
        int hx = (vz * Ax + 128) >> 8;
        for (int dx = 0; dx <= 1; dx++) {
            int vx = dx ? hx : vz - hx;
            int hy = dx ? (vx * Ay + 128) >> 8 : vx - ((vx * (256 - Ay) + 128) >> 8);
            W[dx | 2 | (dz << 2)] = hy;
            W[dx | (dz << 2)] = vx - hy;
        }
    }
}

/* cudaFilterModeLinear, clamp, unnormalised coordinates (CUDA Programming Guide, "Texture
 * Fetching", linear filtering): xB = x - 0.5, i = floor(xB), alpha = frac(xB), value = blend of
 * texels i and i+1 on each axis. frac_bits = 8 models NVIDIA's texture unit: 8-bit per-axis
 * fractions combined into 8-bit corner weights (hw_corner_weights), the blend summed exactly and
 * rounded once to float32 by the caller. frac_bits = 0 blends with exact weights. */
static double tex_linear(const orc_volume *v, double x, double y, double z, int frac_bits) {
    double xb = x - 0.5, yb = y - 0.5, zb = z - 0.5;
    if (frac_bits == 8) {
        /* the texture unit clamps the coordinate itself to [0, n-1] (texel-centre space) before
         * splitting it into a texel index and a fraction; this matters through the staged
         * rounding of the corner weights */
        xb = xb < 0.0 ? 0.0 : (xb > v->ni - 1.0 ? v->ni - 1.0 : xb);
        yb = yb < 0.0 ? 0.0 : (yb > v->nj - 1.0 ? v->nj - 1.0 : yb);
        zb = zb < 0.0 ? 0.0 : (zb > v->nk - 1.0 ? v->nk - 1.0 : zb);
    }
    const float *T = v->density;
    if (frac_bits == 8) {
        /* fixed point with 8 fractional bits: fix = round(xB * 256), texel fix >> 8, weight fix & 255
         * (a fraction that rounds up to 1 carries into the next texel with weight 0) */
        const long fx = (long)floor(xb * 256.0 + 0.5), fy = (long)floor(yb * 256.0 + 0.5), fz = (long)floor(zb * 256.0 + 0.5);
        const int ii[2] = {(int)(fx >> 8), clamp_index((double)((fx >> 8) + 1), v->ni)};
        const int jj[2] = {(int)(fy >> 8), clamp_index((double)((fy >> 8) + 1), v->nj)};
        const int kk[2] = {(int)(fz >> 8), clamp_index((double)((fz >> 8) + 1), v->nk)};
        int W[8];
        hw_corner_weights((int)(fx & 255), (int)(fy & 255), (int)(fz & 255), W);
        double s = 0.0;
        for (int c = 0; c < 8; c++) s += (double)W[c] * (double)T[vidx(v, ii[c & 1], jj[(c >> 1) & 1], kk[c >> 2])];
        return s / 256.0;
    }
    double fi = floor(xb), fj = floor(yb), fk = floor(zb);
    int i0 = clamp_index(fi, v->ni), i1 = clamp_index(fi + 1.0, v->ni);
    int j0 = clamp_index(fj, v->nj), j1 = clamp_index(fj + 1.0, v->nj);
    int k0 = clamp_index(fk, v->nk), k1 = clamp_index(fk + 1.0, v->nk);
    double a = quantize_weight(xb - fi, frac_bits);
    double b = quantize_weight(yb - fj, frac_bits);
    double c = quantize_weight(zb - fk, frac_bits);
    double c00 = (1 - a) * T[vidx(v, i0, j0, k0)] + a * T[vidx(v, i1, j0, k0)];
    double c10 = (1 - a) * T[vidx(v, i0, j1, k0)] + a * T[vidx(v, i1, j1, k0)];
    double c01 = (1 - a) * T[vidx(v, i0, j0, k1)] + a * T[vidx(v, i1, j0, k1)];
    double c11 = (1 - a) * T[vidx(v, i0, j1, k1)] + a * T[vidx(v, i1, j1, k1)];
    double c0 = (1 - b) * c00 + b * c10;
    double c1 = (1 - b) * c01 + b * c11;
    return (1 - c) * c0 + c * c1;
}

static inline int float_to_int_sat(float x) {
    /* cvt.rzi.s32.f32 semantics: NaN -> 0, saturating */
    if (x != x) return 0;
    if (x >= 2147483647.0f) return INT_MAX;
    if (x <= -2147483648.0f) return INT_MIN;
    return (int)x;
}

/* Apply the polychromatic Beer-Lambert sum of project_kernel.cu:637-646. */
static void attenuate_f32(const orc_scene *sc, const float *ad, float *I, float *P) {
    const int M = sc->n_materials;
    float inten = 0.0f, prob = 0.0f;
    for (int bin = 0; bin < sc->n_bins; bin++) {
        float x = 0.0f;
        for (int m = 0; m < M; m++) x = fmaf(ad[m], sc->mu[bin * M + m], x);
        float p = expf(-1.0f * x) * sc->pdf[bin];
        prob += p;
        inten = fmaf(sc->energies[bin], p, inten);
    }
    *I = inten;
    *P = prob;
}

/* One ray in the reference's float32 arithmetic. ad_out receives the per-material area densities
 * in g/cm^2 (project_kernel.cu:558-584). Returns the number of samples (t, volume) with the volume
 * traced, enabled and alpha inside its interval. */
/* Optional record of the samples of one single-volume ray (orc_ray_samples_f32). */
typedef struct {
    float *alpha, *p, *w;
    int cap, n;
} orc_rec;

static double ray_f32(const orc_scene *sc, int u, int v, float *ad_out, float *I, float *P, orc_rec *rec) {
    const int NV = sc->n_volumes, M = sc->n_materials;
    const float *W = sc->world_from_index;
    const float step = sc->step;
    float uf = (float)((double)u + 0.5);
    float vf = (float)((double)v + 0.5);
    const int pr_ray = sc->fp_profile & 3, pr_norm = (sc->fp_profile >> 2) & 3;
    const int pr_dir = (sc->fp_profile >> 4) & 3, pr_pos = (sc->fp_profile >> 6) & 1;
    const int pr_seg = (sc->fp_profile >> 7) & 1;
    float rx = ray3(pr_ray, uf, W[0], vf, W[1], W[2]);
    float ry = ray3(pr_ray, uf, W[3], vf, W[4], W[5]);
    float rz = ray3(pr_ray, uf, W[6], vf, W[7], W[8]);
    float ray_length = sqrtf(norm2(pr_norm, rx, ry, rz));
    float inv = 1.0f / ray_length;
    rx *= inv;
    ry *= inv;
    rz *= inv;

    float minA = ray_length, maxA = 0.0f;
    float minv[ORC_MAX_VOL], maxv[ORC_MAX_VOL];
    float rxi[ORC_MAX_VOL], ryi[ORC_MAX_VOL], rzi[ORC_MAX_VOL];
    int trace[ORC_MAX_VOL];
    for (int i = 0; i < NV; i++) {
        const orc_volume *V = &sc->vol[i];
        trace[i] = 0;
        if (!V->enabled) continue;
        const float *A = V->ijk_from_world;
        rxi[i] = dot3(pr_dir, A[0], rx, A[1], ry, A[2], rz);
        ryi[i] = dot3(pr_dir, A[4], rx, A[5], ry, A[6], rz);
        rzi[i] = dot3(pr_dir, A[8], rx, A[9], ry, A[10], rz);
        const float r3[3] = {rxi[i], ryi[i], rzi[i]};
        const float hi[3] = {(float)(V->ni - 0.5), (float)(V->nj - 0.5), (float)(V->nk - 0.5)};
        const float lo = -0.5f;
        float mn = 0.0f, mx = sc->max_ray_length > 0.0f ? sc->max_ray_length : INFINITY;
        int ok = 1;
        for (int ax = 0; ax < 3; ax++) {
            float s = V->source_ijk[ax];
            if (0.0f != r3[ax]) {
                float reci = 1.0f / r3[ax];
                float a0 = (lo - s) * reci;
                float a1 = (hi[ax] - s) * reci;
                mn = fmaxf(mn, fminf(a0, a1));
                mx = fminf(mx, fmaxf(a0, a1));
            } else if (lo > s || s > hi[ax]) {
                ok = 0;
                break;
            }
        }
        minv[i] = mn;
        maxv[i] = mx;
        if (!ok) continue; /* do_trace = 0, global range not updated (project_kernel.cu:292-294) */
        trace[i] = 1;
        minA = fminf(minA, mn);
        maxA = fmaxf(maxA, mx);
    }
    float span_steps = ceilf((maxA - minA) / step);
    if (span_steps > (float)ORC_MAX_STEPS || span_steps != span_steps) {
        /* non-finite or absurd geometry: reported as NaN (the product kernel does the same) */
        for (int m = 0; m < M; m++) ad_out[m] = NAN;
        *I = NAN;
        *P = NAN;
        return 0.0;
    }
    int num_steps = float_to_int_sat(span_steps);

    float ad[ORC_MAX_MAT];
    for (int m = 0; m < M; m++) ad[m] = 0.0f;
    if (sc->attenuate_outside)
        ad[sc->air_index] = (float)((double)ad[sc->air_index] + (double)(minA / step) * ORC_AIR_DENSITY);

    float px[ORC_MAX_VOL], py[ORC_MAX_VOL], pz[ORC_MAX_VOL];
    float seg[ORC_MAX_VOL][ORC_MAX_MAT];
    float prev[3] = {-1.0f, -1.0f, -1.0f};
    int vox[8] = {0, 0, 0, 0, 0, 0, 0, 0}; /* [dz][dy][dx] */
    float alpha = minA;
    double nsamp = 0.0;
    for (int t = 0; t < num_steps; t++) {
        for (int vol = 0; vol < NV; vol++) {
            const orc_volume *V = &sc->vol[vol];
            if (!V->enabled) continue;
            px[vol] = sample_pos(pr_pos, alpha, rxi[vol], V->source_ijk[0]);
            py[vol] = sample_pos(pr_pos, alpha, ryi[vol], V->source_ijk[1]);
            pz[vol] = sample_pos(pr_pos, alpha, rzi[vol], V->source_ijk[2]);
            for (int m = 0; m < M; m++) seg[vol][m] = 0.0f;
            float bx = floorf(px[vol]), by = floorf(py[vol]), bz = floorf(pz[vol]);
            if (bx != prev[0] || by != prev[1] || bz != prev[2]) {
                for (int dz = 0; dz <= 1; dz++)
                    for (int dy = 0; dy <= 1; dy++)
                        for (int dx = 0; dx <= 1; dx++)
                            vox[dz * 4 + dy * 2 + dx] = tex_point(V, (double)(px[vol] + (float)dx),
                                                                  (double)(py[vol] + (float)dy),
                                                                  (double)(pz[vol] + (float)dz));
                prev[0] = bx;
                prev[1] = by;
                prev[2] = bz;
            }
            float fx = px[vol] - bx, fy = py[vol] - by, fz = pz[vol] - bz;
            float gx = 1.0f - fx, gy = 1.0f - fy, gz = 1.0f - fz;
            /* xy products, then one z factor per corner (project_kernel.cu:441-448) */
            const float xy[4] = {gx * gy, fx * gy, gx * fy, fx * fy};
            const float zf[2] = {gz, fz};
            for (int c = 0; c < 8; c++) {
                int lab = vox[c];
                if (lab < 0 || lab >= M) continue;
                if (pr_seg) /* seg += xy * z contracted into one fma */
                    seg[vol][lab] = fmaf(xy[c & 3], zf[c >> 2], seg[vol][lab]);
                else
                    seg[vol][lab] += xy[c & 3] * zf[c >> 2];
            }
        }
        int cur = NV, n = 0;
        for (int i = 0; i < NV; i++) {
            if (!trace[i] || !sc->vol[i].enabled) continue;
            if (alpha < minv[i] || alpha > maxv[i]) continue;
            float any = 0.0f;
            for (int m = 0; m < M; m++) {
                any += seg[i][m];
                if (any > 0.0f) break;
            }
            if (0.0f == any) continue;
            nsamp += 1.0;
            int pr = sc->vol[i].priority;
            if (pr < cur) {
                cur = pr;
                n = 1;
            } else if (pr == cur) {
                n += 1;
            }
        }
        if (n == 0) {
            if (sc->attenuate_outside)
                ad[sc->air_index] = (float)((double)ad[sc->air_index] + ORC_AIR_DENSITY);
        } else {
            float weight = 1.0f / (float)n;
            weight *= (0 == t || num_steps - 1 == t) ? 0.5f : 1.0f;
            for (int vol = 0; vol < NV; vol++) {
                const orc_volume *V = &sc->vol[vol];
                /* no range re-check here: project_kernel.cu:541 */
                if (trace[vol] && V->priority == cur && V->enabled) {
                    double rho_d = tex_linear(V, (double)(px[vol] + 0.5f), (double)(py[vol] + 0.5f),
                                              (double)(pz[vol] + 0.5f), sc->frac_bits);
                    float rho = (float)(V->half_filter ? round_to_half(rho_d) : rho_d);
                    float wr = weight * rho;
                    for (int m = 0; m < M; m++) ad[m] = fmaf(wr, seg[vol][m], ad[m]);
                    if (rec && rec->n < rec->cap) {
                        rec->alpha[rec->n] = alpha;
                        rec->p[3 * rec->n] = px[vol];
                        rec->p[3 * rec->n + 1] = py[vol];
                        rec->p[3 * rec->n + 2] = pz[vol];
                        rec->w[rec->n] = weight;
                        rec->n++;
                    }
                }
            }
        }
        alpha += step;
    }
    if (sc->attenuate_outside)
        ad[sc->air_index] =
            (float)((double)ad[sc->air_index] + (double)((ray_length - maxA) / step) * ORC_AIR_DENSITY);
    for (int m = 0; m < M; m++) ad[m] *= step;
    for (int m = 0; m < M; m++) ad[m] /= 10.0f;
    for (int m = 0; m < M; m++) ad_out[m] = ad[m];
    attenuate_f32(sc, ad, I, P);
    return nsamp;
}

/* One ray of the same algorithm in float64 with exact weights and undrifted alpha. */
static double ray_f64(const orc_scene *sc, int u, int v, double *ad_out, double *I, double *P) {
    const int NV = sc->n_volumes, M = sc->n_materials;
    const double *W = sc->world_from_index_d;
    const double step = (double)sc->step;
    double uu = u + 0.5, vv = v + 0.5;
    double rx = uu * W[0] + vv * W[1] + W[2];
    double ry = uu * W[3] + vv * W[4] + W[5];
    double rz = uu * W[6] + vv * W[7] + W[8];
    double ray_length = sqrt(rx * rx + ry * ry + rz * rz);
    rx /= ray_length;
    ry /= ray_length;
    rz /= ray_length;
    double minA = ray_length, maxA = 0.0;
    double minv[ORC_MAX_VOL], maxv[ORC_MAX_VOL], rxi[ORC_MAX_VOL], ryi[ORC_MAX_VOL], rzi[ORC_MAX_VOL];
    int trace[ORC_MAX_VOL];
    for (int i = 0; i < NV; i++) {
        const orc_volume *V = &sc->vol[i];
        trace[i] = 0;
        if (!V->enabled) continue;
        const double *A = V->ijk_from_world_d;
        rxi[i] = A[0] * rx + A[1] * ry + A[2] * rz;
        ryi[i] = A[4] * rx + A[5] * ry + A[6] * rz;
        rzi[i] = A[8] * rx + A[9] * ry + A[10] * rz;
        const double r3[3] = {rxi[i], ryi[i], rzi[i]};
        const double hi[3] = {V->ni - 0.5, V->nj - 0.5, V->nk - 0.5};
        double mn = 0.0, mx = sc->max_ray_length > 0.0f ? (double)sc->max_ray_length : INFINITY;
        int ok = 1;
        for (int ax = 0; ax < 3; ax++) {
            double s = V->source_ijk_d[ax];
            if (0.0 != r3[ax]) {
                double a0 = (-0.5 - s) / r3[ax], a1 = (hi[ax] - s) / r3[ax];
                mn = fmax(mn, fmin(a0, a1));
                mx = fmin(mx, fmax(a0, a1));
            } else if (-0.5 > s || s > hi[ax]) {
                ok = 0;
                break;
            }
        }
        minv[i] = mn;
        maxv[i] = mx;
        if (!ok) continue;
        trace[i] = 1;
        minA = fmin(minA, mn);
        maxA = fmax(maxA, mx);
    }
    double nsd = ceil((maxA - minA) / step);
    if (nsd > (double)ORC_MAX_STEPS || nsd != nsd) {
        for (int m = 0; m < M; m++) ad_out[m] = NAN;
        *I = NAN;
        *P = NAN;
        return 0.0;
    }
    long num_steps = nsd > 0 ? (long)nsd : 0;
    double ad[ORC_MAX_MAT];
    for (int m = 0; m < M; m++) ad[m] = 0.0;
    if (sc->attenuate_outside) ad[sc->air_index] += minA / step * ORC_AIR_DENSITY;
    double px[ORC_MAX_VOL], py[ORC_MAX_VOL], pz[ORC_MAX_VOL];
    double seg[ORC_MAX_VOL][ORC_MAX_MAT];
    double prev[3] = {-1.0, -1.0, -1.0};
    int vox[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double nsamp = 0.0;
    for (long t = 0; t < num_steps; t++) {
        double alpha = minA + (double)t * step;
        for (int vol = 0; vol < NV; vol++) {
            const orc_volume *V = &sc->vol[vol];
            if (!V->enabled) continue;
            px[vol] = V->source_ijk_d[0] + alpha * rxi[vol] - 1.0;
            py[vol] = V->source_ijk_d[1] + alpha * ryi[vol] - 1.0;
            pz[vol] = V->source_ijk_d[2] + alpha * rzi[vol] - 1.0;
            for (int m = 0; m < M; m++) seg[vol][m] = 0.0;
            double bx = floor(px[vol]), by = floor(py[vol]), bz = floor(pz[vol]);
            if (bx != prev[0] || by != prev[1] || bz != prev[2]) {
                for (int dz = 0; dz <= 1; dz++)
                    for (int dy = 0; dy <= 1; dy++)
                        for (int dx = 0; dx <= 1; dx++)
                            vox[dz * 4 + dy * 2 + dx] = tex_point(V, bx + dx, by + dy, bz + dz);
                prev[0] = bx;
                prev[1] = by;
                prev[2] = bz;
            }
            double fx = px[vol] - bx, fy = py[vol] - by, fz = pz[vol] - bz;
            double gx = 1 - fx, gy = 1 - fy, gz = 1 - fz;
            double w[8] = {gx * gy * gz, fx * gy * gz, gx * fy * gz, fx * fy * gz,
                           gx * gy * fz, fx * gy * fz, gx * fy * fz, fx * fy * fz};
            for (int c = 0; c < 8; c++) {
                int lab = vox[c];
                if (lab >= 0 && lab < M) seg[vol][lab] += w[c];
            }
        }
        int cur = NV, n = 0;
        for (int i = 0; i < NV; i++) {
            if (!trace[i] || !sc->vol[i].enabled) continue;
            if (alpha < minv[i] || alpha > maxv[i]) continue;
            double any = 0.0;
            for (int m = 0; m < M; m++) any += seg[i][m];
            if (0.0 == any) continue;
            nsamp += 1.0;
            int pr = sc->vol[i].priority;
            if (pr < cur) {
                cur = pr;
                n = 1;
            } else if (pr == cur) {
                n += 1;
            }
        }
        if (n == 0) {
            if (sc->attenuate_outside) ad[sc->air_index] += ORC_AIR_DENSITY;
        } else {
            double weight = 1.0 / n;
            if (0 == t || num_steps - 1 == t) weight *= 0.5;
            for (int vol = 0; vol < NV; vol++) {
                const orc_volume *V = &sc->vol[vol];
                if (trace[vol] && V->priority == cur && V->enabled) {
                    double rho = tex_linear(V, px[vol] + 0.5, py[vol] + 0.5, pz[vol] + 0.5, 0);
                    for (int m = 0; m < M; m++) ad[m] += weight * rho * seg[vol][m];
                }
            }
        }
    }
    if (sc->attenuate_outside) ad[sc->air_index] += (ray_length - maxA) / step * ORC_AIR_DENSITY;
    for (int m = 0; m < M; m++) ad_out[m] = ad[m] * step / 10.0;
    double inten = 0.0, prob = 0.0;
    for (int bin = 0; bin < sc->n_bins; bin++) {
        double x = 0.0;
        for (int m = 0; m < M; m++) x += ad_out[m] * (double)sc->mu[bin * M + m];
        double p = exp(-x) * (double)sc->pdf[bin];
        prob += p;
        inten += (double)sc->energies[bin] * p;
    }
    *I = inten;
    *P = prob;
    return nsamp;
}

/*
 * Project the rays `ray_ids` (flat pixel indices v*width+u; NULL = all width*height rays in
 * row-major order). Outputs are indexed by the position of the ray in that list:
 *   intensity[r], photon_prob[r]              float (ORC_MODE_F32) or double (ORC_MODE_F64)
 *   area_density[m * n_rays + r]              same type; may be NULL
 * Returns the total sample count through *samples (may be NULL). Returns 0, or -1 on bad input.
 */
int orc_project(const orc_scene *sc, int mode, const int64_t *ray_ids, int64_t n_rays, void *intensity,
                void *photon_prob, void *area_density, double *samples, int n_threads) {
    if (!sc || sc->n_volumes < 0 || sc->n_volumes > ORC_MAX_VOL || sc->n_materials < 1 ||
        sc->n_materials > ORC_MAX_MAT || sc->width < 1 || sc->height < 1)
        return -1;
    if (sc->attenuate_outside && (sc->air_index < 0 || sc->air_index >= sc->n_materials)) return -1;
    const int64_t total = ray_ids ? n_rays : (int64_t)sc->width * sc->height;
    const int M = sc->n_materials;
    double nsamp = 0.0;
#ifdef _OPENMP
    if (n_threads < 1) n_threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(n_threads) reduction(+ : nsamp)
#endif
    for (int64_t r = 0; r < total; r++) {
        int64_t pix = ray_ids ? ray_ids[r] : r;
        int u = (int)(pix % sc->width), v = (int)(pix / sc->width);
        if (mode == ORC_MODE_F32) {
            float ad[ORC_MAX_MAT], I, P;
            nsamp += ray_f32(sc, u, v, ad, &I, &P, NULL);
            ((float *)intensity)[r] = I;
            ((float *)photon_prob)[r] = P;
            if (area_density)
                for (int m = 0; m < M; m++) ((float *)area_density)[(int64_t)m * total + r] = ad[m];
        } else {
            double ad[ORC_MAX_MAT], I, P;
            nsamp += ray_f64(sc, u, v, ad, &I, &P);
            ((double *)intensity)[r] = I;
            ((double *)photon_prob)[r] = P;
            if (area_density)
                for (int m = 0; m < M; m++) ((double *)area_density)[(int64_t)m * total + r] = ad[m];
        }
    }
    if (samples) *samples = nsamp;
    return 0;
}

/* The samples ORC_MODE_F32 takes along ray (u, v) of a single-volume scene: per contributing step
 * its float32 alpha, position p = (x, y, z) in the volume's shifted IJK frame (the -1 voxel offset
 * applied) and trapezoid weight, in march order. Returns how many were taken (at most `cap` are
 * written), or -1 for a scene with other than one volume. */
int orc_ray_samples_f32(const orc_scene *sc, int u, int v, float *alpha, float *p, float *w, int cap) {
    if (!sc || sc->n_volumes != 1) return -1;
    orc_rec rec = {alpha, p, w, cap, 0};
    float ad[ORC_MAX_MAT], I, P;
    double n = ray_f32(sc, u, v, ad, &I, &P, &rec);
    return n > (double)cap ? (int)n : rec.n;
}

/* Texture-filter emulation exposed for the tests that pin it against the GPU's texture unit. */
double orc_tex_linear(const orc_scene *sc, int vol, double x, double y, double z) {
    return tex_linear(&sc->vol[vol], x, y, z, sc->frac_bits);
}
int orc_tex_point(const orc_scene *sc, int vol, double x, double y, double z) {
    return tex_point(&sc->vol[vol], x, y, z);
}
int orc_max_volumes(void) { return ORC_MAX_VOL; }
int orc_max_materials(void) { return ORC_MAX_MAT; }
