// drr_coincide.h -- where two volumes' label-cache keys can coincide along a ray.
//
// The reference keeps one label cache for all volumes, keyed by the last voxel base any enabled
// volume moved it to (deepdrr/projector/project_kernel.cu:394-431); a volume whose base equals the
// key reads the cached labels, even if another volume's labels filled them. Along one ray, volume
// i's sample position is p_i(alpha) = s_i + alpha r_i - 1 in its own IJK frame (float32 in the
// kernel), so two volumes' bases can only be equal where every component of p_v - p_u, an affine
// function of alpha, is within a voxel; the key a volume meets can also be the previous step's,
// which widens the band by one step along the ray. coincidence_range returns an alpha interval
// outside which no two enabled volumes' bases can coincide at the same or at consecutive steps:
// the hull of one interval per pair, with 0.05 voxel of slack for float32 rounding and one step of
// padding on each side. Plain C++ so the kernel and the CPU test share it.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define DRR_CO_HD __host__ __device__ __forceinline__
#else
#define DRR_CO_HD inline
#endif

namespace drr {

// s[i][3]: volume i's source position in its IJK frame; r[i][3]: the unit ray in that frame.
// Writes [*lo, *hi] (empty when *lo > *hi). The arithmetic is float32 (float64 is a small fraction
// of float32's rate on the GPUs this runs on, and this runs once per ray): its rounding moves the
// band's edges by a few ulps of |s| and |alpha (r_v - r_u)|, below 3e-3 voxel for positions up to
// 10^4 voxels, far inside the 0.05 voxel of slack; a reciprocal stands in for two divisions.
DRR_CO_HD void coincidence_range(int nv, const bool *enabled, const float (*s)[3], const float (*r)[3], float step,
                                 double *lo_out, double *hi_out) {
    const float inf = INFINITY;
    float dlo = inf, dhi = -inf;
    for (int u = 0; u < nv; u++) {
        if (!enabled[u]) continue;
        for (int v = u + 1; v < nv; v++) {
            if (!enabled[v]) continue;
            float lo = -inf, hi = inf;
            for (int ax = 0; ax < 3; ax++) {
                // |(s_v - s_u) + alpha (r_v - r_u)| < band on this axis
                const float a = s[v][ax] - s[u][ax];
                const float b = r[v][ax] - r[u][ax];
                const float band = 1.05f + step * fmaxf(fabsf(r[u][ax]), fabsf(r[v][ax]));
                if (fabsf(b) < 1e-30f) {  // parallel on this axis: always or never within the band
                    if (!(fabsf(a) < band)) lo = inf, hi = -inf;
                } else {
                    const float ib = 1.0f / b;  // |ib| <= 1e30: the products below stay finite
                    const float x0 = (-band - a) * ib, x1 = (band - a) * ib;
                    lo = fmaxf(lo, fminf(x0, x1));
                    hi = fminf(hi, fmaxf(x0, x1));
                }
            }
            if (lo <= hi) {
                dlo = fminf(dlo, lo - step);
                dhi = fmaxf(dhi, hi + step);
            }
        }
    }
    *lo_out = (double)dlo;
    *hi_out = (double)dhi;
}

}  // namespace drr
