// drr_coincide.h -- where two volumes' label-cache keys can coincide along a ray.
//
// The reference keeps one label cache for all volumes, keyed by the last voxel base any enabled
// volume moved it to (deepdrr/projector/project_kernel.cu:394-431); a volume whose base equals the
// key reads the cached labels, even if another volume's labels filled them. Along one ray, volume
// i's sample position is p_i(alpha) = s_i + alpha r_i - 1 in its own IJK frame (float32 in the
// kernel), so two volumes' bases can only be equal where every component of p_v - p_u, an affine
// function of alpha, is within a voxel; the key a volume meets can also be the previous step's,
// which widens the band by one step along the ray. coincidence_range returns, in float64, an alpha
// interval outside which no two enabled volumes' bases can coincide at the same or at consecutive
// steps: the hull of one interval per pair, with 0.05 voxel of slack for float32 rounding and one
// step of padding on each side. Plain C++ so the kernel and the CPU test share it.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define DRR_CO_HD __host__ __device__ __forceinline__
#else
#define DRR_CO_HD inline
#endif

namespace drr {

// s[i][3]: volume i's source position in its IJK frame; r[i][3]: the unit ray in that frame.
// Writes [*lo, *hi] (empty when *lo > *hi).
DRR_CO_HD void coincidence_range(int nv, const bool *enabled, const float (*s)[3], const float (*r)[3], float step,
                                 double *lo_out, double *hi_out) {
    double dlo = 1e300, dhi = -1e300;
    for (int u = 0; u < nv; u++) {
        if (!enabled[u]) continue;
        for (int v = u + 1; v < nv; v++) {
            if (!enabled[v]) continue;
            double lo = -1e300, hi = 1e300;
            for (int ax = 0; ax < 3; ax++) {
                // |(s_v - s_u) + alpha (r_v - r_u)| < band on this axis
                const double a = (double)s[v][ax] - (double)s[u][ax];
                const double b = (double)r[v][ax] - (double)r[u][ax];
                const double band = 1.05 + (double)step * fmax(fabs((double)r[u][ax]), fabs((double)r[v][ax]));
                if (fabs(b) < 1e-12) {
                    if (!(fabs(a) < band)) lo = 1e300, hi = -1e300;
                } else {
                    const double x0 = (-band - a) / b, x1 = (band - a) / b;
                    lo = fmax(lo, fmin(x0, x1));
                    hi = fmin(hi, fmax(x0, x1));
                }
            }
            if (lo <= hi) {
                dlo = fmin(dlo, lo - (double)step);
                dhi = fmax(dhi, hi + (double)step);
            }
        }
    }
    *lo_out = dlo;
    *hi_out = dhi;
}

}  // namespace drr
