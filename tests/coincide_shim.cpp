// CPU shim over deepdrr_gb300/csrc/drr_coincide.h for test_coincide_cpu.py: the kernel's range and a
// brute-force float32 march that finds where two volumes' label-cache keys actually coincide.
#include "../deepdrr_gb300/csrc/drr_coincide.h"

#include <cmath>

// Positions as the kernel computes them: fma(alpha, r, s) - 1 in float32, floors of each volume in
// processing order. Counts steps where a volume's base equals the base of the volume processed just
// before it (same step, or the last enabled volume of the previous step) at an alpha outside
// [lo, hi]; returns that count (0 = the range covers every coincidence) and writes the number of
// coincidences seen.
extern "C" int check_range(int nv, const float *s, const float *r, float step, float alpha0, int nsteps,
                           int *coincidences) {
    bool en[4] = {true, true, true, true};
    float sv[4][3], rv[4][3];
    for (int i = 0; i < nv; i++)
        for (int k = 0; k < 3; k++) sv[i][k] = s[3 * i + k], rv[i][k] = r[3 * i + k];
    double lo, hi;
    drr::coincidence_range(nv, en, sv, rv, step, &lo, &hi);
    int outside = 0, seen = 0;
    float prev[3] = {NAN, NAN, NAN};
    volatile float alpha = alpha0;
    for (int t = 0; t < nsteps; t++) {
        for (int i = 0; i < nv; i++) {
            float b[3];
            for (int k = 0; k < 3; k++) {
                volatile float f = std::fma((float)alpha, rv[i][k], sv[i][k]);
                volatile float p = f - 1.0f;
                b[k] = std::floor((float)p);
            }
            const bool same = b[0] == prev[0] && b[1] == prev[1] && b[2] == prev[2];
            if (same && (t > 0 || i > 0)) {
                ++seen;
                if (!((double)alpha >= lo && (double)alpha <= hi)) ++outside;
            }
            prev[0] = b[0], prev[1] = b[1], prev[2] = b[2];
        }
        alpha = alpha + step;
    }
    *coincidences = seen;
    return outside;
}
