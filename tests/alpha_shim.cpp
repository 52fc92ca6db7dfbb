// CPU shim over deepdrr_gb300/csrc/drr_alpha.h for test_alpha_cpu.py: the fast-forward used by the
// kernel and the serial float32 loop it replaces.
#include "../deepdrr_gb300/csrc/drr_alpha.h"

extern "C" int fast_forward(float *alpha, float step, float bound, int limit, int inclusive) {
    return drr::advance_alpha(alpha, step, bound, limit, inclusive != 0);
}

extern "C" int serial(float *alpha, float step, float bound, int limit, int inclusive) {
    volatile float a = *alpha;
    int k = 0;
    while (k < limit && (inclusive ? a <= bound : a < bound)) {
        a = a + step;
        ++k;
    }
    *alpha = a;
    return k;
}
