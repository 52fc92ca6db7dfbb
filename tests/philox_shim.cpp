// CPU shim over deepdrr_gb300/csrc/drr_philox.h for test_noise_cpu.py: the generator and the
// Poisson sampler compiled for the host from the same source the noise kernels use.
#include "../deepdrr_gb300/csrc/drr_philox.h"

extern "C" void philox(const unsigned *ctr, const unsigned *key, unsigned *out) {
    const drr::Ctr4 r = drr::philox4x32_10(drr::Ctr4{ctr[0], ctr[1], ctr[2], ctr[3]}, key[0], key[1]);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
    out[3] = r.w;
}

extern "C" void poisson_many(const float *lam, long long n, unsigned long long seed, float *out) {
    for (long long i = 0; i < n; i++) {
        drr::UniformStream u(seed, (unsigned long long)i);
        out[i] = (float)drr::poisson((double)lam[i], u);
    }
}
