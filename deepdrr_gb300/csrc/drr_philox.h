// drr_philox.h -- counter-based random numbers and Poisson variates for the detector noise model.
//
// Philox4x32-10 is the generator of Salmon, Moraes, Dror and Shaw, "Parallel random numbers: as
// easy as 1, 2, 3" (SC 2011): ten rounds of two 32x32->64-bit multiplies on a 128-bit counter under
// a 64-bit key that is bumped by the Weyl constants between rounds. Each value depends only on
// (key, counter), so a kernel can recompute a pixel's variate wherever it needs it (halo pixels of
// a convolution included) and the result does not depend on the launch shape.
//
// Poisson variates: inversion by sequential search below lambda = 10; above it the transformed
// rejection with squeeze of W. Hoermann, "The transformed rejection method for generating Poisson
// random variables", Insurance: Mathematics and Economics 12 (1993) 39-45 (algorithm PTRS).
//
// Plain C++ so the host build of the same code runs in the CPU tests (known-answer vectors).
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define DRR_RNG_HD __host__ __device__ __forceinline__
#else
#define DRR_RNG_HD inline
#endif

namespace drr {

struct Ctr4 {
    uint32_t x, y, z, w;
};

DRR_RNG_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
    const uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

DRR_RNG_HD Ctr4 philox4x32_10(Ctr4 c, uint32_t k0, uint32_t k1) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 0; r < 10; r++) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c.x, hi0, lo0);
        mulhilo32(0xCD9E8D57u, c.z, hi1, lo1);
        c = Ctr4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    }
    return c;
}

// A stream of uniforms in (0, 1) for one (key, element): counter (element lo, element hi, 0, block).
struct UniformStream {
    uint32_t k0, k1, e0, e1, block;
    uint32_t buf[4];
    int used;

    DRR_RNG_HD UniformStream(uint64_t key, uint64_t element)
        : k0((uint32_t)key), k1((uint32_t)(key >> 32)), e0((uint32_t)element), e1((uint32_t)(element >> 32)),
          block(0), used(4) {}

    // 24 random bits centred in their interval: never 0 or 1
    DRR_RNG_HD double next() {
        if (used == 4) {
            const Ctr4 r = philox4x32_10(Ctr4{e0, e1, 0u, block++}, k0, k1);
            buf[0] = r.x;
            buf[1] = r.y;
            buf[2] = r.z;
            buf[3] = r.w;
            used = 0;
        }
        return ((double)(buf[used++] >> 8) + 0.5) * (1.0 / 16777216.0);
    }
};

// Poisson(lambda) for lambda >= 0 (NaN for a negative or non-finite lambda). Every loop is bounded:
// the search stops at k = 1000 for lambda < 10 (tail probability below 1e-900), and PTRS gives up
// after 1000 rejections (each proposal is accepted with probability above 0.8) and returns the
// rounded mean.
DRR_RNG_HD double poisson(double lam, UniformStream &u) {
    if (!(lam >= 0.0) || lam > 1.0e300) return nan("");
    if (lam == 0.0) return 0.0;
    if (lam < 10.0) {
        const double x = u.next();
        double p = exp(-lam), F = p;
        int k = 0;
        while (x > F && k < 1000) {
            ++k;
            p *= lam / k;
            F += p;
        }
        return (double)k;
    }
    const double slam = sqrt(lam), loglam = log(lam);
    const double b = 0.931 + 2.53 * slam;
    const double a = -0.059 + 0.02483 * b;
    const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4);
    const double vr = 0.9277 - 3.6224 / (b - 2.0);
    for (int it = 0; it < 1000; it++) {
        const double U = u.next() - 0.5;
        const double V = u.next();
        const double us = 0.5 - fabs(U);
        const double k = floor((2.0 * a / us + b) * U + lam + 0.43);
        if (us >= 0.07 && V <= vr) return k;
        if (k < 0.0 || (us < 0.013 && V > us)) continue;
        if (log(V) + log(inv_alpha) - log(a / (us * us) + b) <= -lam + k * loglam - lgamma(k + 1.0)) return k;
    }
    return floor(lam + 0.5);
}

}  // namespace drr
