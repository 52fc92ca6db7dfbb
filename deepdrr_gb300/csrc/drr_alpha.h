// drr_alpha.h -- exact fast-forward of the reference's float32 ray parameter.
//
// The reference marches with `alpha += step` in float32 (deepdrr/projector/project_kernel.cu:552),
// so every sample position depends on the exact sequence of rounded additions. drr_advance_alpha
// reproduces that sequence without performing every addition: inside one binade of alpha the ulp u
// is fixed, so alpha + step rounds to alpha + delta with a constant integer number of ulps delta
// (round-to-nearest of step/u; on an exact tie the first addition makes alpha's last bit even and
// every later one adds the even neighbour of step/u). The helper jumps through each binade in one
// step and falls back to single additions near binade boundaries, for zero or subnormal alpha, and
// whenever a jump would not be provably exact. It is plain C++ so the same code runs in the kernel
// and in the CPU test that compares it with the serial loop.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define DRR_HD __host__ __device__ __forceinline__
#else
#define DRR_HD inline
#endif

namespace drr {

DRR_HD float fadd32(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    volatile float r = a + b;  // IEEE binary32 addition, no contraction or extended precision
    return r;
#endif
}

DRR_HD uint32_t float_bits(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, sizeof(u));
    return u;
#endif
}

DRR_HD float bits_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, sizeof(f));
    return f;
#endif
}

// Advance *alpha by float32 additions of `step` while it stays below `bound` (or at most `bound`
// when `inclusive`), performing at most `limit` additions. Returns the number of additions; *alpha
// ends exactly where the serial loop `while (k < limit && alpha < bound) alpha += step, ++k;` ends.
// Requires step > 0 and finite; alpha and bound may be any floats (NaN bound: no addition).
DRR_HD int advance_alpha(float *alpha, float step, float bound, int limit, bool inclusive) {
    float a = *alpha;
    int k = 0;
    const uint32_t sbits = float_bits(step);
    const int sexp = (int)((sbits >> 23) & 0xff);
    if (sexp == 0 || sexp == 0xff) {  // subnormal / inf / NaN step: serial additions only
        while (k < limit && (inclusive ? a <= bound : a < bound)) {
            a = fadd32(a, step);
            ++k;
        }
        *alpha = a;
        return k;
    }
    const int64_t smant = (int64_t)((sbits & 0x7fffff) | 0x800000);  // step = smant * 2^(sexp - 150)
    while (k < limit && (inclusive ? a <= bound : a < bound)) {
        const uint32_t abits = float_bits(a);
        const int aexp = (int)((abits >> 23) & 0xff);
        if ((abits >> 31) != 0 || aexp == 0 || aexp >= 0xfe) {
            // zero, negative, subnormal or near-overflow alpha: one ordinary addition
            a = fadd32(a, step);
            ++k;
            continue;
        }
        // alpha = am * u with u = 2^(aexp - 150), am in [2^23, 2^24)
        const int64_t am = (int64_t)((abits & 0x7fffff) | 0x800000);
        const int sh = aexp - sexp;  // step / u = smant * 2^-sh
        if (sh < -30) {  // step far larger than alpha: ordinary addition
            a = fadd32(a, step);
            ++k;
            continue;
        }
        int64_t delta;  // ulps added by one addition
        if (sh <= 0) {
            delta = smant << (-sh);  // step is a whole number of ulps
        } else if (sh > 62) {
            delta = 0;  // step below half an ulp
        } else {
            const int64_t m = smant >> sh;          // floor(step / u)
            const int64_t rem = smant - (m << sh);  // remainder, in units of 2^-sh
            const int64_t half = (int64_t)1 << (sh - 1);
            if (rem < half) {
                delta = m;
            } else if (rem > half) {
                delta = m + 1;
            } else {  // exact tie: round to even
                if (am & 1) {  // odd mantissa: one addition makes it even
                    a = fadd32(a, step);
                    ++k;
                    continue;
                }
                delta = m + (m & 1);
            }
        }
        if (delta == 0) {  // alpha never moves: the serial loop runs out its limit
            k = limit;
            break;
        }
        // the rounded sum stays in this binade while am + delta + 1 <= 2^24 - 1 before each addition
        const int64_t m = delta;
        // largest j such that every addition of the jump stays below the binade top:
        // am + (j-1) * delta + m + 1 <= 2^24 - 1
        const int64_t top = ((int64_t)1 << 24) - 2 - m - am;
        int64_t j = top >= 0 ? top / delta + 1 : 0;
        if (j <= 0) {
            a = fadd32(a, step);
            ++k;
            continue;
        }
        // first j with am + j * delta past the bound (bound is a float: exact in this grid as a real)
        const int64_t room = (int64_t)(limit - k);
        if (j > room) j = room;
        const uint32_t bbits = float_bits(bound);
        const int bexp = (int)((bbits >> 23) & 0xff);
        if ((bbits >> 31) == 0 && bexp != 0xff && bexp >= aexp && bexp - aexp < 24) {
            // bound = bm * 2^(bexp - 150) = (bm << (bexp - aexp)) * u, an integer in units of u
            const int64_t bm = (int64_t)((bbits & 0x7fffff) | (bexp ? 0x800000 : 0));
            const int64_t bu = bm << (bexp - aexp);
            // keep going while am + j*delta < bu (or <= bu when inclusive)
            const int64_t need = inclusive ? (bu - am) / delta + 1 : (bu - am + delta - 1) / delta;
            if (need < j) j = need;
        } else if ((bbits >> 31) != 0 || bexp < aexp) {
            j = 0;  // bound below alpha's binade: alpha already past it (loop condition handles it)
        }
        if (j <= 0) {
            a = fadd32(a, step);
            ++k;
            continue;
        }
        const int64_t nm = am + j * delta;  // stays in [2^23, 2^24)
        a = bits_float((uint32_t)(aexp << 23) | (uint32_t)(nm & 0x7fffff));
        k += (int)j;
    }
    *alpha = a;
    return k;
}

}  // namespace drr
