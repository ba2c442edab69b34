// cm_feed.h -- seeded counter-based stream for the random-insertion reference.
//
// The reference draws its ideal-gas placements from Xoroshiro128Plus or
// StableRNG streams seeded per thread chunk (src/rigid_body.jl:8-19), so its
// random counts depend on the thread count.  The engine instead keys an
// independent stream on (seed, frame, solute molecule, repetition, slot), so
// counts do not depend on batching, launch shape or the number of GPUs, and
// the host-side checker can reproduce every placement bit for bit.
//
// Distributions follow the reference:
//   - bulk molecule: uniform over the ascending list of bulk molecules, or over
//     all solvent molecules when the list is empty (src/mddf.jl:74-80);
//   - new centre: uniform in the unit cell (src/rigid_body.jl:115-120 draws it
//     uniformly in a 10^4-scaled box that the cell list wraps back);
//   - Euler angles beta, gamma, theta: uniform in [0, 2pi)
//     (src/rigid_body.jl:122-125), produced here as (cos, sin) pairs by
//     rejection sampling on the unit disk, so no transcendental function is
//     evaluated and host and device agree exactly.
//
// Generator: SplitMix64 (Steele, Lea, Flood, "Fast splittable pseudorandom
// number generators", OOPSLA 2014): state += golden gamma, output = mix64(state).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define CM_HD __host__ __device__ __forceinline__
#else
#define CM_HD inline
#endif

namespace cmfeed {

constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ULL;
constexpr uint64_t kTagRef = 1ULL;   // per-frame draws of the reference solute molecules
constexpr uint64_t kTagSlot = 2ULL;  // per-(frame, solute, repetition, slot) placement

CM_HD uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

CM_HD uint64_t key(uint64_t seed, uint64_t tag, uint64_t a, uint64_t b, uint64_t c) {
    uint64_t k = mix64(seed + kGamma * (tag + 1ULL));
    k = mix64(k ^ a);
    k = mix64(k ^ b);
    return mix64(k ^ c);
}

CM_HD uint64_t next(uint64_t &s) {
    s += kGamma;
    return mix64(s);
}

// Uniform double in [0, 1) with 53 random bits.
CM_HD double uniform(uint64_t &s) { return (double)(next(s) >> 11) * 0x1.0p-53; }

// Uniform integer in [0, n): high 64 bits of the 128-bit product next * n.
CM_HD uint64_t below(uint64_t &s, uint64_t n) {
    uint64_t r = next(s);
#if defined(__CUDA_ARCH__)
    return __umul64hi(r, n);
#else
    return (uint64_t)(((unsigned __int128)r * (unsigned __int128)n) >> 64);
#endif
}

// Exact IEEE operations without contraction on either side.
CM_HD double mul(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
CM_HD double add(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
CM_HD double sub(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
CM_HD double div(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}

// (cos t, sin t) of an angle t uniform in [0, 2pi): with (u, v) uniform in the
// unit disk, t = 2 atan2(v, u) is uniform, cos t = (u^2 - v^2)/r^2 and
// sin t = 2uv/r^2.  At most 64 rejections (probability 0.2146^64 of running out).
CM_HD void angle(uint64_t &s, double &c, double &sn) {
    for (int t = 0; t < 64; ++t) {
        double u = sub(mul(2.0, uniform(s)), 1.0);
        double v = sub(mul(2.0, uniform(s)), 1.0);
        double uu = mul(u, u), vv = mul(v, v);
        double r2 = add(uu, vv);
        if (r2 > 0.0 && r2 < 1.0) {
            double uv = mul(u, v);
            c = div(sub(uu, vv), r2);
            sn = div(add(uv, uv), r2);
            return;
        }
    }
    c = 1.0;
    sn = 0.0;
}

// eulermat (src/rigid_body.jl:45-57) from the (cos, sin) of beta, gamma, theta;
// row-major output, products grouped left to right as in the reference.
CM_HD void eulermat(double c1, double s1, double c2, double s2, double c3, double s3, double *A) {
    A[0] = mul(c2, c3);
    A[1] = -mul(c2, s3);
    A[2] = s2;
    A[3] = add(mul(c1, s3), mul(mul(c3, s1), s2));
    A[4] = sub(mul(c1, c3), mul(mul(s1, s2), s3));
    A[5] = -mul(c2, s1);
    A[6] = sub(mul(s1, s3), mul(mul(c1, c3), s2));
    A[7] = add(mul(mul(c1, s2), s3), mul(c3, s1));
    A[8] = mul(c1, c2);
}

}  // namespace cmfeed
