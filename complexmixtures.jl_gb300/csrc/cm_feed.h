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

// ---------------------------------------------------------------------------
// angle() for an FP32 search, without FP64 arithmetic on the common path.

// Leading zero bits of x != 0, and the high 64 bits of a 64 x 64-bit product.
CM_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}
CM_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * (unsigned __int128)b) >> 64);
#endif
}
CM_HD float f32_of_bits(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float f;
    __builtin_memcpy(&f, &b, 4);
    return f;
#endif
}
CM_HD float div32(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

// The FP32 value (round to nearest, ties to even) of the integer
// hi 2^64 + lo < 2^127, by integer operations: the leading bit moved to bit 63
// of `top`, 24 bits kept, then the round bit and the sticky bits below it.
CM_HD float u128_to_f32(uint64_t hi, uint64_t lo) {
    int e;
    uint64_t top;
    bool sticky;
    if (hi != 0) {
        const int lz = clz64(hi);
        top = lz ? (hi << lz) | (lo >> (64 - lz)) : hi;
        sticky = (lo << lz) != 0;
        e = 127 - lz;
    } else {
        if (lo == 0) return 0.0f;
        const int lz = clz64(lo);
        top = lo << lz;
        sticky = false;
        e = 63 - lz;
    }
    uint32_t m = (uint32_t)(top >> 40);
    const bool round = ((top >> 39) & 1) != 0;
    sticky = sticky || (top & ((uint64_t(1) << 39) - 1)) != 0;
    if (round && (sticky || (m & 1))) ++m;
    if (m >> 24) {
        m >>= 1;
        ++e;
    }
    return f32_of_bits(((uint32_t)(e + 127) << 23) | (m & 0x7fffffu));
}

// angle()'s test on the point (u, v) = (a, b) 2^-53 (a, b integers, |a|, |b|
// <= 2^53): accept when 0 < RN(RN(u^2) + RN(v^2)) < 1.  Each rounded square
// is within 2^52 units of 2^-106 of a^2 (resp. b^2), so with X = a^2 + b^2
// (exact, 128-bit) the rounded sum is below 1 when X < 2^106 - 2^55 and at
// least 1 when X >= 2^106 + 2^55; in between (probability about 1e-15) the
// FP64 test itself decides.  sq: a^2 and b^2 as (hi, lo) pairs.
CM_HD bool disk_accept(int64_t a, int64_t b, uint64_t *sq) {
    const uint64_t kOne = uint64_t(1) << 42;  // 2^106 = kOne 2^64
    const uint64_t ma = a < 0 ? (uint64_t)(-a) : (uint64_t)a;
    const uint64_t mb = b < 0 ? (uint64_t)(-b) : (uint64_t)b;
    sq[1] = ma * ma;
    sq[0] = mulhi64(ma, ma);
    sq[3] = mb * mb;
    sq[2] = mulhi64(mb, mb);
    const uint64_t xl = sq[1] + sq[3], xh = sq[0] + sq[2] + (xl < sq[1] ? 1 : 0);
    if (xh < kOne - 1 || (xh == kOne - 1 && xl < 0xFF80000000000000ULL)) return (xh | xl) != 0;
    if (xh > kOne || (xh == kOne && xl >= (uint64_t(1) << 55))) return false;
    // 2 U - 1 of angle() is exactly a 2^-53
    const double u = (double)a * 0x1.0p-53, v = (double)b * 0x1.0p-53;
    const double r2 = add(mul(u, u), mul(v, v));
    return r2 > 0.0 && r2 < 1.0;
}

// angle() for the FP32 search: the same draws and the same acceptance
// (disk_accept), and (cos, sin) in FP32 within 3.01 u32 (u32 = 2^-24) of
// angle()'s: cos = (a^2 - b^2) / X and sin = 2ab / X are the FP32 quotients of
// the integers (shifted right together below 2^64) rounded to FP32 (3 u32 of
// the exact quotients, plus 2^-62), and angle()'s FP64 values are within
// 6 2^-53 of the same quotients.
CM_HD void angle32(uint64_t &s, float &c, float &sn) {
    for (int t = 0; t < 64; ++t) {
        const int64_t a = (int64_t)(next(s) >> 11) * 2 - (int64_t(1) << 53);
        const int64_t b = (int64_t)(next(s) >> 11) * 2 - (int64_t(1) << 53);
        uint64_t sq[4];
        if (!disk_accept(a, b, sq)) continue;
        const uint64_t ah = sq[0], al = sq[1], bh = sq[2], bl = sq[3];
        const uint64_t xl = al + bl, xh = ah + bh + (xl < al ? 1 : 0);
        const bool nneg = ah < bh || (ah == bh && al < bl);
        uint64_t nl, nh;
        if (nneg) {
            nl = bl - al;
            nh = bh - ah - (bl < al ? 1 : 0);
        } else {
            nl = al - bl;
            nh = ah - bh - (al < bl ? 1 : 0);
        }
        const uint64_t ma = a < 0 ? (uint64_t)(-a) : (uint64_t)a;
        const uint64_t mb = b < 0 ? (uint64_t)(-b) : (uint64_t)b;
        const uint64_t pl = ma * mb, ph = mulhi64(ma, mb);
        const uint64_t mh = (ph << 1) | (pl >> 63), ml = pl << 1;
        // |N|, M <= X: one right shift by k brings all three below 2^64; the
        // bits shifted out move N / X and M / X by less than 2^-63
        const int k = xh ? 64 - clz64(xh) : 0;
        const uint64_t d64 = k ? (xl >> k) | (xh << (64 - k)) : xl;
        const uint64_t n64 = k ? (nl >> k) | (nh << (64 - k)) : nl;
        const uint64_t m64 = k ? (ml >> k) | (mh << (64 - k)) : ml;
        const float d = u128_to_f32(0, d64);
        const float n = u128_to_f32(0, n64);
        const float m = u128_to_f32(0, m64);
        c = div32(nneg ? -n : n, d);
        sn = div32((a < 0) != (b < 0) ? -m : m, d);
        return;
    }
    c = 1.0f;
    sn = 0.0f;
}

}  // namespace cmfeed
