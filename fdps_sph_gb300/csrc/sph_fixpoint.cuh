// Fixed-point terms for the order-free density sums.
//
// The density kernel rounds every term m_j W_ij (FP32, >= 0) to a multiple of 2^-40 and sums the
// multiples as integers, so the sum does not depend on the order of the terms.  A 64-bit
// float-to-integer conversion per term (__float2ll_rn) issues on the FP64 pipe, a small fraction
// of the FP32 rate on GB300.  For terms in [0, 16] the same integer comes from four FP32 additions
// and two 32-bit integer additions:
//
//   a  = t + 96            rounds t to a multiple of 2^-17 (96 = 1.5 * 2^6, whose binade
//                          [64, 128) has the spacing 2^-17); bits(a) - bits(96) = a_int, the
//                          number of 2^-17 steps, for t in [-32, 32)
//   lo = t - (a - 96)      exact (Sterbenz), |lo| <= 2^-18
//   b  = lo + 1.5 * 2^-17  rounds lo to a multiple of 2^-40 (the spacing of [2^-17, 2^-16]);
//                          bits(b) - bits(1.5 * 2^-17) = round(lo * 2^40), also at b = 2^-16
//
// and round(t * 2^40) = a_int * 2^23 + round(lo * 2^40), ties to even included (both offsets
// are even multiples of the spacing).  The two counts accumulate in 32-bit wrapping sums, read
// as signed after at most 256 terms (|a_int| <= 2^21, |round(lo * 2^40)| <= 2^22).  The
// additions are the _rn intrinsics, so the compiler cannot fuse t's product into the first one.
// Plain C++ as well, so the host can check it against the C library.
#pragma once

#if defined(__CUDACC__)
#define SPH_FIX_HD __host__ __device__ __forceinline__
#else
#include <cstring>
#define SPH_FIX_HD inline
#endif

constexpr float SPH_FIX_C1 = 96.0f;                  // 1.5 * 2^6
constexpr float SPH_FIX_C2 = 1.1444091796875e-05f;   // 1.5 * 2^-17
constexpr unsigned SPH_FIX_B1 = 0x42C00000u;         // bits of SPH_FIX_C1
constexpr unsigned SPH_FIX_B2 = 0x37400000u;         // bits of SPH_FIX_C2
constexpr float SPH_FIX_TMAX = 16.0f;                // largest term the split takes
constexpr int SPH_FIX_TERMS = 256;                   // terms per pair of 32-bit sums

SPH_FIX_HD unsigned sph_fix_bits(float v) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(v);
#else
    unsigned b;
    std::memcpy(&b, &v, sizeof b);
    return b;
#endif
}

SPH_FIX_HD float sph_fix_add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;   // host: IEEE single addition (SSE / NEON), no excess precision
#endif
}

SPH_FIX_HD float sph_fix_sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

// adds round-half-even(t * 2^40) to the sums (H, L), whose value is H * 2^23 + L; t in [0, 16]
SPH_FIX_HD void sph_fix40_add(float t, unsigned &H, unsigned &L) {
    const float a = sph_fix_add(t, SPH_FIX_C1);
    const float lo = sph_fix_sub(t, sph_fix_sub(a, SPH_FIX_C1));
    const float b = sph_fix_add(lo, SPH_FIX_C2);
    H += sph_fix_bits(a) - SPH_FIX_B1;
    L += sph_fix_bits(b) - SPH_FIX_B2;
}

// the same on a grid 2^f times coarser, for t in [0, 16 * 2^f]: b1 / b2 = SPH_FIX_B1 / B2 + f * 2^23
// (the constants' bits with the exponent moved by f), c1 / c2 the floats with those bits.  Every
// quantity is 2^f times the one of sph_fix40_add(t * 2^-f), so the counts are the same, for
// |f| <= 60 (no constant leaves the normal range; a t that is subnormal rounds to 0 either way)
SPH_FIX_HD void sph_fix40_add(float t, unsigned &H, unsigned &L, float c1, float c2, unsigned b1, unsigned b2) {
    const float a = sph_fix_add(t, c1);
    const float lo = sph_fix_sub(t, sph_fix_sub(a, c1));
    const float b = sph_fix_add(lo, c2);
    H += sph_fix_bits(a) - b1;
    L += sph_fix_bits(b) - b2;
}

// The density kernel adds the raw bit patterns of a and b (two terms at a time, in paired FP32
// arithmetic) and takes nt * b1 and nt * b2 off when it reads the sums (nt terms, zero terms of
// non-members included, which add exactly b1 and b2): the same sums, mod 2^32, as above.

// the value of the sums after at most SPH_FIX_TERMS additions
SPH_FIX_HD long long sph_fix40_value(unsigned H, unsigned L) {
    return (long long)(int)H * 8388608LL + (long long)(int)L;
}
