// Fixed-point recombination of the split-precision GEMM accumulators with integer
// instructions only.  A GB300 SM retires about two FP64 operations per clock but over a
// hundred integer ones, so the epilogue of the split GEMM converts its FP32 accumulators to
// a common 2^-28 fixed point, adds them as 64-bit integers and assembles the IEEE-754 double
// of the sum (with its power-of-two scale) from the integer bit by bit.  Host and device share
// these functions, so the arithmetic is tested on the CPU.
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define DCG_HD __host__ __device__ __forceinline__
#else
#define DCG_HD inline
#endif

namespace dcg {

DCG_HD int clz64(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)u);
#else
    return __builtin_clzll(u);
#endif
}

DCG_HD double bits_to_double(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double d;
    memcpy(&d, &b, sizeof d);
    return d;
#endif
}

// f * 2^28 rounded to the nearest integer (halves away from zero), from the FP32 bit pattern
// of f.  Exact whenever f is a multiple of 2^-28; |f| must stay below 2^34 (|result| < 2^62).
// Zero and subnormal inputs give 0.
DCG_HD int64_t fx28_from_float_bits(uint32_t bits) {
    const int ex = (int)((bits >> 23) & 0xFFu);
    if (ex == 0) return 0;
    const int64_t m = (int64_t)((bits & 0x7FFFFFu) | 0x800000u);   // f = m 2^(ex - 150)
    int sh = ex - 122;                                               // f 2^28 = m 2^sh
    if (sh > 38) sh = 38;                                            // out-of-range input: saturate
    int64_t v;
    if (sh >= 0)
        v = m << sh;
    else if (sh < -24)
        v = 0;
    else
        v = (m + ((int64_t)1 << (-sh - 1))) >> (-sh);
    return (bits >> 31) ? -v : v;
}

// X * 2^scale as a double, rounded to nearest (ties to even), from integer operations; the
// rare results outside the normal exponent range take the library's ldexp.
DCG_HD double fx_to_double(int64_t X, int scale) {
    if (X == 0) return 0.0;
    const uint64_t sgn = X < 0 ? (1ull << 63) : 0ull;
    const uint64_t u = X < 0 ? (uint64_t)0 - (uint64_t)X : (uint64_t)X;
    int p = 63 - clz64(u);   // position of the leading bit
    uint64_t mant;
    if (p <= 52) {
        mant = u << (52 - p);
    } else {
        const int s = p - 52;
        mant = u >> s;
        const uint64_t rem = u & ((1ull << s) - 1ull), half = 1ull << (s - 1);
        if (rem > half || (rem == half && (mant & 1ull))) {
            mant++;
            if (mant >> 53) {
                mant >>= 1;
                p++;
            }
        }
    }
    const int be = p + scale + 1023;
    if (be <= 0 || be >= 2047) return ldexp((double)X, scale);
    return bits_to_double(sgn | ((uint64_t)be << 52) | (mant & 0xFFFFFFFFFFFFFull));
}

}  // namespace dcg
