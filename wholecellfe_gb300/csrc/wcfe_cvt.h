// wcfe_cvt.h — FP64 <-> FP32 conversions on the integer pipe.
//
// On GB300 the FP64 pipe, which also executes the hardware F64<->F32
// conversions, retires about 2 lanes per clock per SM.  The mixed form
// crosses the FP32/FP64 boundary a few dozen times per vertex and step, so
// these conversions are written here from the IEEE-754 binary64/binary32
// layouts as integer operations:
//  - f64_to_f32_rn: round to nearest, ties to even, for results in the normal
//    float range and for values that round to zero; subnormal results and
//    overflow/NaN take the hardware conversion (a rare, identical-result call);
//  - f32_to_f64: exact, for normal floats and zeros; subnormals, inf and NaN
//    take the hardware conversion.
// Both give the same bits as the hardware conversion (checked by the tests
// on the host against the compiler's conversions).
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define WCFE_HD __host__ __device__ __forceinline__
#else
#define WCFE_HD inline
#endif

namespace wcfe {

WCFE_HD uint64_t dbits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}
WCFE_HD double bitsd(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}
WCFE_HD uint32_t fbits(float x) {
#if defined(__CUDA_ARCH__)
    return (uint32_t)__float_as_uint(x);
#else
    uint32_t b;
    memcpy(&b, &x, 4);
    return b;
#endif
}
WCFE_HD float bitsf(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float x;
    memcpy(&x, &b, 4);
    return x;
#endif
}

// The rare cases take the hardware conversion in a function that is not
// inlined, so that the compiler cannot turn the branch into a select that
// executes the hardware conversion for every value.
#if defined(__CUDACC__)
static __host__ __device__ __noinline__ float f64_to_f32_slow(double x) { return (float)x; }
static __host__ __device__ __noinline__ double f32_to_f64_slow(float f) { return (double)f; }
#else
inline float f64_to_f32_slow(double x) { return (float)x; }
inline double f32_to_f64_slow(float f) { return (double)f; }
#endif

// binary64 -> binary32, round to nearest even
WCFE_HD float f64_to_f32_rn(double x) {
    const uint64_t b = dbits(x);
    const uint64_t s = b & 0x8000000000000000ull;
    const uint64_t a = b ^ s;
    // normal binary32 results: biased binary64 exponent in [897, 1150]
    if (a - (897ull << 52) < (254ull << 52)) {
        uint64_t r = a - (896ull << 52);            // rebias the exponent to binary32's
        r += 0x0FFFFFFFull + ((r >> 29) & 1ull);    // round the 52-bit fraction to 23 bits, ties to even
        return bitsf((uint32_t)(r >> 29) | (uint32_t)(s >> 32));
    }
    // |x| < 2^-150 (exponent <= 872) rounds to a signed zero
    if (a < (873ull << 52)) return bitsf((uint32_t)(s >> 32));
    return f64_to_f32_slow(x);                     // subnormal results, overflow, inf, NaN
}

// binary32 -> binary64, exact
WCFE_HD double f32_to_f64(float f) {
    const uint32_t b = fbits(f);
    const uint32_t s = b & 0x80000000u;
    const uint32_t a = b ^ s;
    if (a - 0x00800000u < 0x7f000000u) return bitsd((((uint64_t)a << 29) + (896ull << 52)) | ((uint64_t)s << 32));
    if (a == 0) return bitsd((uint64_t)s << 32);  // signed zero
    return f32_to_f64_slow(f);                     // subnormal, inf, NaN
}

}  // namespace wcfe
