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

WCFE_HD uint32_t dhi(double x) {
#if defined(__CUDA_ARCH__)
    return (uint32_t)__double2hiint(x);
#else
    return (uint32_t)(dbits(x) >> 32);
#endif
}
WCFE_HD uint32_t dlo(double x) {
#if defined(__CUDA_ARCH__)
    return (uint32_t)__double2loint(x);
#else
    return (uint32_t)dbits(x);
#endif
}
WCFE_HD double dmake(uint32_t hi, uint32_t lo) {
#if defined(__CUDA_ARCH__)
    return __hiloint2double((int)hi, (int)lo);
#else
    return bitsd(((uint64_t)hi << 32) | lo);
#endif
}

// binary64 -> binary32, round to nearest even.  32-bit integer operations only.
WCFE_HD float f64_to_f32_rn(double x) {
    const uint32_t hi = dhi(x), lo = dlo(x);
    const uint32_t s = hi & 0x80000000u;
    const uint32_t ah = hi ^ s;
    // normal binary32 results: biased binary64 exponent in [897, 1150]
    if (ah - (897u << 20) < (254u << 20)) {
        const uint32_t rh = ah - (896u << 20);        // rebias the exponent to binary32's
        // round the 52-bit fraction to 23 bits (ties to even): add 2^28 - 1 + bit 29, carry into the high word
        const uint32_t t = lo + 0x0FFFFFFFu + ((lo >> 29) & 1u);
        const uint32_t rh2 = rh + (t < lo ? 1u : 0u);
        return bitsf(((rh2 << 3) | (t >> 29)) | s);
    }
    // |x| < 2^-150 (exponent <= 872) rounds to a signed zero
    if (ah < (873u << 20)) return bitsf(s);
    return f64_to_f32_slow(x);                     // subnormal results, overflow, inf, NaN
}

// binary32 -> binary64, exact.  32-bit integer operations only.
WCFE_HD double f32_to_f64(float f) {
    const uint32_t b = fbits(f);
    const uint32_t s = b & 0x80000000u;
    const uint32_t a = b ^ s;
    if (a - 0x00800000u < 0x7f000000u) return dmake(((a >> 3) + (896u << 20)) | s, a << 29);
    if (a == 0) return dmake(s, 0u);               // signed zero
    return f32_to_f64_slow(f);                     // subnormal, inf, NaN
}

}  // namespace wcfe
