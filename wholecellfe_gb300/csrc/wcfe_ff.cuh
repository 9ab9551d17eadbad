// wcfe_ff.cuh — float-float ("double-single") arithmetic for the mixed form's state.
//
// A value is an unevaluated sum hi + lo of two binary32 numbers with
// hi = RN(hi + lo), about 48 significant bits.  The mixed form keeps its state
// (positions, velocities, strain, bond vectors, bond densities) in this format
// so that the per-step accumulations run on the FP32 pipe: on GB300 an FP64
// add or FMA retires at about 1/64 of the FP32 rate, and a float-float add
// costs about ten FP32 operations.
//
// The error-free transformations are Knuth's TwoSum, Dekker's FastTwoSum and
// the FMA-based TwoProduct (Ogita, Rump and Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26(6), 2005).  The additions use explicit
// round-to-nearest intrinsics so that the compiler neither contracts nor
// reorders them.
#pragma once
#include <math.h>
#include <stdint.h>

#include "wcfe_cvt.h"

namespace wcfe {

struct ff {
    float hi, lo;
};

#if defined(__CUDA_ARCH__)
#define FF_ADD(a, b) __fadd_rn((a), (b))
#define FF_SUB(a, b) __fsub_rn((a), (b))
#define FF_MUL(a, b) __fmul_rn((a), (b))
#define FF_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#else
#define FF_ADD(a, b) ((float)((a) + (b)))
#define FF_SUB(a, b) ((float)((a) - (b)))
#define FF_MUL(a, b) ((float)((a) * (b)))
#define FF_FMA(a, b, c) (fmaf((a), (b), (c)))
#endif

// s + e = a + b exactly (TwoSum)
WCFE_HD ff two_sum(float a, float b) {
    const float s = FF_ADD(a, b);
    const float bb = FF_SUB(s, a);
    const float e = FF_ADD(FF_SUB(a, FF_SUB(s, bb)), FF_SUB(b, bb));
    return {s, e};
}
// s + e = a + b exactly when |a| >= |b| or a == 0 (FastTwoSum)
WCFE_HD ff fast_two_sum(float a, float b) {
    const float s = FF_ADD(a, b);
    return {s, FF_SUB(b, FF_SUB(s, a))};
}
// a + b, both float-float
WCFE_HD ff ff_add(ff a, ff b) {
    const ff s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, FF_ADD(s.lo, FF_ADD(a.lo, b.lo)));
}
// a - b, both float-float
WCFE_HD ff ff_sub(ff a, ff b) { return ff_add(a, {-b.hi, -b.lo}); }
// a + b, b a float
WCFE_HD ff ff_add_f(ff a, float b) {
    const ff s = two_sum(a.hi, b);
    return fast_two_sum(s.hi, FF_ADD(s.lo, a.lo));
}
// a * b, b a float (TwoProduct of the high part)
WCFE_HD ff ff_mul_f(ff a, float b) {
    const float p = FF_MUL(a.hi, b);
    const float e = FF_FMA(a.lo, b, FF_FMA(a.hi, b, -p));
    return fast_two_sum(p, e);
}
// a * b, both float-float (the lo * lo term is below the format's precision)
WCFE_HD ff ff_mul(ff a, ff b) {
    const float p = FF_MUL(a.hi, b.hi);
    const float e = FF_FMA(a.hi, b.lo, FF_FMA(a.lo, b.hi, FF_FMA(a.hi, b.hi, -p)));
    return fast_two_sum(p, e);
}
// a + b * c with b float-float and c a float
WCFE_HD ff ff_fma_f(ff a, ff b, float c) { return ff_add(a, ff_mul_f(b, c)); }
// a + b * c, both products' factors float-float
WCFE_HD ff ff_fma(ff a, ff b, ff c) { return ff_add(a, ff_mul(b, c)); }
// square root: s = sqrt(hi) corrected by one Newton step on the exact residual
WCFE_HD ff ff_sqrt(ff a) {
    if (!(a.hi > 0.0f)) return {0.0f, 0.0f};
    const float s = sqrtf(a.hi);
    const float r = FF_ADD(FF_FMA(-s, s, a.hi), a.lo);   // a - s^2
    return fast_two_sum(s, r / (2.0f * s));
}
WCFE_HD ff ff_abs(ff a) { return a.hi < 0.0f ? ff{-a.hi, -a.lo} : a; }
WCFE_HD bool ff_lt(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
// the float nearest to the value (hi, for a normalised pair)
WCFE_HD float ff_f(ff a) { return a.hi; }

// conversions to and from binary64: hi = RN(x), lo = RN(x - hi)
WCFE_HD ff ff_from_d(double x) {
    const float h = f64_to_f32_rn(x);
    return {h, f64_to_f32_rn(x - f32_to_f64(h))};
}
WCFE_HD double ff_to_d(ff a) { return f32_to_f64(a.hi) + f32_to_f64(a.lo); }

// per-vertex vectors in HBM: 3 components (+ a pad) as hi and lo float4, 32 bytes
struct alignas(16) ff4 {
    float hx, hy, hz, hw;
    float lx, ly, lz, lw;
};
WCFE_HD ff ffx(const ff4& v) { return {v.hx, v.lx}; }
WCFE_HD ff ffy(const ff4& v) { return {v.hy, v.ly}; }
WCFE_HD ff ffz(const ff4& v) { return {v.hz, v.lz}; }
WCFE_HD ff4 make_ff4(ff x, ff y, ff z) { return {x.hi, y.hi, z.hi, 0.0f, x.lo, y.lo, z.lo, 0.0f}; }

// per-vertex strain: Voigt (xx, yy, zz, xy) hi and lo, then (xz, yz) hi and lo, 48 bytes
struct alignas(16) ffea {
    float hxx, hyy, hzz, hxy;
    float lxx, lyy, lzz, lxy;
    float hxz, hyz, lxz, lyz;
};

}  // namespace wcfe
