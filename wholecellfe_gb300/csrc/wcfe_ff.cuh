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
// a / b, both float-float: the quotient of the high parts corrected by one step on the
// remainder a - q b (Dekker's long division)
WCFE_HD ff ff_div(ff a, ff b) {
    const float q1 = a.hi / b.hi;
    const ff r = ff_sub(a, ff_mul_f(b, q1));
    return fast_two_sum(q1, r.hi / b.hi);
}
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

// ---- positions: triple-float --------------------------------------------------
// A position coordinate is h + (m + l): a float h and a normalised float-float
// remainder (m, l) with |m + l| <= ulp(h) / 2 or so, about 72 significant bits.  Any
// binary64 value splits into it exactly, so a state set from doubles is held
// exactly, and adding a step displacement d rounds only inside the remainder
// (an absolute error near 2^-47 |m + d|, about 1e-20 um at cell scale, against
// 2^-53 |x| = 1e-15 um for a binary64 position update).  The planar mixed form
// keeps z = 0, so the third float of x and y lives in the w slots of the ff4
// layout: hi float4 (x.h, y.h, 0, x.l), lo float4 (x.m, y.m, 0, y.l); ffx / ffy
// then read the float-float (h, m) part unchanged.
struct tf {
    float h, m, l;
};
// x + d exactly but for the rounding of the remainder sum (m, l) + d
WCFE_HD tf tf_add_ff(tf x, ff d) {
    const ff r = ff_add({x.m, x.l}, d);
    const ff s = two_sum(x.h, r.hi);
    const ff n = two_sum(s.lo, r.lo);
    return {s.hi, n.hi, n.lo};
}
// a - b as float-float (the displacement between two positions)
WCFE_HD ff tf_sub(tf a, tf b) {
    const ff s = two_sum(a.h, -b.h);
    return ff_add(s, ff_sub({a.m, a.l}, {b.m, b.l}));
}
// the float-float part (h, m); the omitted l is below 2^-48 |x|
WCFE_HD ff tf_ff(tf a) { return {a.h, a.m}; }
// exact split of a binary64 value: h = RN(x), m = RN(x - h), l = x - h - m
WCFE_HD tf tf_from_d(double x) {
    const float h = f64_to_f32_rn(x);
    const double r = x - f32_to_f64(h);
    const float m = f64_to_f32_rn(r);
    return {h, m, f64_to_f32_rn(r - f32_to_f64(m))};
}
// RN(h + m + l): h + m is exact in binary64, the one rounding is the last addition
WCFE_HD double tf_to_d(tf a) { return (f32_to_f64(a.h) + f32_to_f64(a.m)) + f32_to_f64(a.l); }
WCFE_HD tf tfx(const ff4& v) { return {v.hx, v.lx, v.hw}; }
WCFE_HD tf tfy(const ff4& v) { return {v.hy, v.ly, v.lw}; }
// the position layout above (z = 0 in the planar mixed form, kept as its float-float)
WCFE_HD ff4 make_pos4(tf x, tf y, ff z) { return {x.h, y.h, z.hi, x.l, x.m, y.m, z.lo, y.l}; }

// per-vertex strain: Voigt (xx, yy, zz, xy) hi and lo, then (xz, yz) hi and lo, 48 bytes
struct alignas(16) ffea {
    float hxx, hyy, hzz, hxy;
    float lxx, lyy, lzz, lxy;
    float hxz, hyz, lxz, lyz;
};

}  // namespace wcfe
