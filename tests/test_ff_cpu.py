"""Float-float arithmetic of the mixed form (wholecellfe_gb300/csrc/wcfe_ff.cuh) on
the host: the error-free transformations are exact, and the float-float add,
multiply and the binary64 conversions carry about 48 bits."""
import os
import subprocess
import tempfile

from conftest import ROOT

DRIVER = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include "wcfe_ff.cuh"
using namespace wcfe;
typedef long double LD;
static LD val(ff a) { return (LD)a.hi + (LD)a.lo; }
static bool normal_pair(ff a) { return (float)((double)a.hi + (double)a.lo) == a.hi; }
int main() {
    std::mt19937_64 g(7);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    long bad = 0, n = 0;
    double worst_add = 0, worst_mul = 0, worst_mulf = 0, worst_rt = 0, worst_sub = 0;
    for (int i = 0; i < 2000000; ++i) {
        const double x = u(g) * std::ldexp(1.0, (int)(g() % 40) - 20);
        const double y = u(g) * std::ldexp(1.0, (int)(g() % 40) - 20);
        const float fx = (float)x, fy = (float)y;
        // TwoSum and FastTwoSum are exact
        ff s = two_sum(fx, fy);
        if ((double)s.hi + (double)s.lo != (double)fx + (double)fy) ++bad;
        ff t = std::fabs(fx) >= std::fabs(fy) ? fast_two_sum(fx, fy) : fast_two_sum(fy, fx);
        if ((double)t.hi + (double)t.lo != (double)fx + (double)fy) ++bad;
        // conversions: hi = RN(x), |x - (hi + lo)| <= 2^-48 |x|
        ff a = ff_from_d(x), b = ff_from_d(y);
        if (a.hi != fx || !normal_pair(a)) ++bad;
        worst_rt = std::fmax(worst_rt, (double)(std::fabs((LD)x - val(a)) / std::fabs((LD)x)));
        if (std::fabs(ff_to_d(a) - (double)val(a)) > 1e-30 + 1e-16 * std::fabs(x)) ++bad;
        // add of same-sign values and sub, relative to the exact result of the pairs
        ff c = ff_add(a, b);
        LD ex = val(a) + val(b);
        if (!normal_pair(c)) ++bad;
        if ((x > 0) == (y > 0)) worst_add = std::fmax(worst_add, (double)(std::fabs(val(c) - ex) / std::fabs(ex)));
        else worst_sub = std::fmax(worst_sub, (double)(std::fabs(val(c) - ex) / (std::fabs(val(a)) + std::fabs(val(b)))));
        ff m = ff_mul(a, b);
        LD em = val(a) * val(b);
        worst_mul = std::fmax(worst_mul, (double)(std::fabs(val(m) - em) / std::fabs(em)));
        ff mf = ff_mul_f(a, fy);
        LD emf = val(a) * (LD)fy;
        worst_mulf = std::fmax(worst_mulf, (double)(std::fabs(val(mf) - emf) / std::fabs(emf)));
        // adding a small increment to a large value: the step update pattern
        ff acc = ff_add_f(a, fy * 1e-6f);
        LD ea = val(a) + (LD)(fy * 1e-6f);
        worst_add = std::fmax(worst_add, (double)(std::fabs(val(acc) - ea) / std::fabs(ea)));
        n += 1;
    }
    printf("%ld %ld %.3e %.3e %.3e %.3e %.3e\n", bad, n, worst_rt, worst_add, worst_sub, worst_mul, worst_mulf);
    return 0;
}
"""


def test_float_float_arithmetic():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        exe = os.path.join(d, "t")
        open(src, "w").write(DRIVER)
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                               os.path.join(ROOT, "wholecellfe_gb300", "csrc"), src, "-o", exe])
        r = subprocess.run([exe], capture_output=True, text=True, check=True)
        bad, n, rt, add, sub, mul, mulf = r.stdout.split()
        assert int(bad) == 0 and int(n) == 2000000
        assert float(rt) <= 2.0 ** -47
        assert float(add) <= 2.0 ** -44
        assert float(sub) <= 2.0 ** -44
        assert float(mul) <= 2.0 ** -44
        assert float(mulf) <= 2.0 ** -45
