"""The integer-pipe FP64<->FP32 conversions (wholecellfe_gb300/csrc/wcfe_cvt.h)
give the same bits as the compiler's conversions, on the host, over random
values across the whole exponent range and the edge cases."""
import os
import subprocess
import tempfile

from conftest import ROOT

DRIVER = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include "wcfe_cvt.h"
using namespace wcfe;
int main() {
    std::mt19937_64 g(12345);
    long bad = 0, n = 0;
    auto chk_d = [&](double x) {
        float a = f64_to_f32_rn(x), b = (float)x;
        if (memcmp(&a, &b, 4) && !(std::isnan(a) && std::isnan(b))) { if (bad < 5) printf("d %a %a %a\n", x, a, b); ++bad; }
        ++n;
    };
    auto chk_f = [&](float f) {
        double a = f32_to_f64(f), b = (double)f;
        if (memcmp(&a, &b, 8) && !(std::isnan(a) && std::isnan(b))) { if (bad < 5) printf("f %a\n", f); ++bad; }
        ++n;
    };
    for (int i = 0; i < 4000000; ++i) {
        uint64_t r = g();
        double x; memcpy(&x, &r, 8);
        chk_d(x);
        uint32_t r32 = (uint32_t)(r >> 7);
        float f; memcpy(&f, &r32, 4);
        chk_f(f);
    }
    // values near binary32 range limits, ties, and typical magnitudes
    const double edges[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38, 1.1754943508222875e-38,
                            1.1754942106924411e-38, 1.401298464324817e-45, 1e-46, 1e300, -1e300, INFINITY, -INFINITY, NAN,
                            1.0000000596046448, 1.0000001788139343, 0.1, 10.0, 1e-7, 2.5e-5};
    for (double e : edges) { chk_d(e); chk_d(std::nextafter(e, 1e308)); chk_d(std::nextafter(e, -1e308)); chk_f((float)e); }
    std::uniform_real_distribution<double> u(-20.0, 20.0);
    for (int i = 0; i < 2000000; ++i) { double x = u(g) * std::pow(10.0, (int)(g() % 40) - 30); chk_d(x); chk_f((float)x); }
    printf("%ld %ld\n", bad, n);
    return bad != 0;
}
"""


def test_integer_conversions_match_hardware():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        exe = os.path.join(d, "t")
        open(src, "w").write(DRIVER)
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "wholecellfe_gb300", "csrc"), src,
                               "-o", exe])
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
        bad, n = map(int, r.stdout.split()[-2:])
        assert bad == 0 and n > 10_000_000
