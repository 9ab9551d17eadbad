// flop_count.cpp — operation count of the membrane element (A3, evalElementRe UL:710-928
// for the cell, UL:989-1176 for the substrate) by compiling the oracle's own C source
// with a counting scalar in place of double.  Test infrastructure: it pins the
// element-assembly FLOP figure used as the work unit (tests/test_oracle_flops.py).
//
// Counted as one flop each: add, subtract, multiply, divide, sqrt, exp, acos.  Not
// counted: comparisons, negation, fabs, and arithmetic on literals (folded by the compiler).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

struct Counted {
    double v;
    Counted() = default;
    Counted(double x) : v(x) {}
    explicit operator int() const { return (int)v; }
    explicit operator long() const { return (long)v; }
    explicit operator unsigned() const { return (unsigned)v; }
    explicit operator float() const { return (float)v; }
};
static long long n_add, n_mul, n_div, n_sqrt, n_exp, n_acos, n_cmp, n_neg, n_abs;
inline Counted operator+(Counted a, Counted b) { ++n_add; return a.v + b.v; }
inline Counted operator-(Counted a, Counted b) { ++n_add; return a.v - b.v; }
inline Counted operator*(Counted a, Counted b) { ++n_mul; return a.v * b.v; }
inline Counted operator/(Counted a, Counted b) { ++n_div; return a.v / b.v; }
inline Counted operator-(Counted a) { ++n_neg; return -a.v; }
inline Counted& operator+=(Counted& a, Counted b) { a = a + b; return a; }
inline Counted& operator-=(Counted& a, Counted b) { a = a - b; return a; }
inline Counted& operator*=(Counted& a, Counted b) { a = a * b; return a; }
inline Counted& operator/=(Counted& a, Counted b) { a = a / b; return a; }
inline bool operator<(Counted a, Counted b) { ++n_cmp; return a.v < b.v; }
inline bool operator>(Counted a, Counted b) { ++n_cmp; return a.v > b.v; }
inline bool operator<=(Counted a, Counted b) { ++n_cmp; return a.v <= b.v; }
inline bool operator>=(Counted a, Counted b) { ++n_cmp; return a.v >= b.v; }
inline bool operator==(Counted a, Counted b) { ++n_cmp; return a.v == b.v; }
inline bool operator!=(Counted a, Counted b) { ++n_cmp; return a.v != b.v; }
inline Counted sqrt(Counted a) { ++n_sqrt; return std::sqrt(a.v); }
inline Counted exp(Counted a) { ++n_exp; return std::exp(a.v); }
inline Counted acos(Counted a) { ++n_acos; return std::acos(a.v); }
inline Counted fabs(Counted a) { ++n_abs; return std::fabs(a.v); }

#define double Counted
#include "wcfe_oracle.c"
#undef double

static void reset() { n_add = n_mul = n_div = n_sqrt = n_exp = n_acos = n_cmp = n_neg = n_abs = 0; }
static void report(const char* what, long long per) {
    const long long flops = n_add + n_mul + n_div + n_sqrt + n_exp + n_acos;
    std::printf("%s add=%lld mul=%lld div=%lld sqrt=%lld exp=%lld acos=%lld flops=%lld cmp=%lld\n", what,
                n_add / per, n_mul / per, n_div / per, n_sqrt / per, n_exp / per, n_acos / per, flops / per,
                n_cmp / per);
}

int main() {
    wcfe_params p;
    wo_params_default(&p, WCFE_VARIANT_K1);
    // one element of a typical deformed state: a 1-um triangle, small strain history
    const Counted X1[3] = {0.0, 0.0, 0.0}, X2[3] = {1.0, 0.05, 0.0}, X3[3] = {0.45, 0.9, 0.0};
    const Counted x1[3] = {0.001, -0.002, 0.0}, x2[3] = {1.003, 0.049, 0.0}, x3[3] = {0.452, 0.897, 0.0};
    const Counted ea1[6] = {0.01, -0.005, 0.0, 0.002, 0.0, 0.0}, ea2[6] = {0.008, -0.004, 0.0, 0.001, 0.0, 0.0},
                  ea3[6] = {0.012, -0.006, 0.0, 0.003, 0.0, 0.0};
    const Counted cA3[3] = {100.0, 100.0, 100.0}, cC3[3] = {0.2, 0.3, 0.1};
    const Counted cen[3] = {0.2, 0.1, 0.0};
    wo_elem_out o;
    for (int mat = 1; mat <= 2; ++mat) {
        const Counted t_act = mat == 1 ? t_act_of(&p, Counted(0.3)) : Counted(0.0);
        reset();
        wo_element(X1, X2, X3, x1, x2, x3, ea1, ea2, ea3, cA3, cC3, Counted(5e-5), mat, p.mu, &p, t_act, cen, &o);
        report(mat == 1 ? "element_cell" : "element_substrate", 1);
    }
    return 0;
}
