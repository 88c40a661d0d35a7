// ns_fastmath.cuh -- exp, log and 1/x for the transport law mu(T), k(T)
// (coefficients.f90:27-59), with fewer FP64-pipe instructions than the
// general library functions (the FP64 pipe bounds the stage kernels).
//
// Written from the table-driven method of P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989, and "... of the logarithm function",
// ACM TOMS 16(4), 1990, with Taylor polynomials on the reduced intervals:
//
//   exp(a) = 2^(q/256) * e^r,  q = nearest integer to 256*a/ln2,
//            |r| <= ln2/512 = 0.00135; 2^(j/256) (j = q mod 256) from a
//            table, e^r - 1 by its Taylor polynomial of degree 4 (remainder
//            r^5/120 < 3.8e-17 relative).
//   x = 2^e * m, m in [1,2); j = the top 8 fraction bits of m;
//   c_j = 1/(1 + (j + 1/2)/256) rounded to 12 significant bits, so that
//   r = m*c_j - 1 (one FMA) has |r| < 2^-8.9;
//   log(x) = e*ln2 - log(c_j) + log1p(r), log1p by its Taylor polynomial of
//            degree 6 (remainder r^7/7 < 3e-20);
//   1/x    = 2^-e * c_j / (1 + r), 1/(1+r) by its geometric series to
//            degree 6 (remainder r^7 < 2e-19 relative).
//
// The tables are filled on the host (std::exp2, std::log) by
// ns::ensure_math_tables before the first launch on a device; they are a
// __device__ variable of ns_kernels.cu, the one translation unit that
// includes this header.  Arguments outside the ranges the reduction handles
// (non-finite, x <= 0 or subnormal or |log2 x| >= 1000, |a| >= 512) take the
// library functions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ns {
namespace fm {

struct Tables {
    double exp2j[256];   // 2^(j/256)
    double logc[256];    // c_j
    double lognc[256];   // -log(c_j)
};

// filled by ensure_math_tables (ns_kernels.cu, the only includer)
static __device__ Tables g_tables;

__device__ __forceinline__ double exp_t(double a)
{
    // |a| < 512 from the exponent field (no FP64 compare)
    if ((__double2hiint(a) & 0x7ff00000) >= (1032 << 20)) return exp(a);
    const double inv = 0x1.71547652b82fep+8;             // 256 / ln 2
    const double shifter = 0x1.8p52;                     // 1.5 * 2^52
    const double t = fma(a, inv, shifter);
    const int q = __double2loint(t);                     // low word: the integer q
    const double qd = t - shifter;
    // ln2/256 = l2hi + l2lo, l2hi with 35 significant bits so that qd * l2hi
    // is exact for |q| < 2^18 (computed in 200-bit arithmetic)
    const double l2hi = 0x1.62e42fefc0000p-9, l2lo = -0x1.c610ca86c3899p-45;
    double r = fma(-qd, l2hi, a);
    r = fma(-qd, l2lo, r);
    // e^r - 1 = r + r^2/2 + r^3/6 + r^4/24
    double p = fma(r, 1.0 / 24.0, 1.0 / 6.0);
    p = fma(p, r, 0.5);
    p = fma(p, r, 1.0);
    p = p * r;
    const double tj = __ldg(&g_tables.exp2j[q & 255]);
    const double y = fma(tj, p, tj);
    // times 2^(q >> 8): add to the exponent field (no overflow for |a| < 512)
    const long long bits = __double_as_longlong(y) + (long long)(q >> 8) * (1LL << 52);
    return __longlong_as_double(bits);
}

// log(x) and 1/x together (x = Tref*T in the transport law)
__device__ __forceinline__ void log_rcp_t(double x, double &lg, double &rc)
{
    const long long bx = __double_as_longlong(x);
    const int ex = (int)((bx >> 52) & 0x7ff);
    // normal x with |log2 x| < 1000: 2^-e below stays normal
    if (ex < 23 || ex > 2023 || bx < 0) {
        lg = log(x);
        rc = 1.0 / x;
        return;
    }
    const int e = ex - 1023;
    const int j = (int)((bx >> 44) & 255);
    // m in [1,2): x with its exponent field set to 1023
    const double m = __longlong_as_double((bx & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
    const double c = __ldg(&g_tables.logc[j]);
    const double r = fma(m, c, -1.0);
    // log1p(r) = r - r^2/2 + r^3/3 - r^4/4 + r^5/5 - r^6/6
    double p = fma(r, -1.0 / 6.0, 0.2);
    p = fma(p, r, -0.25);
    p = fma(p, r, 1.0 / 3.0);
    p = fma(p, r, -0.5);
    p = p * r;
    p = fma(p, r, r);
    // e as a double without a conversion instruction: 2^52 + e, minus 2^52
    const double ed = __longlong_as_double(0x4330000000000000LL + (long long)(e + 1024)) -
                      (4503599627370496.0 + 1024.0);
    lg = fma(ed, 0x1.62e42fefa39efp-1, __ldg(&g_tables.lognc[j]) + p);   // e*ln2 + ...
    // 1/(1+r) - 1 = -r + r^2 - ... + r^6, Horner in -r
    const double nr = -r;
    double h = 1.0 + nr;
    h = fma(h, nr, 1.0);
    h = fma(h, nr, 1.0);
    h = fma(h, nr, 1.0);
    h = fma(h, nr, 1.0);
    h = h * nr;
    // 1/x = 2^-e * c * (1 + h), the power of two by exponent-field arithmetic
    const double cg = fma(c, h, c);
    rc = __longlong_as_double(__double_as_longlong(cg) - (long long)e * (1LL << 52));
}

}  // namespace fm
}  // namespace ns
