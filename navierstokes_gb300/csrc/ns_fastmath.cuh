// ns_fastmath.cuh -- exp, log and 1/x for the transport law mu(T), k(T)
// (coefficients.f90:27-59), with fewer FP64-pipe instructions than the
// general library functions (the FP64 pipe bounds the stage kernels).
//
// Written from the table-driven method of P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989, and "... of the logarithm function",
// ACM TOMS 16(4), 1990, with Taylor polynomials on the reduced intervals:
//
//   exp(a) = 2^(q/64) * e^r,  q = nearest integer to 64*a/ln2,
//            |r| <= ln2/128 = 0.0054; 2^(j/64) (j = q mod 64) from a table,
//            e^r - 1 by its Taylor polynomial of degree 5 (remainder
//            r^6/720 < 3.5e-17 relative).
//   x = 2^e * m, m in [1,2); j = the top 7 fraction bits of m;
//   c_j = 1/(1 + (j + 1/2)/128) rounded to 12 significant bits, so that
//   r = m*c_j - 1 (one FMA) has |r| < 2^-8;
//   log(x) = e*ln2 - log(c_j) + log1p(r), log1p by its Taylor polynomial of
//            degree 7 (remainder r^8/8 < 2^-67);
//   1/x    = 2^-e * c_j / (1 + r), 1/(1+r) by its geometric series to
//            degree 7 (remainder r^8 < 2^-63 relative).
//
// The tables are filled on the host (std::exp2, std::log) by
// ns::ensure_math_tables before the first launch on a device; they are a
// __device__ variable of ns_kernels.cu, the one translation unit that
// includes this header.  Arguments
// outside the ranges the reduction handles (non-finite, x <= 0 or
// subnormal or |log2 x| >= 1000, |a| > 700) take the library functions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ns {
namespace fm {

struct Tables {
    double exp2j[64];    // 2^(j/64)
    double logc[128];    // c_j
    double lognc[128];   // -log(c_j)
};

// filled by ensure_math_tables (ns_kernels.cu, the only includer)
static __device__ Tables g_tables;

__device__ __forceinline__ double exp_t(double a)
{
    if (!(fabs(a) <= 700.0)) return exp(a);
    const double inv = 0x1.71547652b82fep+6;             // 64 / ln 2
    const double shifter = 0x1.8p52;                     // 1.5 * 2^52
    const double t = fma(a, inv, shifter);
    const int q = __double2loint(t);                     // low word: the integer q
    const double qd = t - shifter;
    // ln2/64 = l2hi + l2lo, l2hi with 36 significant bits so that qd * l2hi
    // is exact for |q| < 2^17 (computed in 200-bit arithmetic)
    const double l2hi = 0x1.62e42fefa0000p-7, l2lo = 0x1.cf79abc9e3b3ap-46;
    double r = fma(-qd, l2hi, a);
    r = fma(-qd, l2lo, r);
    // e^r - 1 = r + r^2/2 + r^3/6 + r^4/24 + r^5/120
    double p = fma(r, 1.0 / 120.0, 1.0 / 24.0);
    p = fma(p, r, 1.0 / 6.0);
    p = fma(p, r, 0.5);
    p = fma(p, r, 1.0);
    p = p * r;
    const double tj = __ldg(&g_tables.exp2j[q & 63]);
    const double y = fma(tj, p, tj);
    // times 2^(q >> 6): add to the exponent field (no overflow for |a| <= 700)
    const long long bits = __double_as_longlong(y) + (long long)(q >> 6) * (1LL << 52);
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
    const int j = (int)((bx >> 45) & 127);
    // m in [1,2): x with its exponent field set to 1023
    const double m = __longlong_as_double((bx & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
    const double c = __ldg(&g_tables.logc[j]);
    const double r = fma(m, c, -1.0);
    // log1p(r) = r - r^2/2 + r^3/3 - r^4/4 + r^5/5 - r^6/6 + r^7/7
    double p = fma(r, 1.0 / 7.0, -1.0 / 6.0);
    p = fma(p, r, 1.0 / 5.0);
    p = fma(p, r, -0.25);
    p = fma(p, r, 1.0 / 3.0);
    p = fma(p, r, -0.5);
    p = p * r;
    p = fma(p, r, r);
    // e as a double without a conversion instruction: 2^52 + e, minus 2^52
    const double ed = __longlong_as_double(0x4330000000000000LL + (long long)(e + 1024)) -
                      (4503599627370496.0 + 1024.0);
    // ln 2 = ln2hi + ln2lo, ln2hi with 40 significant bits (ed * ln2hi exact)
    const double ln2hi = 0x1.62e42fefa4000p-1, ln2lo = -0x1.8432a1b0e2634p-43;
    const double hi = fma(ed, ln2hi, __ldg(&g_tables.lognc[j]));
    lg = hi + fma(ed, ln2lo, p);
    // 1/(1+r) - 1 = -r + r^2 - ... - r^7, Horner in -r
    const double nr = -r;
    double h = 1.0 + nr;
    h = fma(h, nr, 1.0);
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
