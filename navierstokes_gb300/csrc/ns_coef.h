// ns_coef.h -- the reference's coefficient tables and the host-side setup
// built from them, shared by every translation unit that sets up a step
// (ns_api.cu, ns_batch.cu, ns_noalloc.cu).  Host code only; no allocation:
// every builder writes into storage the caller owns.
//
// The numbers are the reference's own (they have to be, for parity):
//   DRP first derivative and its one-sided closures  init.f90:288-338
//   13-point selective filter df(0..6)                filtering.f90:54-66
//   boundary filter dfb(-1..5), REAL(8) in x          filtering.f90:25-31
//   the same, default-REAL (FP32) literals in y       filtering.f90:114-120
//   LDDRK alpha, beta and stage times c_k            rk.f90:27-46
//   Peclet number and conduction constant             global.f90:38-39
// ns_coef_table() (include/ns_gb300.h) exports them so that a test can
// compare them with the oracle's.
#pragma once

#include <cmath>
#include <cstring>

#include "ns_internal.cuh"

namespace ns {
namespace coef {

constexpr double kA[3] = {0.770882380518, -0.166705904415, 0.0208431427703};
constexpr double kA4[7] = {0.049041958000, -0.46884035700, -0.47476091400, 1.27327473700,
                           -0.51848452600, 0.16613853300,  -0.026369431000};
constexpr double kA4b[7] = {0.026369431000, -0.16613853300, 0.51848452600, -1.27327473700,
                            0.47476091400,  0.46884035700,  -0.049041958000};
constexpr double kA5[7] = {-0.20933762200, -1.08487567600, 2.14777605000, -1.38892832200,
                           0.76894976600,  -0.28181465000, 0.048230454000};
constexpr double kA5b[7] = {-0.048230454000, 0.28181465000,  -0.76894976600, 1.38892832200,
                            -2.14777605000,  1.08487567600, 0.20933762200};
constexpr double kA6[7] = {-2.19228033900, 4.74861140100, -5.10885191500, 4.46156710400,
                           -2.83349874100, 1.12832886100, -0.20387637100};
constexpr double kA6b[7] = {0.20387637100, -1.12832886100, 2.83349874100, -4.46156710400,
                            5.10885191500, -4.74861140100, 2.19228033900};
// df(0..6); the filter is symmetric, df(-s) = df(s)
constexpr double kDf[7] = {0.190899511506,  -0.171503832236, 0.123632891797, -0.069975429105,
                           0.029662754736, -0.008520738659, 0.001254597714};
constexpr double kDfbX[7] = {-0.057717512738, 0.199278374994,  -0.292668277650, 0.244537361546,
                             -0.134605018019, 0.056184263460, -0.015009191593};
constexpr double kDfbY[7] = {(double)-0.057717512738f, (double)0.199278374994f,
                             (double)-0.292668277650f, (double)0.244537361546f,
                             (double)-0.134605018019f, (double)0.056184263460f,
                             (double)-0.015009191593f};
constexpr double kAlpha[6] = {0.0, -0.737101392796, -1.634740794341,
                              -0.744739003780, -1.469897351522, -2.813971388035};
constexpr double kBeta[6] = {0.032918605146, 0.823256998200, 0.381530948900,
                             0.200092213184, 1.718581042715, 0.27};
constexpr double kCt[6] = {0.0, 0.032918605146, 0.249351723343,
                           0.466911705055, 0.582030414044, 0.847252983783};
constexpr double kPe = 1000.0, kAlphaCond = 0.5;

// Per-line derivative table of n positions (kCoefStride doubles each, see
// ns_internal.cuh) with 1/h and the 1-D metric folded in; mesh == nullptr:
// no metric.  With NS_METRIC_BANDS the metric applies in the D-point bands at
// both ends only (diff.f90:276-350 with meshx = 1 elsewhere).
inline void line_table(double *tab, int n, double h, const double *mesh, int D, int metric_mode)
{
    std::memset(tab, 0, sizeof(double) * kCoefStride * (size_t)n);
    for (int q = 0; q < n; q++) {
        double mt = 1.0;
        if (mesh && (metric_mode == NS_METRIC_EVERYWHERE || q < D || q >= n - D)) mt = mesh[q];
        double *c = tab + (size_t)q * kCoefStride;
        const double *src = q == 0 ? kA6 : q == 1 ? kA5 : q == 2 ? kA4 : q == n - 3 ? kA4b
                            : q == n - 2 ? kA5b : q == n - 1 ? kA6b : nullptr;
        if (src)
            for (int z = 0; z < 7; z++) c[z] = src[z] * mt / h;
        else
            for (int s = 0; s < 3; s++) c[4 + s] = kA[s] * mt / h;
    }
}

// Filter coefficients pre-multiplied by the strength sigmaf; dfb is kDfbX or
// kDfbY.
inline FilterCoef filter(double sigmaf, const double *dfb)
{
    FilterCoef f;
    std::memset(&f, 0, sizeof f);
    f.c0 = 1.0 - sigmaf * kDf[0];
    for (int s = 1; s <= 6; s++) f.m[s] = -sigmaf * kDf[s];
    f.bm1 = -sigmaf * dfb[0];
    f.b0 = 1.0 - sigmaf * dfb[1];
    for (int s = 1; s <= 5; s++) f.b[s] = -sigmaf * dfb[s + 1];
    return f;
}

// Warm-up length of a filter recurrence cut into pieces: the number of
// points after which the response of the homogeneous recurrence
// e(q) = -sigmaf * sum_{s=1..6} df(s) e(q-s) to any unit history stays below
// `thresh`, plus 8, and at least `floor`.  -1 when it never decays within
// 4096 points (the sweeps then run serially, one piece per line).  The
// FP64 sweeps use thresh = 2^-60 and floor 36; the FP32 ones 2^-50 (pairs)
// or 2^-32 and floor 16.
inline int warmup(double sigmaf, double thresh, int floor)
{
    constexpr int kMax = 4096;
    double e[kMax + 6];
    int worst = 0;
    for (int u = 0; u < 6; u++) {
        for (int q = 0; q < kMax + 6; q++) e[q] = 0.0;
        e[u] = 1.0;
        int last = 0;
        for (int q = 6; q < kMax + 6; q++) {
            double v = 0.0;
            for (int s = 1; s <= 6; s++) v += -sigmaf * kDf[s] * e[q - s];
            e[q] = v;
            if (std::fabs(v) >= thresh) last = q - 5;
        }
        if (last >= kMax - 64) return -1;
        if (last > worst) worst = last;
    }
    const int w = worst + 8;
    return w < floor ? floor : w;
}

// Warm-up of the FP64 sweeps cut into pieces.  A piece that starts from
// unfiltered history first runs warm32 steps in FP32, until the response to
// that history is below 2^-24 (the FP32 rounding), then warm - warm32 steps in
// FP64, until the response to the FP32 phase's rounding is below
// 2^-total_bits of the data: the same bound as an all-FP64 warm-up to that
// level, with most of the FP64 steps replaced by FP32 ones (for sigmaf = 0.2
// and the forward sweeps' 2^-60: 20 FP32 + 28 FP64 instead of 44 FP64).
// warm = -1 (serial sweeps) when the recurrence does not decay.
inline void fp64_warmups(double sigmaf, int &warm, int &warm32, int total_bits = 60)
{
    const int w32 = warmup(sigmaf, std::ldexp(1.0, -24), 0);
    const int w64 = warmup(sigmaf, std::ldexp(1.0, 24 - total_bits), 16);
    if (w32 < 0 || w64 < 0) {
        warm = -1;
        warm32 = 0;
        return;
    }
    warm32 = w32;
    warm = w32 + w64;
}

// The three in-place sweeps of lddfilterx/lddfiltery (filtering.f90:39-94)
// on one contiguous line of n values, serially, in FP64.
inline void serial_filter_line(double *u, int n, double sigmaf, const double *dfb)
{
    for (int q = 1; q <= 6; q++) {
        double Du = 0.0;
        for (int s = -1; s <= 5; s++) Du += dfb[s + 1] * u[q + s];
        u[q] -= sigmaf * Du;
    }
    for (int q = 6; q <= n - 7; q++) {
        double Du = 0.0;
        for (int s = -6; s <= 6; s++) Du += kDf[s < 0 ? -s : s] * u[q + s];
        u[q] -= sigmaf * Du;
    }
    for (int q = n - 2; q >= n - 7; q--) {
        double Du = 0.0;
        for (int s = -1; s <= 5; s++) Du += dfb[s + 1] * u[q - s];
        u[q] -= sigmaf * Du;
    }
}

}  // namespace coef
}  // namespace ns
