// ns_kernels.cu -- FP64 stage kernels of the LDDRK step (rk.f90:12-75).
//
// On GB300 the FP64 pipe (about 1.2 TFLOP/s, 1.9 DFMA/clk/SM) binds long
// before HBM does, so the stage is split into kernels that never recompute
// an FP64 quantity: every intermediate the reference keeps in module arrays
// (TEMP, dUdm/dUdn, TAU, k*dT, psiDiff) is written once to HBM and read
// back by the next kernel.  Per stage:
//
//   k_prim    (NS only)  T = gamma*p/rho, 1/rho              rhs.f90:20
//   k_first              dU/dx, dU/dy (DRP + closures + metric), mu(T),
//                        k(T), k*dT/dx, k*dT/dy, tau, psiDiff
//                        diff.f90:6-151,276-350; derivs.f90:9-56;
//                        coefficients.f90:27-59; eqeuler.f90:28-47
//   k_update             second derivatives, EULERNONLINEAR, rk_steep,
//                        bufferxy                  eqeuler.f90:53-99;
//                                                  rk.f90:77-169
//   k_filter<x>          lddfilterx as chunked recurrences  filtering.f90:9-96
//   k_filter<y>          lddfiltery                         filtering.f90:98-190
//   k_bc                 ccpml                              cc.f90:6-68
#include <algorithm>
#include <cmath>
#include <mutex>

#include "ns_fastmath.cuh"
#include "ns_internal.cuh"
#include "ns_check.cuh"
#include "ns_tma.cuh"

namespace ns {

cudaError_t ensure_math_tables(int device)
{
    static std::mutex mu;
    static bool done[1024];
    std::lock_guard<std::mutex> lock(mu);
    if (device < 0 || device >= 1024) return cudaErrorInvalidDevice;
    if (done[device]) return cudaSuccess;
    fm::Tables t;
    for (int j = 0; j < 256; j++) t.exp2j[j] = std::exp2(j / 256.0);
    for (int j = 0; j < 256; j++) {
        // 1/(1 + (j + 1/2)/256) rounded to 12 significant bits
        const double c = std::ldexp(std::nearbyint(std::ldexp(1.0 / (1.0 + (j + 0.5) / 256.0), 12)), -12);
        t.logc[j] = c;
        t.lognc[j] = -std::log(c);
    }
    int cur = 0;
    cudaError_t e = cudaGetDevice(&cur);
    if (e == cudaSuccess && cur != device) e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(fm::g_tables, &t, sizeof t);
    if (cur != device) cudaSetDevice(cur);
    if (e == cudaSuccess) done[device] = true;
    return e;
}

__global__ void k_math_eval(int fn, const double *__restrict__ x, double *__restrict__ y, int n)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    if (fn == 0) {
        y[q] = fm::exp_t(x[q]);
    } else {
        double lg, rc;
        fm::log_rcp_t(x[q], lg, rc);
        y[q] = (fn == 1) ? lg : rc;
    }
}

cudaError_t launch_math_eval(int fn, const double *x, double *y, int n, cudaStream_t s)
{
    k_math_eval<<<(n + 255) / 256, 256, 0, s>>>(fn, x, y, n);
    return cudaGetLastError();
}

// mu(T) and k(T), 1/mu0 and 1/k0 included (coefficients.f90:27-59): from
// the piecewise-polynomial table when T lies in its range (11 FP64
// instructions), else by the table-driven log, 1/x and exp (43).
__device__ __forceinline__ void transport(double T, const double *__restrict__ trtab,
                                          const Physics &ph, double &mu, double &kc)
{
    const long long bt = __double_as_longlong(T);
    const int e = (int)(bt >> 52) - 1023;  // the exponent when T > 0
    if (trtab && bt > 0 && e >= kTrEmin && e < kTrEmin + kTrOctaves) {
        const int piece = ((e - kTrEmin) << 8) | (int)((bt >> 44) & 255);
        // T minus the piece's left end: the same exponent, so exact
        const double u = T - __longlong_as_double(bt & ~((1LL << 44) - 1));
        const double2 *c = reinterpret_cast<const double2 *>(trtab + (size_t)piece * kTrStride);
        const double2 m01 = __ldg(c), m23 = __ldg(c + 1), m45 = __ldg(c + 2);
        const double2 k01 = __ldg(c + 3), k23 = __ldg(c + 4), k45 = __ldg(c + 5);
        mu = fma(fma(fma(fma(fma(m45.y, u, m45.x), u, m23.y), u, m23.x), u, m01.y), u, m01.x);
        kc = fma(fma(fma(fma(fma(k45.y, u, k45.x), u, k23.y), u, k23.x), u, k01.y), u, k01.x);
        return;
    }
    const double x = ph.Tref * T;
    double L, y;
    fm::log_rcp_t(x, L, y);  // log(x), 1/x
    // 1/mu0 and 1/k0 enter as log(1/mu0) + D, log(1/k0) + D (Physics)
    const double amu = fma(ph.A_mi, L, fma(fma(ph.C_mi, y, ph.B_mi), y, ph.D_mi_s));
    const double ak = fma(ph.A_k, L, fma(fma(ph.C_k, y, ph.B_k), y, ph.D_k_s));
    mu = fm::exp_t(amu);
    kc = fm::exp_t(ak);
}

__global__ void k_transport_eval(const double *__restrict__ T, const double *__restrict__ trtab,
                                 Physics ph, double *__restrict__ mu, double *__restrict__ k,
                                 int n)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    double m, kc;
    transport(T[q], trtab, ph, m, kc);
    mu[q] = m;
    k[q] = kc;
}

cudaError_t launch_transport_eval(const ns_ctx *c, const double *T, double *mu, double *k, int n,
                                  cudaStream_t s)
{
    k_transport_eval<<<(n + 255) / 256, 256, 0, s>>>(T, c->trtab, c->phys, mu, k, n);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// k_prim: T and 1/rho (rhs.f90:20), pointwise.
// ---------------------------------------------------------------------------
// Rows row0 .. row0+rows-1 (the whole grid in the step graph).
__global__ void __launch_bounds__(256) k_prim(Dims d, const double *__restrict__ U,
                                              double *__restrict__ aux, double gamma, int row0,
                                              int rows)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = row0 + blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= d.imax || j >= row0 + rows) return;
    const long long idx = (long long)j * d.pitch + i;
    const double rho = U[idx];
    const double p = U[3 * d.plane + idx];
    const double ri = 1.0 / rho;
    aux[AUX_RINV * d.plane + idx] = ri;
    aux[AUX_T * d.plane + idx] = (gamma * p) * ri;
}

// ---------------------------------------------------------------------------
// k_first: first derivatives and everything pointwise built from them.
// ---------------------------------------------------------------------------
// With TMA, one elected thread loads the block's halo tile of U (and of T)
// into shared memory and the interior stencils read it there; the closure
// points near the domain edges read global memory.  Both give identical bits.
// Rows row0 .. row0+rows-1 (the whole grid in the step graph).
template <bool VISC, int NK, bool TMA>
__global__ void __launch_bounds__(256)
    k_first(const __grid_constant__ CUtensorMap umap, const __grid_constant__ CUtensorMap tmap,
            int *__restrict__ err, Dims d, const double *__restrict__ U,
            double *__restrict__ dudm, double *__restrict__ dudn, double *__restrict__ aux,
            const double *__restrict__ xcoef, const double *__restrict__ ycoef,
            const double *__restrict__ trtab, Physics ph, int row0, int rows)
{
    constexpr int TW = kFirstTileW, TH = kFirstTileH;
    __shared__ alignas(128) double su[TMA ? NK : 1][TMA ? TH : 1][TMA ? TW : 1];
    __shared__ alignas(128) double sT[TMA && VISC ? TH : 1][TMA && VISC ? TW : 1];
    __shared__ alignas(8) unsigned long long tbar;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i = blockIdx.x * kFirstBX + tx;
    const int j = row0 + blockIdx.y * kFirstBY + ty;
    // the tile indices below assume this launch shape; the TMA box's x must
    // be a multiple of 16 bytes (an even number of doubles)
    NS_CHECK(err, kChkKernels, blockDim.x == kFirstBX && blockDim.y == kFirstBY);
    NS_CHECK(err, kChkKernels, ((blockIdx.x * kFirstBX - kFirstTileL) & 1) == 0);
    NS_CHECK(err, kChkKernels, row0 >= 0 && row0 + rows <= d.jmax && d.imax >= 7 && d.jmax >= 7);
    if constexpr (TMA) {
        const bool lead = (tx == 0 && ty == 0);
        if (lead) mbar_init(&tbar, 1);
        __syncthreads();
        if (lead) {
            // boxes at (i0-4, j0-3): points outside the grid read as zero and
            // are never used (their neighbours take the closure branch)
            const int x0 = blockIdx.x * kFirstBX - kFirstTileL;
            const int y0 = row0 + blockIdx.y * kFirstBY - 3;
            mbar_expect_tx(&tbar, (unsigned)(sizeof(su) + (VISC ? sizeof(sT) : 0)));
            tma_load_3d(&su[0][0][0], &umap, x0, y0, 0, &tbar);
            if (VISC) tma_load_3d(&sT[0][0], &tmap, x0, y0, 0, &tbar);
        }
        if (!mbar_wait_bounded(&tbar, 0, err)) return;
    }
    if (i >= d.imax || j >= row0 + rows) return;
    const long long idx = (long long)j * d.pitch + i;
    const long long P = d.plane, st = d.pitch;
    const double *cx = xcoef + kCoefStride * i;
    const double *cy = ycoef + kCoefStride * j;
    const double cx1 = cx[4], cx2 = cx[5], cx3 = cx[6];
    const double cy1 = cy[4], cy2 = cy[5], cy3 = cy[6];
    const bool xin = TMA && i >= 3 && i < d.imax - 3;
    const bool yin = TMA && j >= 3 && j < d.jmax - 3;
    const int sr = ty + 3, sc = tx + kFirstTileL;
    double gx[NK], gy[NK];
#pragma unroll
    for (int k = 0; k < NK; k++) {
        const double *f = U + k * P + idx;
        const double *t = &su[TMA ? k : 0][TMA ? sr : 0][TMA ? sc : 0];
        gx[k] = xin ? dint(t, 1, cx1, cx2, cx3) : dline(f, 1, i, d.imax, cx);
        gy[k] = yin ? dint(t, TW, cy1, cy2, cy3) : dline(f, st, j, d.jmax, cy);
        dudm[k * P + idx] = gx[k];
        dudn[k * P + idx] = gy[k];
    }
    if (VISC) {
        // dT/dx, dT/dy (derivs.f90:25-26), mu(T), k(T) (coefficients.f90:27-59)
        const double *fT = aux + AUX_T * P + idx;
        const double *t = &sT[TMA ? sr : 0][TMA ? sc : 0];
        const double T = TMA ? t[0] : fT[0];
        const double Tx = xin ? dint(t, 1, cx1, cx2, cx3) : dline(fT, 1, i, d.imax, cx);
        const double Ty = yin ? dint(t, TW, cy1, cy2, cy3) : dline(fT, st, j, d.jmax, cy);
        double mu, kc;
        transport(T, trtab, ph, mu, kc);
        aux[AUX_KTX * P + idx] = Tx * kc;  // kdT (derivs.f90:48-56)
        aux[AUX_KTY * P + idx] = Ty * kc;
        // TAU_IJ (eqeuler.f90:37-39)
        const double div = gx[1] + gy[2];
        const double m23 = (2.0 / 3.0) * mu;
        const double mu2 = 2.0 * mu;
        aux[AUX_TAU1 * P + idx] = fma(mu2, gx[1], -(m23 * div));
        aux[AUX_TAU2 * P + idx] = mu * (gy[1] + gx[2]);
        aux[AUX_TAU3 * P + idx] = fma(mu2, gy[2], -(m23 * div));
    }
    if (NK >= 5) {
        const double rho = TMA ? su[0][sr][sc] : U[idx];
        aux[AUX_PSID * P + idx] = (rho * ph.alpha_cond) * (gx[NK - 1] + gy[NK - 1]);
    }
}

// ---------------------------------------------------------------------------
// k_update: second-level derivatives, EULERNONLINEAR (eqeuler.f90:53-99),
// rk_steep on the interior (rk.f90:153-169) and bufferxy on the bands
// (rk.f90:77-151), all points of the grid.
// ---------------------------------------------------------------------------
// Planes of aux whose derivatives k_update takes: tau1, tau2, tau3, k dT/dx,
// k dT/dy (viscous) and psiDiff (nk = 5), consecutive from kAuxTileZ0.
template <bool VISC, int NK>
constexpr int kAuxTileZ0 = VISC ? AUX_TAU1 : AUX_PSID;
template <bool VISC, int NK>
constexpr int kAuxTilePlanes = (VISC ? 5 : 0) + (NK >= 5 ? 1 : 0);

// With TMA, the halo tile of those planes arrives in shared memory while the
// pointwise inputs load; interior stencils read it there, closures read
// global memory (identical bits either way).
template <bool VISC, int NK, bool FIRST, bool SRC, bool TMA>
__global__ void __launch_bounds__(256)
    k_update(const __grid_constant__ CUtensorMap amap, int *__restrict__ err, Dims d,
             double *__restrict__ U, double *__restrict__ W,
             const double *__restrict__ dudm, const double *__restrict__ dudn,
             const double *__restrict__ aux, const double *__restrict__ xcoef,
             const double *__restrict__ ycoef, const double *__restrict__ Ubase,
             const double *__restrict__ sigx, const double *__restrict__ sigy,
             const double *__restrict__ src, const double *__restrict__ stage_sin, Physics ph,
             StageCoef sc)
{
    constexpr int TW = kFirstTileW, TH = kFirstTileH;
    constexpr int NZ = TMA ? kAuxTilePlanes<VISC, NK> : 1;
    static_assert(!TMA || kAuxTilePlanes<VISC, NK> > 0, "no aux tile to load");
    // sa[z] = aux plane kAuxTileZ0 + z
    __shared__ alignas(128) double sa[NZ][TMA ? TH : 1][TMA ? TW : 1];
    __shared__ alignas(8) unsigned long long tbar;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i = blockIdx.x * kFirstBX + tx;
    const int j = blockIdx.y * kFirstBY + ty;
    const bool lead = (tx == 0 && ty == 0);
    NS_CHECK(err, kChkKernels, blockDim.x == kFirstBX && blockDim.y == kFirstBY);
    NS_CHECK(err, kChkKernels, ((blockIdx.x * kFirstBX - kFirstTileL) & 1) == 0);
    NS_CHECK(err, kChkKernels, d.imax >= 7 && d.jmax >= 7 && d.pitch >= d.imax);
    if constexpr (TMA) {
        if (lead) mbar_init(&tbar, 1);
        __syncthreads();
        if (lead) {
            mbar_expect_tx(&tbar, (unsigned)sizeof(sa));
            tma_load_3d(&sa[0][0][0], &amap, blockIdx.x * kFirstBX - kFirstTileL,
                        blockIdx.y * kFirstBY - 3, kAuxTileZ0<VISC, NK>, &tbar);
        }
    }
    const bool valid = i < d.imax && j < d.jmax;
    const long long idx = (long long)j * d.pitch + i;
    const long long P = d.plane, st = d.pitch;
    double u[NK];
    if (valid) {
#pragma unroll
        for (int k = 0; k < NK; k++) u[k] = U[k * P + idx];
    }
    // every thread waits, so no block exits with its tile load in flight
    if constexpr (TMA)
        if (!mbar_wait_bounded(&tbar, 0, err)) return;
    if (!valid) return;
    const bool xin = TMA && i >= 3 && i < d.imax - 3;
    const bool yin = TMA && j >= 3 && j < d.jmax - 3;
    const int sr = ty + 3, scol = tx + kFirstTileL;
    // tile point of aux plane `a` at this thread's point
    auto tp = [&](int a) {
        return &sa[TMA ? a - kAuxTileZ0<VISC, NK> : 0][TMA ? sr : 0][TMA ? scol : 0];
    };

    const bool interior = (i > 0) && (i < d.imax - 1) && (j > 0) && (j < d.jmax - 1);
    if (interior) {
        double gx[NK], gy[NK];
#pragma unroll
        for (int k = 0; k < NK; k++) {
            gx[k] = dudm[k * P + idx];
            gy[k] = dudn[k * P + idx];
        }
        const double rho = u[0], uu = u[1], vv = u[2], pp = u[3];
        const double ri = VISC ? aux[AUX_RINV * P + idx] : 1.0 / rho;
        double r[NK];
        // DUDT(1), eqeuler.f90:63
        double t = uu * gx[0];
        t = fma(rho, gx[1], t);
        t = fma(vv, gy[0], t);
        t = fma(rho, gy[2], t);
        r[0] = -t;
        // DUDT(2), :68
        double a2 = uu * gx[1];
        a2 = fma(ri, gx[3], a2);
        a2 = fma(vv, gy[1], a2);
        // DUDT(3), :74
        double a3 = uu * gx[2];
        a3 = fma(vv, gy[2], a3);
        a3 = fma(ri, gy[3], a3);
        // DUDT(4), :80-92
        const double gp = ph.gamma * pp;
        double a4 = gp * gx[1];
        a4 = fma(uu, gx[3], a4);
        a4 = fma(gp, gy[2], a4);
        a4 = fma(vv, gy[3], a4);
        if (SRC) {
            const double s = stage_sin[sc.stage] * src[idx];
            a4 = a4 - s;
        }
        const double *cx = xcoef + kCoefStride * i;
        const double *cy = ycoef + kCoefStride * j;
        const double cx1 = cx[4], cx2 = cx[5], cx3 = cx[6];
        const double cy1 = cy[4], cy2 = cy[5], cy3 = cy[6];
        // d/dx of aux plane ax (global: gax) plus d/dy of plane ay (gay): in
        // the interior one FMA chain over both stencils from the tile (one
        // addition fewer), at the closures the two sums of dline
        auto dxy = [&](int ax, const double *gax, int ay, const double *gay) -> double {
            if (xin && yin) {
                const double *a = tp(ax), *b = tp(ay);
                double r = cx1 * (a[1] - a[-1]);
                r = fma(cx2, a[2] - a[-2], r);
                r = fma(cx3, a[3] - a[-3], r);
                r = fma(cy1, b[TW] - b[-TW], r);
                r = fma(cy2, b[2 * TW] - b[-2 * TW], r);
                r = fma(cy3, b[3 * TW] - b[-3 * TW], r);
                return r;
            }
            return (xin ? dint(tp(ax), 1, cx1, cx2, cx3) : dline(gax, 1, i, d.imax, cx)) +
                   (yin ? dint(tp(ay), TW, cy1, cy2, cy3) : dline(gay, st, j, d.jmax, cy));
        };
        if (VISC) {
            const double *t1 = aux + AUX_TAU1 * P + idx;
            const double *t2 = aux + AUX_TAU2 * P + idx;
            const double *t3 = aux + AUX_TAU3 * P + idx;
            const double *s1 = tp(AUX_TAU1), *s2 = tp(AUX_TAU2), *s3 = tp(AUX_TAU3);
            const double dtau_u = dxy(AUX_TAU1, t1, AUX_TAU2, t2);  // dtau11/dx + dtau12/dy
            const double dtau_v = dxy(AUX_TAU2, t2, AUX_TAU3, t3);  // dtau12/dx + dtau22/dy
            const double d2T = dxy(AUX_KTX, aux + AUX_KTX * P + idx, AUX_KTY,
                                   aux + AUX_KTY * P + idx);
            const double rv = ph.inv_re * ri;
            a2 = fma(-rv, dtau_u, a2);
            a3 = fma(-rv, dtau_v, a3);
            const double tau1 = TMA ? s1[0] : t1[0];
            const double tau2 = TMA ? s2[0] : t2[0];
            const double tau3 = TMA ? s3[0] : t3[0];
            double phi = gx[1] * tau1;
            phi = fma(gx[2], tau2, phi);
            phi = fma(gy[1], tau2, phi);
            phi = fma(gy[2], tau3, phi);
            a4 = fma(-ph.gm1_re, phi, a4);
            a4 = fma(-ph.inv_re_pr, d2T, a4);
        }
        r[1] = -a2;
        r[2] = -a3;
        r[3] = -a4;
        if (NK >= 5) {
            // DUDT(5), :94-95
            const double *pd = aux + AUX_PSID * P + idx;
            const double d2p = dxy(AUX_PSID, pd, AUX_PSID, pd);
            double a5 = uu * gx[NK - 1];
            a5 = fma(vv, gy[NK - 1], a5);
            a5 = fma(-(ph.inv_pe * ri), d2p, a5);
            r[NK - 1] = -a5;
        }
        // rk_steep (rk.f90:163-164)
#pragma unroll
        for (int k = 0; k < NK; k++) {
            double w;
            if (FIRST)
                w = ph.dt * r[k];
            else
                w = fma(sc.alpha, W[k * P + idx], ph.dt * r[k]);
            W[k * P + idx] = w;
            u[k] = fma(sc.beta, w, u[k]);
        }
    }
    // bufferxy: buffery then bufferx at each point (rk.f90:86-105, :123, :145)
    const bool by = (j < d.D) || (j >= d.jmax - d.D);
    const bool bx = (i < d.D) || (i >= d.imax - d.D);
    if (by || bx) {
        double ub[NK];
#pragma unroll
        for (int k = 0; k < NK; k++) ub[k] = Ubase[k * P + idx];
        if (by) {
            const double s = sigy[j];
#pragma unroll
            for (int k = 0; k < NK; k++) u[k] = fma(s, u[k] - ub[k], ub[k]);
        }
        if (bx) {
            const double s = sigx[i];
#pragma unroll
            for (int k = 0; k < NK; k++) u[k] = fma(s, u[k] - ub[k], ub[k]);
        }
    }
    if (interior || by || bx) {
#pragma unroll
        for (int k = 0; k < NK; k++) U[k * P + idx] = u[k];
    }
}

// ---------------------------------------------------------------------------
// k_filter: the in-place selective filter sweeps of filtering.f90 along x
// (ALONG_Y = false) or y, out of place (src -> dst).
//
// Each line (k,j) or (k,i) is one recurrence: pass 1 ascends positions
// 1..6 with the 7-point boundary filter, pass 2 ascends 6..n-7 with the
// 13-point filter, pass 3 descends n-2..n-7 with the mirrored boundary
// filter; each point's stencil reads the already-filtered points before it
// (0-based positions; the reference's i = q+1).  A line is split into
// chunks over pass 2.  A chunk whose start lies more than `warm` points
// past position 6 starts the recurrence `warm` points early from unfiltered
// history; the error of that history decays by the spectral radius of the
// recurrence at every point, and `warm` is chosen on the host so that it
// falls below 2^-60 of the data before the chunk's first output.
// ---------------------------------------------------------------------------
// One pass-2 point: w[0..5] filtered points q-6..q-1, w[6..12] unfiltered
// points q..q+6.
__device__ __forceinline__ double filter13(const FilterCoef &fc, const double *w)
{
    double v = fc.c0 * w[6];
    v = fma(fc.m[6], w[12] + w[0], v);
    v = fma(fc.m[5], w[11] + w[1], v);
    v = fma(fc.m[4], w[10] + w[2], v);
    v = fma(fc.m[3], w[9] + w[3], v);
    v = fma(fc.m[2], w[8] + w[4], v);
    v = fma(fc.m[1], w[7], v);
    v = fma(fc.m[1], w[5], v);
    return v;
}

// Slides the window one point: v becomes filtered point q, `next` is
// unfiltered point q+7.
__device__ __forceinline__ void shift13(double *w, double v, double next)
{
#pragma unroll
    for (int t = 0; t < 5; t++) w[t] = w[t + 1];
    w[5] = v;
#pragma unroll
    for (int t = 6; t < 12; t++) w[t] = w[t + 1];
    w[12] = next;
}

// The pass-2 point of filter13 in FP32 (the first steps of a warm start);
// cf = c0, m[1..6] rounded to FP32.
__device__ __forceinline__ float filter13_f(const float *cf, const float *w)
{
    float v = cf[0] * w[6];
    v = fmaf(cf[6], w[12] + w[0], v);
    v = fmaf(cf[5], w[11] + w[1], v);
    v = fmaf(cf[4], w[10] + w[2], v);
    v = fmaf(cf[3], w[9] + w[3], v);
    v = fmaf(cf[2], w[8] + w[4], v);
    v = fmaf(cf[1], w[7], v);
    return fmaf(cf[1], w[5], v);
}

// Pass-2 positions [a, b) of one line (6 <= a < b <= n-6): a == 6 starts
// exactly with pass 1 and writes its outputs, a later start runs `warm`
// points of unfiltered history first (or starts exactly when that reaches
// back to position 6), the first warm32 of them in FP32; b == n-6 ends with
// pass 3.
__device__ __forceinline__ void filter_piece(const double *__restrict__ s, double *__restrict__ o,
                                             long long st, int n, int a, int b, int warm,
                                             int warm32, const FilterCoef &fc, int *err)
{
    // positions read: 0..12 (exact start) or a-warm-6 .. , ahead up to n-1;
    // written: a .. b-1 and the pass-1/pass-3 ends
    NS_CHECK(err, kChkKernels, n >= 13 && 6 <= a && a < b && b <= n - 6);
    double w[13];
    int q;
    if (a == 6 || warm < 0 || a - warm <= 6) {
        // exact start: pass 1 (filtering.f90:39-49 / :128-140)
#pragma unroll
        for (int t = 0; t < 13; t++) w[t] = s[t * st];
#pragma unroll
        for (int p = 1; p <= 6; p++) {
            double v = fc.b0 * w[p];
#pragma unroll
            for (int z = 1; z <= 5; z++) v = fma(fc.b[z], w[p + z], v);
            v = fma(fc.bm1, w[p - 1], v);
            w[p] = v;
        }
        if (a == 6) {
#pragma unroll
            for (int p = 0; p < 6; p++) o[p * st] = w[p];
        }
        q = 6;
    } else {
        q = a - warm;
        // the history's own error decays below the FP32 rounding in the
        // first warm32 steps, which therefore run in FP32; the FP64 steps
        // after them take that rounding below 2^-60
        float wf[13], cf[7];
        cf[0] = (float)fc.c0;
#pragma unroll
        for (int z = 1; z < 7; z++) cf[z] = (float)fc.m[z];
#pragma unroll
        for (int t = 0; t < 13; t++) wf[t] = (float)s[(long long)(q - 6 + t) * st];
        for (const int qe = q + warm32; q < qe; q++) {
            const float v = filter13_f(cf, wf);
#pragma unroll
            for (int t = 0; t < 5; t++) wf[t] = wf[t + 1];
            wf[5] = v;
#pragma unroll
            for (int t = 6; t < 12; t++) wf[t] = wf[t + 1];
            wf[12] = (float)s[(long long)(q + 7) * st];
        }
#pragma unroll
        for (int t = 0; t < 13; t++) w[t] = (double)wf[t];
    }
    // pass 2 (filtering.f90:69-79 / :161-171).  Blocks of kFilterPf points,
    // the next block's input loaded before the current block is filtered, so
    // that a thread keeps kFilterPf loads in flight.
    double nx[kFilterPf];
#pragma unroll
    for (int t = 0; t < kFilterPf; t++) {
        const int r = q + 7 + t;
        nx[t] = (r < n) ? s[(long long)r * st] : 0.0;
    }
    for (; q + kFilterPf <= b; q += kFilterPf) {
        double cur[kFilterPf];
#pragma unroll
        for (int t = 0; t < kFilterPf; t++) {
            cur[t] = nx[t];
            const int r = q + kFilterPf + 7 + t;
            nx[t] = (r < n) ? s[(long long)r * st] : 0.0;
        }
#pragma unroll
        for (int t = 0; t < kFilterPf; t++) {
            const double v = filter13(fc, w);
            if (q + t >= a) o[(long long)(q + t) * st] = v;
            shift13(w, v, cur[t]);
        }
    }
    for (; q < b; q++) {
        const double v = filter13(fc, w);
        if (q >= a) o[(long long)q * st] = v;
        shift13(w, v, (q + 7 < n) ? s[(long long)(q + 7) * st] : 0.0);
    }
    if (b == n - 6) {
        // pass 3 (filtering.f90:84-94 / :176-188): w[0..11] = positions n-12..n-1
#pragma unroll
        for (int x = 10; x >= 5; x--) {
            double v = fc.b0 * w[x];
#pragma unroll
            for (int z = 1; z <= 5; z++) v = fma(fc.b[z], w[x - z], v);
            v = fma(fc.bm1, w[x + 1], v);
            w[x] = v;
        }
#pragma unroll
        for (int x = 5; x < 12; x++) o[(long long)(n - 12 + x) * st] = w[x];
    }
}

// Work is dealt out in warp-lines: 32 adjacent lines of one variable (rows
// j for x, columns i for y), one per lane, so a warp's loads and stores of a
// position are 32 neighbouring lines and every lane takes the same branches.
// The pass-2 positions of all warp-lines, laid end to end, are cut into equal
// segments of `seg` positions, one per warp: a segment covers the end of one
// warp-line and the start of the next, each piece with its own start (exact
// or warm) and end (pass 3 or not).  Equal segments give every warp the same
// work up to one warm-up, whatever the number of lines.
template <bool ALONG_Y>
__global__ void __launch_bounds__(128)
    k_filter(Dims d, const double *__restrict__ src, double *__restrict__ dst, long long seg,
             int warm, int warm32, FilterCoef fc, int *err, int p0, int len2)
{
    const int lane = threadIdx.x & 31;
    const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nlines = ALONG_Y ? d.imax : d.jmax;  // lines per variable
    const int gpk = (nlines + 31) >> 5;            // warp-lines per variable
    const int n = ALONG_Y ? d.jmax : d.imax;
    // pass-2 positions p0 .. p0+len2-1: all of them (6 .. n-7), or one row
    // band of ns_rk_euler's last y sweep
    NS_CHECK(err, kChkKernels, p0 >= 6 && len2 >= 1 && p0 + len2 <= n - 6);
    const long long total = (long long)gpk * d.nk * len2;
    const long long s0 = wid * seg;
    const long long s1 = s0 + seg < total ? s0 + seg : total;
    const long long st = ALONG_Y ? d.pitch : 1;
    for (long long sp = s0; sp < s1;) {
        const long long g = sp / len2;
        const long long gend = (g + 1) * len2;
        const long long e = s1 < gend ? s1 : gend;
        const int k = (int)(g / gpk);
        const int line = (int)(g % gpk) * 32 + lane;
        NS_CHECK(err, kChkKernels, k >= 0 && k < d.nk && sp >= g * len2 && e > sp && e <= gend);
        if (line < nlines) {
            const long long base =
                (long long)k * d.plane + (ALONG_Y ? line : (long long)line * d.pitch);
            // the line's last point stays inside plane k
            NS_CHECK(err, kChkKernels, base + (long long)(n - 1) * st < (long long)(k + 1) * d.plane);
            filter_piece(src + base, dst + base, st, n, p0 + (int)(sp - g * len2),
                         p0 + (int)(e - g * len2), warm, warm32, fc, err);
        }
        sp = e;
    }
}

// Launch shape of k_filter: one warp per SM sub-partition, or kw when the
// segments stay long against the warm-up (at least 8x; a second warp per
// sub-partition hides latency but adds a warm-up to every segment); whole
// warp-lines per warp when the warm-up is unbounded (warm < 0).  A warp
// count just above a multiple of the sub-partitions would leave most of them
// waiting for the few that run two warps, so the count is a multiple.
void filter_shape(int nlines, int n, int nk, int warm, int nsm, int kw, long long &seg,
                  unsigned &blocks)
{
    filter_shape_len(nlines, n - 12, nk, warm, nsm, kw, seg, blocks);
}

void filter_shape_len(int nlines, int len2, int nk, int warm, int nsm, int kw, long long &seg,
                      unsigned &blocks)
{
    const long long gtot = (long long)nk * ((nlines + 31) / 32);
    const long long total = gtot * len2;
    const long long S = 4LL * nsm;
    long long nw;
    if (warm < 0) {
        seg = len2;
        nw = gtot;
    } else {
        const int k = (total / (kw * S) >= 8LL * (warm + 6)) ? kw : 1;
        nw = k * S;
        seg = (total + nw - 1) / nw;
        nw = (total + seg - 1) / seg;
    }
    blocks = (unsigned)((nw * 32 + 127) / 128);
}

// ---------------------------------------------------------------------------
// k_bc: ccpml (cc.f90:6-68).  Row t of the left and right columns
// (cc.f90:23-36, corners excepted) and column t of the top and bottom rows
// (cc.f90:39-59); the corner columns recompute the column values they
// extrapolate from at i = 1 and i = imax, so no thread reads a location
// another thread writes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void bc_column_values(const double *__restrict__ U, const Dims &d,
                                                 int i, int j, const double *__restrict__ rhob,
                                                 const double *__restrict__ psib, double gamma,
                                                 double *v)
{
    const long long P = d.plane;
    const long long r = (long long)j * d.pitch;
    if (i == 0) {
        v[0] = rhob[j];
        v[1] = 2.0 * U[1 * P + r + 1] - U[1 * P + r + 2];
        v[2] = 0.0;
        v[3] = 1.0 / gamma;
        if (d.nk >= 5) v[4] = psib[j];
    } else {
        const int a = d.imax - 2, b = d.imax - 3;
        for (int k = 0; k < d.nk; k++) v[k] = 2.0 * U[k * P + r + a] - U[k * P + r + b];
        v[3] = 1.0 / gamma;
    }
}

// blockIdx.y picks the edge: 0 left, 1 right (rows t), 2 top, 3 bottom
// (columns t).  The four write disjoint locations and read only points no
// edge writes, so they run side by side, one memory round trip each.
// Rows r0 .. r1-1 only (the whole grid but in ns_rk_euler's banded last
// stage): the left and right edges of those rows, the top row if r1 = jmax,
// the bottom row if r0 = 0.
__global__ void k_bc(Dims d, double *__restrict__ U, const double *__restrict__ rhob,
                     const double *__restrict__ psib, double gamma, int r0, int r1)
{
    const int edge = blockIdx.y;
    const long long P = d.plane;
    double v[kMaxNk];
    if (edge < 2) {
        const int t = r0 + blockIdx.x * blockDim.x + threadIdx.x;
        if (t > 0 && t < d.jmax - 1 && t < r1) {
            const long long r = (long long)t * d.pitch;
            const int i = edge == 0 ? 0 : d.imax - 1;
            bc_column_values(U, d, i, t, rhob, psib, gamma, v);
            for (int k = 0; k < d.nk; k++) U[k * P + r + i] = v[k];
        }
        return;
    }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool top = edge == 2;
    if (t >= d.imax || (top ? r1 != d.jmax : r0 != 0)) return;
    // top (cc.f90:39-43) from rows jt-1, jt-2; bottom (cc.f90:55-59) from rows 1, 2
    const int jt = d.jmax - 1;
    const int j1 = top ? jt - 1 : 1, j2 = top ? jt - 2 : 2, jw = top ? jt : 0;
    double a[kMaxNk], b[kMaxNk];
    if (t == 0 || t == d.imax - 1) {
        bc_column_values(U, d, t, j1, rhob, psib, gamma, a);
        bc_column_values(U, d, t, j2, rhob, psib, gamma, b);
    } else {
        for (int k = 0; k < d.nk; k++) {
            a[k] = U[k * P + (long long)j1 * d.pitch + t];
            b[k] = U[k * P + (long long)j2 * d.pitch + t];
        }
    }
    const long long w = (long long)jw * d.pitch + t;
    for (int k = 0; k < 3; k++) U[k * P + w] = 2.0 * a[k] - b[k];
    U[3 * P + w] = 1.0 / gamma;
    if (d.nk >= 5) U[4 * P + w] = top ? 1.0 : 0.0;
}

// ---------------------------------------------------------------------------
// Per-step source phase: stage_sin[k] = sin(wf*((iter+c_k)*dt)) for the six
// stages (rk.f90:188), then the device step counter advances.
// ---------------------------------------------------------------------------
struct SinArgs {
    double wf, dt, ct[6];
};

__global__ void k_stage_sin(int *d_iter, double *stage_sin, SinArgs a)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int iter = *d_iter;
    for (int k = 0; k < 6; k++) stage_sin[k] = sin(a.wf * (((double)iter + a.ct[k]) * a.dt));
    *d_iter = iter + 1;
}

__global__ void k_set_iter(int *d_iter, int iter) { *d_iter = iter; }

// ---------------------------------------------------------------------------
// Layout conversion, probes, finite check
// ---------------------------------------------------------------------------
__global__ void k_aos_to_soa(const double *__restrict__ in, double *__restrict__ out, Dims d)
{
    const long long n = (long long)d.nk * d.imax * d.jmax;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e % d.nk);
        const long long pt = e / d.nk;
        const int i = (int)(pt % d.imax);
        const int j = (int)(pt / d.imax);
        out[k * d.plane + (long long)j * d.pitch + i] = in[e];
    }
}

__global__ void k_soa_to_aos(const double *__restrict__ in, double *__restrict__ out, Dims d)
{
    const long long n = (long long)d.nk * d.imax * d.jmax;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e % d.nk);
        const long long pt = e / d.nk;
        const int i = (int)(pt % d.imax);
        const int j = (int)(pt / d.imax);
        out[e] = in[k * d.plane + (long long)j * d.pitch + i];
    }
}

__global__ void k_probes(const double *__restrict__ U, Dims d, int np,
                         const int32_t *__restrict__ idx, double *__restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= np * d.nk) return;
    const int p = t / d.nk, k = t % d.nk;
    const int i = idx[2 * p] - 1, j = idx[2 * p + 1] - 1;
    out[t] = U[k * d.plane + (long long)j * d.pitch + i];
}

__global__ void k_count_nonfinite(const double *__restrict__ U, Dims d,
                                  unsigned long long *count)
{
    unsigned long long local = 0;
    const long long n = (long long)d.nk * d.jmax * d.imax;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % d.imax);
        const long long r = e / d.imax;  // k*jmax + j
        const double v = U[r * d.pitch + i];
        if (!isfinite(v)) local++;
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
static inline dim3 tile_grid(const Dims &d, dim3 blk)
{
    return dim3((d.imax + blk.x - 1) / blk.x, (d.jmax + blk.y - 1) / blk.y);
}

// k_prim or k_first over rows row0 .. row0+rows-1.
template <bool VISC, int NK>
static cudaError_t launch_rows_t(ns_ctx *c, int cls, int row0, int rows, cudaStream_t s)
{
    const Dims &d = c->d;
    const dim3 blk(kFirstBX, kFirstBY);
    const dim3 grd((d.imax + kFirstBX - 1) / kFirstBX, (rows + kFirstBY - 1) / kFirstBY);
    if (cls == NS_KC_PRIM)
        k_prim<<<grd, blk, 0, s>>>(d, c->U, c->aux, c->phys.gamma, row0, rows);
    else if (c->fp64_maps)
        k_first<VISC, NK, true><<<grd, blk, 0, s>>>(c->umap, c->tmap, c->d_err, d, c->U, c->dudm,
                                                    c->dudn, c->aux, c->xcoef, c->ycoef,
                                                    c->trtab, c->phys, row0, rows);
    else
        k_first<VISC, NK, false><<<grd, blk, 0, s>>>(c->umap, c->tmap, c->d_err, d, c->U,
                                                     c->dudm, c->dudn, c->aux, c->xcoef,
                                                     c->ycoef, c->trtab, c->phys, row0, rows);
    return cudaGetLastError();
}

cudaError_t launch_rows(ns_ctx *c, int cls, int row0, int rows, cudaStream_t s)
{
    if (c->split || (cls != NS_KC_PRIM && cls != NS_KC_FIRST)) return cudaErrorInvalidValue;
    if (c->visc)
        return c->d.nk == 5 ? launch_rows_t<true, 5>(c, cls, row0, rows, s)
                            : launch_rows_t<true, 4>(c, cls, row0, rows, s);
    return c->d.nk == 5 ? launch_rows_t<false, 5>(c, cls, row0, rows, s)
                        : launch_rows_t<false, 4>(c, cls, row0, rows, s);
}

// One kernel of class `cls` (NS_KC_*) for `stage`.
int bands_for(const ns_ctx *c, int *pb)
{
    // as many bands (at most kMaxBands) as keep every band's per-warp
    // segments at least four warm-ups long (one warp per SM sub-partition):
    // 8 on 4096 x 2048, 1 on 512 x 512 and smaller grids.  Band b covers
    // pass-2 positions pb[b] .. pb[b+1]-1.
    const Dims &d = c->d;
    const long long total = (long long)d.nk * ((d.imax + 31) / 32) * (d.jmax - 12);
    const long long per_band = 4LL * c->nsm * 4 * (c->warm + 6);
    const int nb =
        c->warm < 0 ? 1 : (int)std::max(1LL, std::min<long long>(kMaxBands, total / per_band));
    const int len2 = d.jmax - 12;
    for (int b = 0; b <= nb; b++) pb[b] = 6 + (int)((long long)b * len2 / nb);
    return nb;
}

void band_rows(const Dims &d, const int *pb, int nb, int b, int &r0, int &r1)
{
    r0 = b == 0 ? 0 : pb[b];
    r1 = b == nb - 1 ? d.jmax : pb[b + 1];
}

cudaError_t launch_filter_y_band(ns_ctx *c, int p0, int p1, cudaStream_t s)
{
    const Dims &d = c->d;
    long long seg;
    unsigned nb;
    filter_shape_len(d.imax, p1 - p0, d.nk, c->warm, c->nsm, kFilterWarpsPerSmsp, seg, nb);
    k_filter<true><<<nb, 128, 0, s>>>(d, c->U2, c->U, seg, c->warm, c->warm32, c->fy, c->d_err, p0, p1 - p0);
    return cudaGetLastError();
}

cudaError_t launch_bc_band(ns_ctx *c, const int *pb, int nb, int b, cudaStream_t s)
{
    const Dims &d = c->d;
    int r0, r1;
    band_rows(d, pb, nb, b, r0, r1);
    const int nt = std::max(r1 - r0, d.imax);
    k_bc<<<dim3((nt + 127) / 128, 4), 128, 0, s>>>(d, c->U, c->rhob, c->psib, c->phys.gamma, r0,
                                                   r1);
    return cudaGetLastError();
}

template <bool VISC, int NK>
static cudaError_t launch_kernel_t(ns_ctx *c, int cls, int stage, cudaStream_t s)
{
    const Dims &d = c->d;
    const dim3 blk(32, 8);
    const dim3 grd = tile_grid(d, blk);
    switch (cls) {
    case NS_KC_PRIM:
    case NS_KC_FIRST:
        return launch_rows_t<VISC, NK>(c, cls, 0, d.jmax, s);
    case NS_KC_UPDATE: {
        StageCoef sc{c->alpha[stage], c->beta[stage], stage};
        const bool src = c->src != nullptr;
        constexpr bool has_tile = kAuxTilePlanes<VISC, NK> > 0;
        const bool tma = has_tile && c->fp64_maps;
#define NS_UPD(FIRST, SRC, TMA)                                                                \
    k_update<VISC, NK, FIRST, SRC, TMA><<<grd, blk, 0, s>>>(                                   \
        c->amap, c->d_err, d, c->U, c->W, c->dudm, c->dudn, c->aux, c->xcoef, c->ycoef,        \
        c->Ubase, c->sigx, c->sigy, c->src, c->stage_sin, c->phys, sc)
#define NS_UPD2(FIRST, SRC)                             \
    do {                                                \
        if constexpr (has_tile) {                       \
            if (tma) NS_UPD(FIRST, SRC, has_tile);      \
            else NS_UPD(FIRST, SRC, false);             \
        } else {                                        \
            NS_UPD(FIRST, SRC, false);                  \
        }                                               \
    } while (0)
        if (stage == 0) {
            if (src) NS_UPD2(true, true); else NS_UPD2(true, false);
        } else {
            if (src) NS_UPD2(false, true); else NS_UPD2(false, false);
        }
#undef NS_UPD2
#undef NS_UPD
        break;
    }
    case NS_KC_FILTER_X: {
        long long seg;
        unsigned nb;
        filter_shape(d.jmax, d.imax, d.nk, c->warm, c->nsm, kFilterWarpsPerSmsp, seg, nb);
        k_filter<false><<<nb, 128, 0, s>>>(d, c->U, c->U2, seg, c->warm, c->warm32, c->fx, c->d_err, 6,
                                            d.imax - 12);
        break;
    }
    case NS_KC_FILTER_Y: {
        long long seg;
        unsigned nb;
        filter_shape(d.imax, d.jmax, d.nk, c->warm, c->nsm, kFilterWarpsPerSmsp, seg, nb);
        k_filter<true><<<nb, 128, 0, s>>>(d, c->U2, c->U, seg, c->warm, c->warm32, c->fy, c->d_err, 6,
                                           d.jmax - 12);
        break;
    }
    case NS_KC_BC: {
        const int nt = d.imax > d.jmax ? d.imax : d.jmax;
        k_bc<<<dim3((nt + 127) / 128, 4), 128, 0, s>>>(d, c->U, c->rhob, c->psib, c->phys.gamma,
                                                       0, d.jmax);
        break;
    }
    case NS_KC_STAGE_SIN: {
        SinArgs a;
        a.wf = c->p.wf;
        a.dt = c->p.dt;
        for (int k = 0; k < 6; k++) a.ct[k] = c->ct[k];
        k_stage_sin<<<1, 32, 0, s>>>(c->d_iter, c->stage_sin, a);
        break;
    }
    default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_kernel(ns_ctx *c, int cls, int stage, cudaStream_t s)
{
    if (cls >= NS_KC_SPLIT_STAGE) return launch_split_kernel(c, cls, stage, s);
    if (c->visc)
        return c->d.nk == 5 ? launch_kernel_t<true, 5>(c, cls, stage, s)
                            : launch_kernel_t<true, 4>(c, cls, stage, s);
    return c->d.nk == 5 ? launch_kernel_t<false, 5>(c, cls, stage, s)
                        : launch_kernel_t<false, 4>(c, cls, stage, s);
}

// The launch sequence of one step (rk.f90:52-73): the source phase, then per
// stage [prim], first, update, filter x, filter y, bc.
int step_sequence(const ns_ctx *c, int *cls, int *stage)
{
    int n = 0;
    if (c->src || c->sp.src) { cls[n] = NS_KC_STAGE_SIN; stage[n++] = 0; }
    if (c->split) {
        for (int st = 0; st < 6; st++) {
            if (c->visc) { cls[n] = NS_KC_SPLIT_VISC; stage[n++] = st; }
            cls[n] = NS_KC_SPLIT_STAGE; stage[n++] = st;
            cls[n] = NS_KC_SPLIT_FX; stage[n++] = st;
            cls[n] = NS_KC_SPLIT_FY; stage[n++] = st;
            cls[n] = NS_KC_SPLIT_BC; stage[n++] = st;
        }
        return n;
    }
    for (int st = 0; st < 6; st++) {
        if (c->visc) { cls[n] = NS_KC_PRIM; stage[n++] = st; }
        cls[n] = NS_KC_FIRST; stage[n++] = st;
        cls[n] = NS_KC_UPDATE; stage[n++] = st;
        cls[n] = NS_KC_FILTER_X; stage[n++] = st;
        cls[n] = NS_KC_FILTER_Y; stage[n++] = st;
        cls[n] = NS_KC_BC; stage[n++] = st;
    }
    return n;
}

// The step without stage 0's k_prim and k_first (the source phase kept):
// the rest of the step once those have run over all rows.
cudaError_t launch_step_tail(ns_ctx *c, cudaStream_t s)
{
    int cls[kMaxStepLaunches], stage[kMaxStepLaunches];
    const int n = step_sequence(c, cls, stage);
    for (int q = 0; q < n; q++) {
        if (stage[q] == 0 && (cls[q] == NS_KC_PRIM || cls[q] == NS_KC_FIRST)) continue;
        if (stage[q] == 5 && (cls[q] == NS_KC_FILTER_Y || cls[q] == NS_KC_BC)) continue;
        cudaError_t e = launch_kernel(c, cls[q], stage[q], s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_step(ns_ctx *c, cudaStream_t s)
{
    int cls[kMaxStepLaunches], stage[kMaxStepLaunches];
    const int n = step_sequence(c, cls, stage);
    for (int q = 0; q < n; q++) {
        cudaError_t e = launch_kernel(c, cls[q], stage[q], s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

int count_step_launches(const ns_ctx *c)
{
    int cls[kMaxStepLaunches], stage[kMaxStepLaunches];
    return step_sequence(c, cls, stage);
}

cudaError_t launch_set_iter(int *d_iter, int iter, cudaStream_t s)
{
    k_set_iter<<<1, 1, 0, s>>>(d_iter, iter);
    return cudaGetLastError();
}

static inline unsigned grid_for(long long n)
{
    long long b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    if (b < 1) b = 1;
    return (unsigned)b;
}

cudaError_t launch_aos_to_soa(const double *in, double *out, const Dims &d, cudaStream_t s)
{
    k_aos_to_soa<<<grid_for((long long)d.nk * d.imax * d.jmax), 256, 0, s>>>(in, out, d);
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(const double *in, double *out, const Dims &d, cudaStream_t s)
{
    k_soa_to_aos<<<grid_for((long long)d.nk * d.imax * d.jmax), 256, 0, s>>>(in, out, d);
    return cudaGetLastError();
}

cudaError_t launch_probes(const double *U, const Dims &d, int np, const int32_t *idx,
                          double *out, cudaStream_t s)
{
    const int n = np * d.nk;
    k_probes<<<(n + 127) / 128, 128, 0, s>>>(U, d, np, idx, out);
    return cudaGetLastError();
}

cudaError_t launch_count_nonfinite(const double *U, const Dims &d, unsigned long long *count,
                                   cudaStream_t s)
{
    k_count_nonfinite<<<grid_for((long long)d.nk * d.imax * d.jmax), 256, 0, s>>>(U, d, count);
    return cudaGetLastError();
}

}  // namespace ns
