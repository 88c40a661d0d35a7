// ns_adjoint.cu -- discrete adjoint of the FP64 Euler step (rk.f90:12-75,
// 1/Re = 0, nk = 4) for the gradient of an observer loss with respect to
// the source field.
//
// Forward: U_{n+1} = Phi(U_n; S), n = 0..N-1, with the source of
// rk.f90:188-189 written as s = sin(wf*(iter+c_k)*dt) * S(i,j).  Loss
// L = sum_n sum_m p'(x_m, t_{n+1})^2 with p' = p - p_b interpolated
// bilinearly at observer m.  The reverse pass applies, per step and stage in
// reverse order, the transposes of ccpml (cc.f90:6-68), lddfiltery and
// lddfilterx (filtering.f90, in reverse sweep order), bufferxy
// (rk.f90:77-151), rk_steep (rk.f90:153-169), EULERNONLINEAR's pointwise
// Jacobians (eqeuler.f90:63-92) and the DRP derivatives with their closures
// and metrics (diff.f90:6-350).  The forward state is checkpointed every K
// steps; each K-step segment is recomputed once, keeping every stage's input
// state and derivatives, so the reverse pass recomputes nothing.  The
// recompute of segment s-1 runs on a second stream beside the reverse of
// segment s (two segment stores): on grids of a few hundred thousand points
// one kernel leaves much of the GPU idle, and the two chains are
// independent.  The forward keeps the stage inputs of the last two segments
// in those stores itself (the last one only, without a second store).
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "ns_check.cuh"
#include "ns_coef.h"
#include "ns_internal.cuh"
#include "ns_tma.cuh"

namespace ns {
namespace adj {

// ---------------------------------------------------------------------------
// Observers: p' at (x, y) by bilinear interpolation of the four grid points
// around it; loss and its gradient.
// ---------------------------------------------------------------------------
struct Obs {
    int i0, j0;     // lower-left grid point (0-based)
    double wx, wy;  // fractional position in the cell
};

__device__ __forceinline__ double obs_p(const double *U, const Dims &d, const Obs &o, double pb)
{
    const double *p = U + 3 * d.plane;
    const long long r0 = (long long)o.j0 * d.pitch + o.i0, r1 = r0 + d.pitch;
    return (1 - o.wx) * (1 - o.wy) * (p[r0] - pb) + o.wx * (1 - o.wy) * (p[r0 + 1] - pb) +
           (1 - o.wx) * o.wy * (p[r1] - pb) + o.wx * o.wy * (p[r1 + 1] - pb);
}

__global__ void k_obs_loss(const double *U, Dims d, const Obs *obs, int nobs, double pb,
                           double *loss)
{
    double acc = 0.0;
    for (int m = threadIdx.x; m < nobs; m += 32) {
        const double v = obs_p(U, d, obs[m], pb);
        acc += v * v;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) *loss += acc;
}

// Copies the 4 state planes (n4 = 4*plane contiguous doubles) to slot
// (*d_step)*6 + stage of the per-stage store; the step index is read on the
// device, so one captured graph serves every step.
__global__ void k_store_stage(const double *__restrict__ U, double *__restrict__ store,
                              const int *__restrict__ d_step, int stage, long long n4)
{
    const long long off = ((long long)(*d_step) * 6 + stage) * n4;
    const double2 *src = reinterpret_cast<const double2 *>(U);
    double2 *dst = reinterpret_cast<double2 *>(store + off);
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n4 / 2;
         e += (long long)gridDim.x * blockDim.x)
        dst[e] = src[e];
}

__global__ void k_step_inc(int *d_step) { *d_step += 1; }

// lam_p += dL/dp of sum_m p'_m^2 at U
__global__ void k_obs_grad(const double *U, Dims d, const Obs *obs, int nobs, double pb,
                           double *lam)
{
    const int m = threadIdx.x + blockIdx.x * blockDim.x;
    if (m >= nobs) return;
    const Obs o = obs[m];
    const double g = 2.0 * obs_p(U, d, o, pb);
    double *lp = lam + 3 * d.plane;
    const long long r0 = (long long)o.j0 * d.pitch + o.i0, r1 = r0 + d.pitch;
    atomicAdd(lp + r0, g * (1 - o.wx) * (1 - o.wy));
    atomicAdd(lp + r0 + 1, g * o.wx * (1 - o.wy));
    atomicAdd(lp + r1, g * (1 - o.wx) * o.wy);
    atomicAdd(lp + r1 + 1, g * o.wx * o.wy);
}

// ---------------------------------------------------------------------------
// ccpml transpose.  Forward order: left, right (all rows), top, bottom (all
// columns); transpose: bottom^T, top^T (columns), then right^T, left^T
// (rows).  An edge value set from 2*q(1) - q(2) sends 2x and -1x of its
// adjoint inward and is zeroed; a value set to a constant is zeroed.
// ---------------------------------------------------------------------------
// Column part (bottom^T, top^T) of column i and row part (right^T, left^T)
// of row j for variable k.
__device__ __forceinline__ void bct_col(double *lam, const Dims &d, int k, int i)
{
    const long long p = d.pitch;
    const int jt = d.jmax - 1;
    double *l = lam + k * d.plane + i;
    // bottom^T (cc.f90:55-59)
    const double b = l[0];
    if (k < 3) {
        l[p] += 2.0 * b;
        l[2 * p] -= b;
    }
    l[0] = 0.0;
    // top^T (cc.f90:39-43)
    const double t = l[(long long)jt * p];
    if (k < 3) {
        l[(long long)(jt - 1) * p] += 2.0 * t;
        l[(long long)(jt - 2) * p] -= t;
    }
    l[(long long)jt * p] = 0.0;
}

__device__ __forceinline__ void bct_row(double *lam, const Dims &d, int k, int j)
{
    const int ir = d.imax - 1;
    double *l = lam + k * d.plane + (long long)j * d.pitch;
    // right^T (cc.f90:32-36)
    const double r = l[ir];
    if (k < 3) {
        l[ir - 1] += 2.0 * r;
        l[ir - 2] -= r;
    }
    l[ir] = 0.0;
    // left^T (cc.f90:23-27): only u is extrapolated
    const double a = l[0];
    if (k == 1) {
        l[1] += 2.0 * a;
        l[2] -= a;
    }
    l[0] = 0.0;
}

// The column parts must precede the row parts only where both touch a
// point: the three columns and rows next to each corner.  Block 0 does the
// six corner columns, then (after a block barrier) the six corner rows;
// the other blocks take every other column and row, which touch disjoint
// points, all at once.  Each (line, variable) pair is one thread.
__global__ void __launch_bounds__(256) k_bct(double *lam, Dims d)
{
    const int ir = d.imax - 1, jt = d.jmax - 1;
    if (blockIdx.x == 0) {
        const int t = threadIdx.x;
        if (t < 24) {
            const int k = t / 6, c = t % 6;
            bct_col(lam, d, k, c < 3 ? c : ir - (c - 3));
        }
        __syncthreads();
        if (t < 24) {
            const int k = t / 6, c = t % 6;
            bct_row(lam, d, k, c < 3 ? c : jt - (c - 3));
        }
        return;
    }
    const int ncol = d.imax - 6, nrow = d.jmax - 6;
    const long long total = 4LL * (ncol + nrow);
    for (long long e = (long long)(blockIdx.x - 1) * blockDim.x + threadIdx.x; e < total;
         e += (long long)(gridDim.x - 1) * blockDim.x) {
        if (e < 4LL * ncol) bct_col(lam, d, (int)(e / ncol), 3 + (int)(e % ncol));
        else {
            const long long r = e - 4LL * ncol;
            bct_row(lam, d, (int)(r / nrow), 3 + (int)(r % nrow));
        }
    }
}

// ---------------------------------------------------------------------------
// Filter transpose.  The forward sweep is a product of elementary updates
// E_q (row q replaced by a combination of its neighbours); its transpose
// applies E_q^T in reverse order: pass 3 ascending q = n-7..n-2, pass 2
// descending q = n-7..6, pass 1 descending q = 6..1.  E_q^T adds c_s*lam_q
// to lam_{q+s} and scales lam_q by c_0.  In the descending pass 2 a window
// of 13 values slides down the line; after step q the value at q+6 is
// final.  Chunks start `warm` steps above their range from the untouched
// adjoint; the missing contributions decay as in the forward recurrence.
// ---------------------------------------------------------------------------
// E_q^T of one pass-2 point q = w[6]: w[0..12] hold the adjoint at q-6..q+6.
__device__ __forceinline__ void transpose13(const FilterCoef &fc, double *w)
{
    const double lq = w[6];
    w[0] = fma(fc.m[6], lq, w[0]);
    w[1] = fma(fc.m[5], lq, w[1]);
    w[2] = fma(fc.m[4], lq, w[2]);
    w[3] = fma(fc.m[3], lq, w[3]);
    w[4] = fma(fc.m[2], lq, w[4]);
    w[5] = fma(fc.m[1], lq, w[5]);
    w[7] = fma(fc.m[1], lq, w[7]);
    w[8] = fma(fc.m[2], lq, w[8]);
    w[9] = fma(fc.m[3], lq, w[9]);
    w[10] = fma(fc.m[4], lq, w[10]);
    w[11] = fma(fc.m[5], lq, w[11]);
    w[12] = fma(fc.m[6], lq, w[12]);
    w[6] = fc.c0 * lq;
}

// The same in FP32 (the first steps of a warm start); cf = c0, m[1..6].
__device__ __forceinline__ void transpose13_f(const float *cf, float *w)
{
    const float lq = w[6];
#pragma unroll
    for (int s = 1; s <= 6; s++) {
        w[6 - s] = fmaf(cf[s], lq, w[6 - s]);
        w[6 + s] = fmaf(cf[s], lq, w[6 + s]);
    }
    w[6] = cf[0] * lq;
}

// Slides the window one point down; `next` is the untouched adjoint at q-7.
__device__ __forceinline__ void shift13_down(double *w, double next)
{
#pragma unroll
    for (int t = 12; t > 0; t--) w[t] = w[t - 1];
    w[0] = next;
}

// Pass-2 positions [a, b) of one line, transposed: b == n-6 starts exactly
// with pass 3^T at the top, a later end runs `warm` points of history
// first, the first warm32 of them in FP32 (or starts exactly when that
// reaches the top); a == 6 ends with pass 1^T.  Writes positions
// a+6 .. b+5 (and 0..11 when a == 6, the top when b == n-6).
__device__ __forceinline__ void filter_piece_t(const double *__restrict__ s, double *__restrict__ o,
                                               long long st, int n, int a, int b, int warm,
                                               int warm32, const FilterCoef &fc)
{
    double w[13];
    int q;
    const int qtop = n - 7;
    if (b == n - 6 || warm < 0 || b - 1 + warm >= qtop) {
        // exact start at the top: pass 3^T on positions n-12..n-1
        double L[12];
#pragma unroll
        for (int x = 0; x < 12; x++) L[x] = s[(long long)(n - 12 + x) * st];
#pragma unroll
        for (int x = 5; x <= 10; x++) {
            const double lq = L[x];
            L[x + 1] = fma(fc.bm1, lq, L[x + 1]);
#pragma unroll
            for (int z = 1; z <= 5; z++) L[x - z] = fma(fc.b[z], lq, L[x - z]);
            L[x] = fc.b0 * lq;
        }
#pragma unroll
        for (int x = 0; x < 12; x++) w[x + 1] = L[x];
        w[0] = s[(long long)(n - 13) * st];
        q = qtop;
    } else {
        q = b - 1 + warm;
        // the untouched history's error decays below the FP32 rounding in the
        // first warm32 steps, which therefore run in FP32 (no outputs there)
        float wf[13], cf[7];
        cf[0] = (float)fc.c0;
#pragma unroll
        for (int z = 1; z < 7; z++) cf[z] = (float)fc.m[z];
#pragma unroll
        for (int t = 0; t < 13; t++) wf[t] = (float)s[(long long)(q - 6 + t) * st];
        for (const int qe = q - warm32; q > qe; q--) {
            transpose13_f(cf, wf);
#pragma unroll
            for (int t = 12; t > 0; t--) wf[t] = wf[t - 1];
            wf[0] = (float)s[(long long)(q - 7) * st];
        }
#pragma unroll
        for (int t = 0; t < 13; t++) w[t] = (double)wf[t];
    }
    // blocks of kFilterPf points, the next block's input loaded ahead
    double nx[kFilterPf];
#pragma unroll
    for (int t = 0; t < kFilterPf; t++) {
        const int r = q - 7 - t;
        nx[t] = (r >= 0) ? s[(long long)r * st] : 0.0;
    }
    for (; q - kFilterPf + 1 >= a; q -= kFilterPf) {
        double cur[kFilterPf];
#pragma unroll
        for (int t = 0; t < kFilterPf; t++) {
            cur[t] = nx[t];
            const int r = q - kFilterPf - 7 - t;
            nx[t] = (r >= 0) ? s[(long long)r * st] : 0.0;
        }
#pragma unroll
        for (int t = 0; t < kFilterPf; t++) {
            transpose13(fc, w);
            if (q - t < b) o[(long long)(q - t + 6) * st] = w[12];
            shift13_down(w, cur[t]);
        }
    }
    for (; q >= a; q--) {
        transpose13(fc, w);
        if (q < b) o[(long long)(q + 6) * st] = w[12];
        shift13_down(w, (q - 7 >= 0) ? s[(long long)(q - 7) * st] : 0.0);
    }
    if (a == 6) {
        // window now holds positions -1..11 in w[0..12]: pass 1^T, q = 6..1
#pragma unroll
        for (int qq = 6; qq >= 1; qq--) {
            const double lq = w[qq + 1];
            w[qq] = fma(fc.bm1, lq, w[qq]);
#pragma unroll
            for (int z = 1; z <= 5; z++) w[qq + 1 + z] = fma(fc.b[z], lq, w[qq + 1 + z]);
            w[qq + 1] = fc.b0 * lq;
        }
#pragma unroll
        for (int p = 0; p < 12; p++) o[(long long)p * st] = w[p + 1];
    }
}

// The transposed sweep dealt out like the forward one (k_filter): warp-lines
// of 32 adjacent lines, their pass-2 positions laid end to end and cut into
// equal segments, one per warp.
template <bool ALONG_Y>
__global__ void __launch_bounds__(128)
    k_filter_t(Dims d, const double *__restrict__ in, double *__restrict__ out, long long seg,
               int warm, int warm32, FilterCoef fc)
{
    const int lane = threadIdx.x & 31;
    const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nlines = ALONG_Y ? d.imax : d.jmax;
    const int gpk = (nlines + 31) >> 5;
    const int n = ALONG_Y ? d.jmax : d.imax;
    const int len2 = n - 12;
    const long long total = (long long)gpk * 4 * len2;
    const long long s0 = wid * seg;
    const long long s1 = s0 + seg < total ? s0 + seg : total;
    const long long st = ALONG_Y ? d.pitch : 1;
    for (long long sp = s0; sp < s1;) {
        const long long g = sp / len2;
        const long long gend = (g + 1) * len2;
        const long long e = s1 < gend ? s1 : gend;
        const int k = (int)(g / gpk);
        const int line = (int)(g % gpk) * 32 + lane;
        if (line < nlines) {
            const long long base =
                (long long)k * d.plane + (ALONG_Y ? line : (long long)line * d.pitch);
            filter_piece_t(in + base, out + base, st, n, 6 + (int)(sp - g * len2),
                           6 + (int)(e - g * len2), warm, warm32, fc);
        }
        sp = e;
    }
}

// ---------------------------------------------------------------------------
// Pointwise part of a stage transpose: bufferxy^T, rk_steep^T and the
// Jacobians of EULERNONLINEAR (eqeuler.f90:63-92, 1/Re = 0) at the stored
// stage input U with its derivatives (ux = dU/dx, uy = dU/dy).
//   in:  lam = dL/dU after the stage's buffer, om = dL/dw' (from later stages)
//   out: lam = pointwise part of dL/dU(stage input), om = dL/dw(stage input),
//        lx, ly = dL/d(dU/dx), dL/d(dU/dy); gS += sin_k * dL/d(dp/dt)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
    k_point_t(Dims d, double *__restrict__ lam, double *__restrict__ om,
              double *__restrict__ lx, double *__restrict__ ly, const double *__restrict__ U,
              const double *__restrict__ ux, const double *__restrict__ uy,
              const double *__restrict__ sigx, const double *__restrict__ sigy,
              double *__restrict__ gS, double gamma, double dt, double alpha, double beta,
              double sink)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= d.imax || j >= d.jmax) return;
    const long long idx = (long long)j * d.pitch + i, P = d.plane;
    double l[4];
#pragma unroll
    for (int k = 0; k < 4; k++) l[k] = lam[k * P + idx];
    // bufferxy^T: U'' = Ub + s*(U' - Ub), y then x
    if (i < d.D || i >= d.imax - d.D) {
        const double s = sigx[i];
#pragma unroll
        for (int k = 0; k < 4; k++) l[k] *= s;
    }
    if (j < d.D || j >= d.jmax - d.D) {
        const double s = sigy[j];
#pragma unroll
        for (int k = 0; k < 4; k++) l[k] *= s;
    }
    const bool interior = (i > 0) && (i < d.imax - 1) && (j > 0) && (j < d.jmax - 1);
    double gx[4] = {0, 0, 0, 0}, gy[4] = {0, 0, 0, 0};
    if (interior) {
        // rk_steep^T: U1 = U + beta*w', w' = alpha*w + dt*R
        double aR[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const double wt = fma(beta, l[k], om[k * P + idx]);
            aR[k] = dt * wt;
            om[k * P + idx] = alpha * wt;
        }
        gS[idx] = fma(sink, aR[3], gS[idx]);
        const double rho = U[idx], uu = U[P + idx], vv = U[2 * P + idx], pp = U[3 * P + idx];
        double dx[4], dy[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            dx[k] = ux[k * P + idx];
            dy[k] = uy[k * P + idx];
        }
        const double ri = 1.0 / rho, ri2 = ri * ri;
        const double div = dx[1] + dy[2];
        const double a0 = aR[0], a1 = aR[1], a2 = aR[2], a3 = aR[3];
        // f_rho = -(u rho_x + rho u_x + v rho_y + rho v_y)
        // f_u   = -(u u_x + p_x/rho + v u_y)
        // f_v   = -(u v_x + v v_y + p_y/rho)
        // f_p   = -(gamma p u_x + u p_x + gamma p v_y + v p_y - s)
        l[0] += -a0 * div + (a1 * dx[3] + a2 * dy[3]) * ri2;
        l[1] += -(a0 * dx[0] + a1 * dx[1] + a2 * dx[2] + a3 * dx[3]);
        l[2] += -(a0 * dy[0] + a1 * dy[1] + a2 * dy[2] + a3 * dy[3]);
        l[3] += -a3 * gamma * div;
        gx[0] = -uu * a0;
        gy[0] = -vv * a0;
        gx[1] = -rho * a0 - uu * a1 - gamma * pp * a3;
        gy[1] = -vv * a1;
        gx[2] = -uu * a2;
        gy[2] = -rho * a0 - vv * a2 - gamma * pp * a3;
        gx[3] = -ri * a1 - uu * a3;
        gy[3] = -ri * a2 - vv * a3;
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++) om[k * P + idx] = 0.0;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        lam[k * P + idx] = l[k];
        lx[k * P + idx] = gx[k];
        ly[k * P + idx] = gy[k];
    }
}

// Coefficient of f[q] in the derivative at row r of a line of length n
// (the per-position tables of ns_api.cu: interior rows hold c_s in entries
// 4..6 for sum_s c_s*(f[r+s]-f[r-s]); closure rows hold 7 coefficients for
// offsets o0..o0+6).
__device__ __forceinline__ double dcoef(const double *tab, int r, int q, int n)
{
    const double *c = tab + kCoefStride * r;
    if (r >= 3 && r < n - 3) {
        const int s = q - r;
        if (s >= 1 && s <= 3) return c[3 + s];
        if (s <= -1 && s >= -3) return -c[3 - s];
        return 0.0;
    }
    const int o0 = (r < 3) ? -r : (n - 7 - r);
    const int z = q - r - o0;
    return (z >= 0 && z < 7) ? c[z] : 0.0;
}

// sum_r D[r][q] * g[r] at a point q in [9, n-9), whose neighbours within 6
// are interior rows (no closure row reaches it): g in global or shared memory
__device__ __forceinline__ double dtrans_int(const double *g, long long st, int q,
                                             const double *__restrict__ tab)
{
    double r = 0.0;
#pragma unroll
    for (int s = 1; s <= 3; s++) {
        r = fma(tab[kCoefStride * (q - s) + 3 + s], g[-s * st], r);
        r = fma(-tab[kCoefStride * (q + s) + 3 + s], g[s * st], r);
    }
    return r;
}

// sum_r D[r][q] * g[r] along one line
__device__ __forceinline__ double dtrans(const double *__restrict__ g, long long st, int q, int n,
                                         const double *__restrict__ tab)
{
    if (q >= 9 && q < n - 9) return dtrans_int(g, st, q, tab);
    double r = 0.0;
    for (int rr = max(0, q - 6); rr <= min(n - 1, q + 6); rr++)
        r = fma(dcoef(tab, rr, q, n), g[(long long)(rr - q) * st], r);
    return r;
}

// Block and tiles of k_deriv_t: 32 x 4 points; lx with its x halo (box
// 40 x 4 x 4 from (i0-4, j0): the x coordinate times 8 bytes stays a
// multiple of 16) and ly with its y halo (box 32 x 10 x 4 from (i0, j0-3)).
// Small blocks (as k_point_t's) leave room beside them for the kernels of
// the recompute stream: 32 x 8 blocks made the reverse pass 2 % slower.
constexpr int kDtBX = 32, kDtBY = 4, kDtXW = 40, kDtXL = 4, kDtYH = kDtBY + 6;

// lam += Dx^T lx + Dy^T ly.  With TMA both tiles arrive in shared memory by
// one bulk copy each and the interior gathers read them there; points within
// 9 of an edge (closure rows reach them) read global memory.  Both give
// identical bits.
template <bool TMA>
__global__ void __launch_bounds__(256)
    k_deriv_t(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap ymap,
              int *__restrict__ err, Dims d, double *__restrict__ lam,
              const double *__restrict__ lx, const double *__restrict__ ly,
              const double *__restrict__ xcoef, const double *__restrict__ ycoef)
{
    __shared__ alignas(128) double sx[TMA ? 4 : 1][TMA ? kDtBY : 1][TMA ? kDtXW : 1];
    __shared__ alignas(128) double sy[TMA ? 4 : 1][TMA ? kDtYH : 1][TMA ? kDtBX : 1];
    __shared__ alignas(8) unsigned long long tbar;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i = blockIdx.x * kDtBX + tx;
    const int j = blockIdx.y * kDtBY + ty;
    NS_CHECK(err, kChkAdjoint, blockDim.x == kDtBX && blockDim.y == kDtBY);
    if constexpr (TMA) {
        const bool lead = (tx == 0 && ty == 0);
        if (lead) mbar_init(&tbar, 1);
        __syncthreads();
        if (lead) {
            const int i0 = blockIdx.x * kDtBX, j0 = blockIdx.y * kDtBY;
            mbar_expect_tx(&tbar, (unsigned)(sizeof(sx) + sizeof(sy)));
            tma_load_3d(&sx[0][0][0], &xmap, i0 - kDtXL, j0, 0, &tbar);
            tma_load_3d(&sy[0][0][0], &ymap, i0, j0 - 3, 0, &tbar);
        }
        if (!mbar_wait_bounded(&tbar, 0, err)) return;
    }
    if (i >= d.imax || j >= d.jmax) return;
    const long long idx = (long long)j * d.pitch + i, P = d.plane;
    const bool xin = TMA && i >= 9 && i < d.imax - 9;
    const bool yin = TMA && j >= 9 && j < d.jmax - 9;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double vx = xin ? dtrans_int(&sx[TMA ? k : 0][TMA ? ty : 0][TMA ? tx + kDtXL : 0], 1,
                                           i, xcoef)
                              : dtrans(lx + k * P + idx, 1, i, d.imax, xcoef);
        const double vy = yin ? dtrans_int(&sy[TMA ? k : 0][TMA ? ty + 3 : 0][TMA ? tx : 0], kDtBX,
                                           j, ycoef)
                              : dtrans(ly + k * P + idx, d.pitch, j, d.jmax, ycoef);
        lam[k * P + idx] += vx + vy;
    }
}

}  // namespace adj
}  // namespace ns

// ===========================================================================
// Host side
// ===========================================================================
struct ns_adjoint {
    ns_ctx *fwd = nullptr;
    int nobs = 0, K = 100, nsteps = 0, iter0 = 0;
    double pb = 0.0;
    ns::adj::Obs *obs = nullptr;
    double *loss = nullptr;
    double *chk = nullptr;     // checkpoints: nchk x 4 planes
    int nchk = 0;
    // segment stores: K steps x 6 stages x 12 planes (U, dU/dx, dU/dy), then
    // 4 planes for the state after the segment's last step; segment sg uses
    // store2 when sg is odd and store2 exists (recompute beside reverse)
    double *store = nullptr, *store2 = nullptr;
    // segments at the end of the run whose stages the forward kept in their
    // stores (0, 1, or 2 when the second store exists)
    int stored_segs = 0;
    cudaStream_t s_rec = nullptr, s_rev = nullptr;
    cudaEvent_t ev_rec[2] = {}, ev_rev[2] = {}, ev_start = nullptr;
    // K = 0: every stage's input of every step kept (nsteps x 6 x 4 planes)
    // when device memory allows; the reverse pass then recomputes only the
    // first derivatives of each stage instead of the whole forward
    double *stages = nullptr;
    int stages_cap = 0;        // steps the stage store holds
    int *d_step = nullptr;
    cudaGraphExec_t fwd_exec = nullptr;  // one step with stage stores and the loss
    bool stored_all = false;   // the last forward kept every stage input
    int store_steps = 0;       // steps the segment store holds (0: one stage's scratch)
    double *endstate = nullptr;
    double *lam = nullptr, *lam2 = nullptr, *om = nullptr, *lx = nullptr, *ly = nullptr;
    double *gS = nullptr;
    double *dudm0 = nullptr, *dudn0 = nullptr;  // the context's own derivative planes
    CUtensorMap lxmap{}, lymap{};  // k_deriv_t's tiles of lx and ly
    bool dt_maps = false;
    int warm_t = -1, warm32_t = 0;  // warm-ups of the transposed filter sweeps
    double sin_host[6];
    bool forward_done = false;
    std::string err;
};

namespace {

// checkpoint interval when every-stage storage was asked for but does not fit
constexpr int kDefaultCheckpoint = 100;

int aerr(ns_adjoint *a, int code, const std::string &m)
{
    if (a) a->err = m;
    ns::record_error(m.c_str());
    return code;
}

#define A_CUDA(a, call)                                                                      \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return aerr((a), NS_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

// Planes of one step in a segment store (6 stages x U, dU/dx, dU/dy).
constexpr size_t kStepPlanes = 6 * 12;

double *seg_store(const ns_adjoint *a, int sg)
{
    return (a->store2 && (sg & 1)) ? a->store2 : a->store;
}

double *seg_slot(double *store, int q, size_t P) { return store + (size_t)q * kStepPlanes * P; }

// (Re)allocates the segment stores for K steps: the first is required, the
// second only lets the recompute run beside the reverse pass.
int ensure_segment_stores(ns_adjoint *a, int K)
{
    const size_t P = (size_t)a->fwd->d.plane;
    const size_t bytes = ((size_t)K * kStepPlanes + 4) * P * sizeof(double);
    if (a->store_steps < K) {
        if (a->store) cudaFree(a->store);
        if (a->store2) cudaFree(a->store2);
        a->store = a->store2 = nullptr;
        a->store_steps = 0;
        A_CUDA(a, cudaMalloc(&a->store, bytes));
        a->store_steps = K;
    }
    if (!a->store2) {
        size_t freeb = 0, total = 0;
        const bool room = cudaMemGetInfo(&freeb, &total) == cudaSuccess && bytes <= freeb / 4 * 3;
        if (!room || cudaMalloc(&a->store2, bytes) != cudaSuccess) {
            cudaGetLastError();
            a->store2 = nullptr;
        }
    }
    return NS_OK;
}

// sin(wf*((iter+c_k)*dt)) of rk.f90:188 for the six stages of step `iter`
void stage_sines(const ns_ctx *c, int iter, double *out)
{
    for (int k = 0; k < 6; k++) out[k] = std::sin(c->p.wf * (((double)iter + c->ct[k]) * c->p.dt));
}

// One forward step stage by stage; when `slot` is non-null, each stage's
// input U and its derivatives are kept there (12 planes per stage).
int forward_step(ns_adjoint *a, int iter, double *slot, cudaStream_t s)
{
    ns_ctx *c = a->fwd;
    const size_t P = (size_t)c->d.plane;
    int cls[ns::kMaxStepLaunches], stg[ns::kMaxStepLaunches];
    const int n = ns::step_sequence(c, cls, stg);
    A_CUDA(a, ns::launch_set_iter(c->d_iter, iter, s));
    for (int q = 0; q < n; q++) {
        if (slot && cls[q] == NS_KC_FIRST) {
            double *base = slot + (size_t)stg[q] * 12 * P;
            A_CUDA(a, cudaMemcpyAsync(base, c->U, 4 * P * sizeof(double), cudaMemcpyDeviceToDevice, s));
            c->dudm = base + 4 * P;
            c->dudn = base + 8 * P;
        }
        A_CUDA(a, ns::launch_kernel(c, cls[q], stg[q], s));
        if (slot && cls[q] == NS_KC_UPDATE) {
            c->dudm = a->dudm0;
            c->dudn = a->dudn0;
        }
    }
    return NS_OK;
}

// The reverse of one stage: U, Um, Un are the stage's input state and its
// first derivatives (4 planes each).
int stage_adjoint(ns_adjoint *a, const double *U, const double *Um, const double *Un, int stage,
                  double sink, cudaStream_t s)
{
    ns_ctx *c = a->fwd;
    const ns::Dims &d = c->d;
    {
        const long long items = 4LL * (d.imax + d.jmax - 12);
        ns::adj::k_bct<<<1 + (unsigned)((items + 255) / 256), 256, 0, s>>>(a->lam, d);
    }
    {
        long long seg;
        unsigned nb;
        ns::filter_shape(d.imax, d.jmax, 4, a->warm_t, c->nsm, ns::kFilterWarpsPerSmsp, seg, nb);
        ns::adj::k_filter_t<true><<<nb, 128, 0, s>>>(d, a->lam, a->lam2, seg, a->warm_t,
                                                      a->warm32_t, c->fy);
        ns::filter_shape(d.jmax, d.imax, 4, a->warm_t, c->nsm, ns::kFilterWarpsPerSmsp, seg, nb);
        ns::adj::k_filter_t<false><<<nb, 128, 0, s>>>(d, a->lam2, a->lam, seg, a->warm_t,
                                                       a->warm32_t, c->fx);
    }
    const dim3 blk(32, 4), grd((d.imax + 31) / 32, (d.jmax + 3) / 4);
    ns::adj::k_point_t<<<grd, blk, 0, s>>>(d, a->lam, a->om, a->lx, a->ly, U, Um, Un,
                                           c->sigx, c->sigy, a->gS, c->phys.gamma, c->p.dt,
                                           c->alpha[stage], c->beta[stage], sink);
    if (a->dt_maps)
        ns::adj::k_deriv_t<true><<<grd, blk, 0, s>>>(a->lxmap, a->lymap, c->d_err, d, a->lam, a->lx,
                                                     a->ly, c->xcoef, c->ycoef);
    else
        ns::adj::k_deriv_t<false><<<grd, blk, 0, s>>>(a->lxmap, a->lymap, c->d_err, d, a->lam,
                                                      a->lx, a->ly, c->xcoef, c->ycoef);
    A_CUDA(a, cudaGetLastError());
    return NS_OK;
}

// One forward step that copies every stage's input into the stage store,
// then adds the step's loss term and advances the device step index.
cudaError_t launch_forward_store(ns_adjoint *a, cudaStream_t s)
{
    ns_ctx *c = a->fwd;
    const long long n4 = 4LL * c->d.plane;
    int cls[ns::kMaxStepLaunches], stg[ns::kMaxStepLaunches];
    const int n = ns::step_sequence(c, cls, stg);
    const unsigned nb = (unsigned)std::min<long long>((n4 / 2 + 255) / 256, 4LL * 152);
    for (int q = 0; q < n; q++) {
        if (cls[q] == NS_KC_FIRST)
            ns::adj::k_store_stage<<<nb, 256, 0, s>>>(c->U, a->stages, a->d_step, stg[q], n4);
        cudaError_t e = ns::launch_kernel(c, cls[q], stg[q], s);
        if (e != cudaSuccess) return e;
    }
    ns::adj::k_obs_loss<<<1, 32, 0, s>>>(c->U, c->d, a->obs, a->nobs, a->pb, a->loss);
    ns::adj::k_step_inc<<<1, 1, 0, s>>>(a->d_step);
    return cudaGetLastError();
}

// The stage store for nsteps steps, when it fits in device memory with a
// quarter of the free memory to spare; false: use checkpoints instead.
bool ensure_stages(ns_adjoint *a, int nsteps)
{
    if (a->stages && a->stages_cap >= nsteps) return true;
    ns_ctx *c = a->fwd;
    const size_t bytes = (size_t)nsteps * 6 * 4 * (size_t)c->d.plane * sizeof(double);
    if (a->fwd_exec) {
        cudaGraphExecDestroy(a->fwd_exec);  // it holds the old store's address
        a->fwd_exec = nullptr;
    }
    if (a->stages) cudaFree(a->stages);
    a->stages = nullptr;
    a->stages_cap = 0;
    size_t freeb = 0, total = 0;
    if (cudaMemGetInfo(&freeb, &total) != cudaSuccess || bytes > freeb / 4 * 3) {
        cudaGetLastError();
        return false;
    }
    if (cudaMalloc(&a->stages, bytes) != cudaSuccess) {
        cudaGetLastError();
        a->stages = nullptr;
        return false;
    }
    a->stages_cap = nsteps;
    return true;
}

int ensure_forward_graph(ns_adjoint *a)
{
    if (a->fwd_exec) return NS_OK;
    cudaStream_t cs;
    A_CUDA(a, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const cudaError_t le = launch_forward_store(a, cs);
        e = cudaStreamEndCapture(cs, &g);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&a->fwd_exec, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) {
        a->fwd_exec = nullptr;
        cudaGetLastError();
        return aerr(a, NS_ERR_CUDA, std::string("capture of the adjoint forward step: ") +
                                        cudaGetErrorString(e));
    }
    return NS_OK;
}

}  // namespace

extern "C" {

int ns_adjoint_create(const ns_params *p, int nobs, const double *obs_x, const double *obs_y,
                      int checkpoint_every, ns_adjoint **out)
{
    if (!out || !p || nobs < 1 || !obs_x || !obs_y || checkpoint_every < 0)
        return aerr(nullptr, NS_ERR_PARAM, "ns_adjoint_create: bad argument");
    *out = nullptr;
    if (!p->inviscid || p->nk != 4 || p->precision != NS_PREC_FP64 ||
        p->source_mode != NS_SRC_FIELD || !p->m || !p->n)
        return aerr(nullptr, NS_ERR_UNSUPPORTED,
                    "ns_adjoint_create: the adjoint covers the FP64 Euler step (inviscid=1, nk=4) "
                    "with a source field (NS_SRC_FIELD) and coordinates m, n");
    ns_adjoint *a = new (std::nothrow) ns_adjoint();
    if (!a) return aerr(nullptr, NS_ERR_OOM, "ns_adjoint_create: host allocation");
    int rc = ns_create(p, &a->fwd);
    if (rc != NS_OK) {
        delete a;
        return rc;
    }
    ns_ctx *c = a->fwd;
    a->K = checkpoint_every;
    a->nobs = nobs;
    // The transposed sweeps' pieces warm up until the error of their
    // unfiltered start is below 2^-50 of the data (the forward sweeps: 2^-60,
    // rounding-level agreement with the serial sweep): about 1e-15 per sweep,
    // far below the 1e-9 to which a gradient is compared with finite
    // differences, and 5 FP64 steps fewer per piece at sigmaf = 0.2.
    ns::coef::fp64_warmups(p->sigmaf, a->warm_t, a->warm32_t, 50);
    a->dudm0 = c->dudm;
    a->dudn0 = c->dudn;
    // base pressure (uniform p_b is required: the loss is on p - p_b)
    a->pb = (p->ub_layout == NS_LAYOUT_FORTRAN || p->ub_layout == NS_LAYOUT_ROWS)
                ? p->Ub[3]
                : p->Ub[3 * (size_t)p->imax * p->jmax];
    std::vector<ns::adj::Obs> ob(nobs);
    const double x0 = p->m[0], y0 = p->n[0];
    for (int q = 0; q < nobs; q++) {
        const double fx = (obs_x[q] - x0) / p->dm, fy = (obs_y[q] - y0) / p->dn;
        const int i0 = (int)std::floor(fx), j0 = (int)std::floor(fy);
        if (i0 < 0 || j0 < 0 || i0 + 1 >= p->imax || j0 + 1 >= p->jmax) {
            ns_destroy(c);
            delete a;
            return aerr(nullptr, NS_ERR_PARAM, "ns_adjoint_create: observer outside the grid");
        }
        ob[q] = {i0, j0, fx - i0, fy - j0};
    }
    const size_t P = (size_t)c->d.plane;
    cudaError_t e = cudaMalloc(&a->obs, nobs * sizeof(ns::adj::Obs));
    if (e == cudaSuccess) e = cudaMalloc(&a->loss, sizeof(double));
    a->store_steps = a->K;
    const size_t store_planes = a->K ? (size_t)a->K * kStepPlanes + 4 : 12;
    if (e == cudaSuccess) e = cudaMalloc(&a->store, store_planes * P * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&a->d_step, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&a->endstate, 4 * P * sizeof(double));
    double **bufs[] = {&a->lam, &a->lam2, &a->om, &a->lx, &a->ly};
    for (double **b : bufs)
        if (e == cudaSuccess) e = cudaMalloc(b, 4 * P * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&a->gS, P * sizeof(double));
    if (e == cudaSuccess)
        e = cudaMemcpy(a->obs, ob.data(), nobs * sizeof(ns::adj::Obs), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        rc = aerr(nullptr, NS_ERR_OOM, std::string("ns_adjoint_create: ") + cudaGetErrorString(e));
        ns_adjoint_destroy(a);
        return rc;
    }
    // the tiled transposed derivative when the context's FP64 tiles are in
    // use (same layout); otherwise every point reads global memory
    a->dt_maps = c->fp64_maps &&
                 ns::make_plane_map(c, &a->lxmap, a->lx, 4, ns::adj::kDtXW, ns::adj::kDtBY) == NS_OK &&
                 ns::make_plane_map(c, &a->lymap, a->ly, 4, ns::adj::kDtBX, ns::adj::kDtYH) == NS_OK;
    *out = a;
    return NS_OK;
}

void ns_adjoint_destroy(ns_adjoint *a)
{
    if (!a) return;
    if (a->fwd) {
        cudaSetDevice(a->fwd->dev);
        cudaStreamSynchronize(a->fwd->stream);
        a->fwd->dudm = a->dudm0;
        a->fwd->dudn = a->dudn0;
    }
    if (a->fwd_exec) cudaGraphExecDestroy(a->fwd_exec);
    void *ps[] = {a->obs, a->loss, a->chk, a->store, a->store2, a->endstate, a->lam, a->lam2,
                  a->om, a->lx, a->ly, a->gS, a->stages, a->d_step};
    for (void *p : ps)
        if (p) cudaFree(p);
    for (cudaStream_t st : {a->s_rec, a->s_rev})
        if (st) cudaStreamDestroy(st);
    for (cudaEvent_t ev : {a->ev_rec[0], a->ev_rec[1], a->ev_rev[0], a->ev_rev[1], a->ev_start})
        if (ev) cudaEventDestroy(ev);
    if (a->fwd) ns_destroy(a->fwd);
    delete a;
}

// Replaces the source field S (imax*jmax doubles, i fastest).
int ns_adjoint_set_source(ns_adjoint *a, const double *field)
{
    if (!a || !field) return aerr(a, NS_ERR_PARAM, "ns_adjoint_set_source: NULL argument");
    ns_ctx *c = a->fwd;
    const size_t row = (size_t)c->d.imax * sizeof(double);
    A_CUDA(a, cudaMemcpy2DAsync(c->src, c->d.pitch * sizeof(double), field, row, row,
                                (size_t)c->d.jmax, cudaMemcpyHostToDevice, c->stream));
    A_CUDA(a, cudaStreamSynchronize(c->stream));
    a->forward_done = false;
    return NS_OK;
}

// Forward pass from U0 (host, layout as ns_set_state) for nsteps steps with
// iter = iter0.. ; checkpoints every K steps; *loss = the observer loss.
int ns_adjoint_forward(ns_adjoint *a, const double *U0, int layout, int iter0, int nsteps,
                       double *loss)
{
    if (!a || !U0 || nsteps < 1 || !loss) return aerr(a, NS_ERR_PARAM, "ns_adjoint_forward: bad argument");
    ns_ctx *c = a->fwd;
    const size_t P = (size_t)c->d.plane;
    int rc = ns_set_state(c, U0, layout);
    if (rc != NS_OK) return rc;
    cudaStream_t s = c->stream;
    a->stored_all = (a->K == 0) && ensure_stages(a, nsteps);
    if (a->stored_all) {
        if ((rc = ensure_forward_graph(a)) != NS_OK) return rc;
        A_CUDA(a, cudaMemsetAsync(a->loss, 0, sizeof(double), s));
        A_CUDA(a, cudaMemsetAsync(a->d_step, 0, sizeof(int), s));
        A_CUDA(a, ns::launch_set_iter(c->d_iter, iter0, s));
        for (int n = 0; n < nsteps; n++) A_CUDA(a, cudaGraphLaunch(a->fwd_exec, s));
        A_CUDA(a, cudaMemcpyAsync(a->endstate, c->U, 4 * P * sizeof(double),
                                  cudaMemcpyDeviceToDevice, s));
        A_CUDA(a, cudaMemcpyAsync(loss, a->loss, sizeof(double), cudaMemcpyDeviceToHost, s));
        if ((rc = ns_synchronize(c)) != NS_OK) return aerr(a, rc, ns_last_error(c));
        a->nsteps = nsteps;
        a->iter0 = iter0;
        a->forward_done = true;
        return NS_OK;
    }
    const int K = a->K ? a->K : kDefaultCheckpoint;
    if ((rc = ensure_segment_stores(a, K)) != NS_OK) return rc;
    const int nchk = (nsteps + K - 1) / K;
    if (nchk > a->nchk) {
        if (a->chk) cudaFree(a->chk);
        a->chk = nullptr;
        A_CUDA(a, cudaMalloc(&a->chk, (size_t)nchk * 4 * P * sizeof(double)));
        a->nchk = nchk;
    }
    // The steps of the last segment, and of the one before it when the
    // second store exists, keep their stage inputs and derivatives in the
    // stores the reverse pass reads them from (it starts without recomputing
    // either); the rest replay the step graph.
    const int last0 = (nchk - 1) * K;
    double *last = seg_store(a, nchk - 1);
    const bool keep_prev = a->store2 && nchk >= 2;
    const int prev0 = keep_prev ? (nchk - 2) * K : last0;
    double *prev = keep_prev ? seg_store(a, nchk - 2) : nullptr;
    A_CUDA(a, cudaMemsetAsync(a->loss, 0, sizeof(double), s));
    for (int n = 0; n < nsteps; n++) {
        if (n % K == 0)
            A_CUDA(a, cudaMemcpyAsync(a->chk + (size_t)(n / K) * 4 * P, c->U, 4 * P * sizeof(double),
                                      cudaMemcpyDeviceToDevice, s));
        if (keep_prev && n == last0)  // the state after the previous segment's last step
            A_CUDA(a, cudaMemcpyAsync(seg_slot(prev, K, P), c->U, 4 * P * sizeof(double),
                                      cudaMemcpyDeviceToDevice, s));
        rc = (n >= last0)   ? forward_step(a, iter0 + n, seg_slot(last, n - last0, P), s)
             : (n >= prev0) ? forward_step(a, iter0 + n, seg_slot(prev, n - prev0, P), s)
                            : ns_step(c, iter0 + n, 1);
        if (rc != NS_OK) return rc;
        ns::adj::k_obs_loss<<<1, 32, 0, s>>>(c->U, c->d, a->obs, a->nobs, a->pb, a->loss);
    }
    A_CUDA(a, cudaMemcpyAsync(seg_slot(last, nsteps - last0, P), c->U, 4 * P * sizeof(double),
                              cudaMemcpyDeviceToDevice, s));
    A_CUDA(a, cudaMemcpyAsync(a->endstate, c->U, 4 * P * sizeof(double), cudaMemcpyDeviceToDevice, s));
    A_CUDA(a, cudaMemcpyAsync(loss, a->loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    if ((rc = ns_synchronize(c)) != NS_OK) return aerr(a, rc, ns_last_error(c));
    a->nsteps = nsteps;
    a->iter0 = iter0;
    a->forward_done = true;
    a->stored_segs = keep_prev ? 2 : 1;
    return NS_OK;
}

// Reverse pass: grad_field[imax*jmax] (i fastest) = dL/dS.
int ns_adjoint_backward(ns_adjoint *a, double *grad_field)
{
    if (!a || !grad_field) return aerr(a, NS_ERR_PARAM, "ns_adjoint_backward: NULL argument");
    if (!a->forward_done) return aerr(a, NS_ERR_STATE, "ns_adjoint_backward before ns_adjoint_forward");
    ns_ctx *c = a->fwd;
    const ns::Dims &d = c->d;
    const size_t P = (size_t)d.plane;
    cudaStream_t s = c->stream;
    A_CUDA(a, cudaMemsetAsync(a->lam, 0, 4 * P * sizeof(double), s));
    A_CUDA(a, cudaMemsetAsync(a->gS, 0, P * sizeof(double), s));
    int rc;
    if (a->stored_all) {
        // every stage input is stored: per stage, only its first derivatives
        // are recomputed (k_first on a copy in the context's U, into the
        // scratch slot), then the stage is reversed
        double *Um = a->store + 4 * P, *Un = a->store + 8 * P;
        for (int n = a->nsteps - 1; n >= 0; n--) {
            const double *Unext = (n == a->nsteps - 1)
                                      ? a->endstate
                                      : a->stages + (size_t)(n + 1) * 6 * 4 * P;
            ns::adj::k_obs_grad<<<(a->nobs + 63) / 64, 64, 0, s>>>(Unext, d, a->obs, a->nobs,
                                                                  a->pb, a->lam);
            A_CUDA(a, cudaMemsetAsync(a->om, 0, 4 * P * sizeof(double), s));
            double sn[6];
            stage_sines(c, a->iter0 + n, sn);
            for (int st = 5; st >= 0; st--) {
                const double *U = a->stages + ((size_t)n * 6 + st) * 4 * P;
                A_CUDA(a, cudaMemcpyAsync(c->U, U, 4 * P * sizeof(double),
                                          cudaMemcpyDeviceToDevice, s));
                c->dudm = Um;
                c->dudn = Un;
                const cudaError_t e = ns::launch_kernel(c, NS_KC_FIRST, st, s);
                c->dudm = a->dudm0;
                c->dudn = a->dudn0;
                A_CUDA(a, e);
                if ((rc = stage_adjoint(a, U, Um, Un, st, sn[st], s)) != NS_OK) return rc;
            }
        }
    }
    const int K = a->K ? a->K : kDefaultCheckpoint;
    const int nseg = a->stored_all ? 0 : (a->nsteps + K - 1) / K;
    // Segments: the recompute of segment sg-1 (stream s_rec) runs beside the
    // reverse of segment sg (stream s_rev) when the second store exists;
    // events order each store's writer after its previous reader.
    cudaStream_t srec = s, srev = s;
    if (nseg > 0) {
        if (!a->s_rec) {
            A_CUDA(a, cudaStreamCreateWithFlags(&a->s_rec, cudaStreamNonBlocking));
            A_CUDA(a, cudaStreamCreateWithFlags(&a->s_rev, cudaStreamNonBlocking));
            for (int k = 0; k < 2; k++) {
                A_CUDA(a, cudaEventCreateWithFlags(&a->ev_rec[k], cudaEventDisableTiming));
                A_CUDA(a, cudaEventCreateWithFlags(&a->ev_rev[k], cudaEventDisableTiming));
            }
            A_CUDA(a, cudaEventCreateWithFlags(&a->ev_start, cudaEventDisableTiming));
        }
        srec = a->s_rec;
        srev = a->s_rev;
        // both start after everything enqueued on the context's stream
        A_CUDA(a, cudaEventRecord(a->ev_start, s));
        A_CUDA(a, cudaStreamWaitEvent(srec, a->ev_start, 0));
        A_CUDA(a, cudaStreamWaitEvent(srev, a->ev_start, 0));
    }
    const bool pipe = a->store2 != nullptr;
    auto seg_n0 = [&](int sg) { return sg * K; };
    auto seg_len = [&](int sg) { return std::min(a->nsteps, (sg + 1) * K) - sg * K; };
    // recompute segment sg from its checkpoint, keeping every stage's input
    // and derivatives, and the state after its last step
    auto rec_begin = [&](int sg) -> int {
        A_CUDA(a, cudaMemcpyAsync(c->U, a->chk + (size_t)sg * 4 * P, 4 * P * sizeof(double),
                                  cudaMemcpyDeviceToDevice, srec));
        return NS_OK;
    };
    auto rec_step = [&](int sg, int q) -> int {
        return forward_step(a, a->iter0 + seg_n0(sg) + q, seg_slot(seg_store(a, sg), q, P), srec);
    };
    auto rec_end = [&](int sg) -> int {
        A_CUDA(a, cudaMemcpyAsync(seg_slot(seg_store(a, sg), seg_len(sg), P), c->U,
                                  4 * P * sizeof(double), cudaMemcpyDeviceToDevice, srec));
        A_CUDA(a, cudaEventRecord(a->ev_rec[sg & 1], srec));
        return NS_OK;
    };
    // reverse of step n of segment sg: the loss term of the state after it,
    // then its six stages
    auto rev_step = [&](int sg, int n) -> int {
        double *st = seg_store(a, sg);
        const int q = n - seg_n0(sg);
        ns::adj::k_obs_grad<<<(a->nobs + 63) / 64, 64, 0, srev>>>(seg_slot(st, q + 1, P), d, a->obs,
                                                                   a->nobs, a->pb, a->lam);
        A_CUDA(a, cudaMemsetAsync(a->om, 0, 4 * P * sizeof(double), srev));
        double sn[6];
        stage_sines(c, a->iter0 + n, sn);
        const double *slot = seg_slot(st, q, P);
        for (int k = 5; k >= 0; k--) {
            const double *U = slot + (size_t)k * 12 * P;
            const int r = stage_adjoint(a, U, U + 4 * P, U + 8 * P, k, sn[k], srev);
            if (r != NS_OK) return r;
        }
        return NS_OK;
    };
#define A_TRY(call)                        \
    do {                                   \
        if ((rc = (call)) != NS_OK) return rc; \
    } while (0)
    // segments sg >= kept need no recompute: the forward left them in place
    const int kept = nseg - std::min(a->stored_segs, nseg);
    if (nseg > 0) {
        if (nseg - 1 >= kept) {
            A_CUDA(a, cudaEventRecord(a->ev_rec[(nseg - 1) & 1], srec));
        } else {
            A_TRY(rec_begin(nseg - 1));
            for (int q = 0; q < seg_len(nseg - 1); q++) A_TRY(rec_step(nseg - 1, q));
            A_TRY(rec_end(nseg - 1));
        }
    }
    // the stores are reused below: a second backward recomputes every segment
    a->stored_segs = 0;
    for (int sg = nseg - 1; sg >= 0; sg--) {
        A_CUDA(a, cudaStreamWaitEvent(srev, a->ev_rec[sg & 1], 0));
        const int nr = seg_len(sg), n1 = seg_n0(sg) + nr;
        // segment sg-1 is recomputed unless the forward kept it
        const bool rec = sg > 0 && sg - 1 < kept;
        const int nc = rec ? seg_len(sg - 1) : 0;
        if (pipe) {
            if (rec) {
                // segment sg-1 goes into the store segment sg+1 was reversed from
                if (sg + 1 < nseg) A_CUDA(a, cudaStreamWaitEvent(srec, a->ev_rev[(sg + 1) & 1], 0));
                A_TRY(rec_begin(sg - 1));
            } else if (sg > 0) {
                A_CUDA(a, cudaEventRecord(a->ev_rec[(sg - 1) & 1], srec));
            }
            // one step of each chain at a time, so that neither stream's
            // queue runs ahead of the other's
            for (int q = 0; q < std::max(nr, nc); q++) {
                if (q < nr) A_TRY(rev_step(sg, n1 - 1 - q));
                if (q < nc) A_TRY(rec_step(sg - 1, q));
            }
            if (rec) A_TRY(rec_end(sg - 1));
            A_CUDA(a, cudaEventRecord(a->ev_rev[sg & 1], srev));
        } else {
            for (int q = 0; q < nr; q++) A_TRY(rev_step(sg, n1 - 1 - q));
            A_CUDA(a, cudaEventRecord(a->ev_rev[sg & 1], srev));
            if (sg > 0) {
                A_CUDA(a, cudaStreamWaitEvent(srec, a->ev_rev[sg & 1], 0));
                A_TRY(rec_begin(sg - 1));
                for (int q = 0; q < nc; q++) A_TRY(rec_step(sg - 1, q));
                A_TRY(rec_end(sg - 1));
            }
        }
    }
#undef A_TRY
    const size_t row = (size_t)d.imax * sizeof(double);
    A_CUDA(a, cudaMemcpy2DAsync(grad_field, row, a->gS, d.pitch * sizeof(double), row,
                                (size_t)d.jmax, cudaMemcpyDeviceToHost, srev));
    A_CUDA(a, cudaStreamSynchronize(srec));
    A_CUDA(a, cudaStreamSynchronize(srev));
    if ((rc = ns_synchronize(c)) != NS_OK) return aerr(a, rc, ns_last_error(c));
    // leave the context's state at the forward end state
    A_CUDA(a, cudaMemcpy(c->U, a->endstate, 4 * P * sizeof(double), cudaMemcpyDeviceToDevice));
    return NS_OK;
}

int ns_adjoint_stored_bytes(const ns_adjoint *a, int64_t *bytes)
{
    if (!a || !bytes) return aerr(nullptr, NS_ERR_PARAM, "ns_adjoint_stored_bytes: NULL argument");
    *bytes = a->stored_all ? (int64_t)a->nsteps * 6 * 4 * a->fwd->d.plane * (int64_t)sizeof(double)
                           : 0;
    return NS_OK;
}

int ns_adjoint_context(ns_adjoint *a, ns_ctx **ctx)
{
    if (!a || !ctx) return aerr(a, NS_ERR_PARAM, "ns_adjoint_context: NULL argument");
    *ctx = a->fwd;
    return NS_OK;
}

}  // extern "C"
