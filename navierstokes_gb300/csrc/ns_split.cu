// ns_split.cu -- split-precision stage loop: FP64 mean flow + FP32 perturbation.
//
// The state is U = Ub + q' with Ub the FP64 base flow (constant in time,
// uniform in x, v = 0, p uniform) and q' = (rho',u',v',p') stored in FP32.
// Every stencil and filter sum runs in FP32 over q'; the LDDRK accumulator w
// (rk.f90:163) stays FP64.  The equations are the Euler right-hand side of
// eqeuler.f90:53-92 (1/Re = 0) written for U = Ub + q': with dUb/dx = 0,
// v_b = 0 and dp_b = 0 every term is perturbation-sized, so no FP32
// difference of two O(1) numbers is ever formed.  The mean flow's own right
// hand side vanishes; the y filter, whose REAL(4) boundary coefficients do
// not preserve constants (filtering.f90:114-120), acts on Ub by a fixed
// FP64 amount that is precomputed per row and added back.
//
// With NP = 3 (NS_PREC_SPLIT) u', v' and p' are each carried as an
// unevaluated sum of two FP32 numbers (hi + lo, about 48 significant bits);
// rho' is a single FP32 number.  With NP = 0 (NS_PREC_SPLIT32) all four are
// single FP32 numbers.  FP32 storage rounds every value three times per
// stage; that noise random-walks at wavenumbers the selective filter does not
// damp.  For a vortex with |u'| ~ 1e-3 next to an acoustic pulse it reached
// ~35 ulps of u' after 300 steps and drove p' through the divergence to
// 7e-10 (1e-4 of p').  With pairs the floor is the rounding of the FP32
// right-hand side, which the base-flow advection in float-float and the
// accumulator update by the FP64 product beta*dt keep near what an FP64
// right-hand side from the same pairs gives (about 1e-11 of p' at the vortex
// after 1000 steps).  Planes of a perturbation buffer: 0 rho', 1 u', 2 v',
// 3 p' (hi parts), then 3 + k the lo part of variable k = 1 .. NP.
//
// FP64 <-> FP32 conversions of the accumulator update are done with integer
// bit operations (ns_f32conv.cuh): on GB300 the F2F instructions run on the
// FP64 pipe, which is about 60x slower than FP32.
#include "ns_internal.cuh"
#include "ns_check.cuh"
#include "ns_f32conv.cuh"
#include "ns_tma.cuh"

namespace ns {

// ---------------------------------------------------------------------------
// Fused stage kernel: FP32 derivatives from a shared-memory tile, Euler RHS,
// FP64 LDDRK update, buffer damping.  Out of place (qin -> qout).
// ---------------------------------------------------------------------------
constexpr int kTX = 32, kTY = kSplitTY, kH = 3;
constexpr int kPT = kTY / 8;  // points per thread (8 thread rows)
constexpr int kSH = kTY + 2 * kH;
// Tile width in shared memory: the TMA box starts 4 columns left of the
// block (its x coordinate times 4 bytes must be a multiple of 16) and spans
// 40 columns (a multiple of 16 bytes): i0-4 .. i0+35 covers the halo of 3.
constexpr int kTL = 4, kSW = 40;

// One-sided closure, written as sum_z c_z*(f_z - f_q): the closure
// coefficients sum to zero, and in this form a constant field gives exactly
// zero in FP32 as well (their FP32 roundings no longer sum to zero).
__device__ __forceinline__ float closure_f32(const float *__restrict__ g, long long st, int q,
                                             int n, const float *__restrict__ c)
{
    const int o0 = (q < 3) ? -q : (n - 7 - q);
    const float *p = g + (long long)o0 * st;
    const float f0 = g[0];
    float r = 0.f;
#pragma unroll
    for (int z = 0; z < 7; z++) r = fmaf(c[z], p[(long long)z * st] - f0, r);
    return r;
}

// Float-float pieces (Knuth two-sum, FMA two-product) for the divergence.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// sum_s c_s*(f[+s] - f[-s]) for s = 1..3 in float-float: the differences
// exact (two-sum), each coefficient as hi + lo (the FP64 table value), the
// products exact (FMA), the sum compensated.  Returns hi and lo.
__device__ __forceinline__ void drp_ff(const float *fp, const float *fm, const float *ch,
                                       const float *cl, float &hi, float &lo)
{
    hi = 0.f;
    lo = 0.f;
#pragma unroll
    for (int s = 0; s < 3; s++) {
        float dh, dl;
        two_sum(fp[s], -fm[s], dh, dl);
        const float ph = ch[s] * dh;
        const float pl = fmaf(ch[s], dh, -ph) + fmaf(ch[s], dl, cl[s] * dh);
        float sh, se;
        two_sum(hi, ph, sh, se);
        hi = sh;
        lo += se + pl;
    }
}

// Variable k (0 rho', 1 u', 2 v', 3 p') is a hi + lo pair when 1 <= k <= NP.
template <int NP>
__device__ __forceinline__ constexpr bool is_pair(int k)
{
    return k >= 1 && k <= NP;
}

// (h, l) + a for a pair with |h| >= |l + a| (Fast2Sum): renormalised pair
__device__ __forceinline__ void pair_add(float &h, float &l, float a)
{
    const float t = l + a;
    const float nh = h + t;
    l = t - (nh - h);
    h = nh;
}

// (h, l) * s with the product's rounding error kept (FMA two-product)
__device__ __forceinline__ void pair_scale(float &h, float &l, float s)
{
    const float p = h * s;
    const float e = fmaf(h, s, -p);
    l = fmaf(l, s, e);
    h = p;
}

// ---------------------------------------------------------------------------
// Viscous terms (Navier-Stokes, base flow uniform in x and y with v = 0):
// the base flow's own stresses and heat flux vanish, so tau and k grad T
// are perturbation-sized and FP32 carries them.
// ---------------------------------------------------------------------------
// T' = T - T_b for T = gamma*p/rho (rhs.f90:20) written without the
// cancellation of two O(1) temperatures:
// T' = gamma*(p'*rho_b - p_b*rho') / (rho_b*(rho_b + rho')).
__device__ __forceinline__ float t_prime(float rho1, float p1, const SplitVisc &v)
{
    const float num = fmaf(p1, v.rho_b, -(v.p_b * rho1));
    return v.gamma * num / (v.rho_b * (v.rho_b + rho1));
}

// mu(T) and k(T) with 1/mu0, 1/k0 folded in (coefficients.f90:27-59): the
// FP32 copy of the context's piecewise-polynomial table (the piece from the
// exponent and the top 8 fraction bits of T, Horner in u = T minus the
// piece's left end, exact by Sterbenz), else the fit itself by logf/expf.
__device__ __forceinline__ void transport_f32(float T, const float *__restrict__ trf,
                                              const SplitVisc &v, float &mu, float &kc)
{
    const unsigned b = __float_as_uint(T);
    const int e = (int)((b >> 23) & 0xffu) - 127;
    if (!(b >> 31) && e >= kTrEmin && e < kTrEmin + kTrOctaves) {
        const int piece = ((e - kTrEmin) << 8) | (int)((b >> 15) & 255u);
        const float u = T - __uint_as_float(b & 0xffff8000u);
        const float *c = trf + (size_t)piece * kTrStride;
        mu = fmaf(fmaf(fmaf(fmaf(fmaf(c[5], u, c[4]), u, c[3]), u, c[2]), u, c[1]), u, c[0]);
        kc = fmaf(fmaf(fmaf(fmaf(fmaf(c[11], u, c[10]), u, c[9]), u, c[8]), u, c[7]), u, c[6]);
        return;
    }
    const float x = v.Tref * T;
    const float L = logf(x), y = 1.0f / x;
    mu = expf(fmaf(v.A_mi, L, fmaf(fmaf(v.C_mi, y, v.B_mi), y, v.D_mi_s)));
    kc = expf(fmaf(v.A_k, L, fmaf(fmaf(v.C_k, y, v.B_k), y, v.D_k_s)));
}

// T' at point (i, j) from global memory (closure points near the edges).
template <int NP>
__device__ __forceinline__ float t_prime_at(const float *__restrict__ q, long long fplane,
                                            long long idx, const SplitVisc &v)
{
    float p1 = q[3 * fplane + idx];
    if (NP >= 3) p1 += q[6 * fplane + idx];
    return t_prime(q[idx], p1, v);
}

// tau' (eqeuler.f90:37-39) and k grad T' (derivs.f90:48-56) of the
// perturbation, at every point: five FP32 planes for the stage kernel.  The
// halo tile of q' arrives by TMA as in the stage kernel; T' is formed for
// every tile point in shared memory, then differentiated there (closures:
// from global memory).  Velocity gradients use the hi parts: their lo parts
// are below 2^-24 of them and the stresses enter the right-hand side times
// 1/Re.
template <int NP>
__global__ void __launch_bounds__(256, kSplitMinBlocks)
    k_split_visc(const __grid_constant__ CUtensorMap qmap, int *__restrict__ err, Dims d,
                 int fpitch, const float *__restrict__ q, float *__restrict__ tau,
                 const float *__restrict__ xc, const float *__restrict__ yc,
                 const float *__restrict__ trf, const SplitVisc v)
{
    constexpr int kTX_ = 32, kTY_ = kSplitTY, kH_ = 3, kSH_ = kTY_ + 2 * kH_;
    constexpr int kTL_ = 4, kSW_ = 40, NPL = 4 + NP;
    __shared__ alignas(128) float sq[NPL][kSH_][kSW_];
    __shared__ float sT[kSH_][kSW_];
    __shared__ alignas(8) unsigned long long tbar;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = blockIdx.x * kTX_, j0 = blockIdx.y * kTY_;
    const long long fplane = (long long)fpitch * d.jmax;
    const bool lead = (tx == 0 && ty == 0);
    NS_CHECK(err, kChkSplit, blockDim.x == kTX_ && blockDim.y == 8 && kTY_ % 8 == 0);
    NS_CHECK(err, kChkSplit, ((i0 - kTL_) & 3) == 0 && fpitch >= d.imax && d.imax >= 7 &&
                                 d.jmax >= 7);
    if (lead) mbar_init(&tbar, 1);
    __syncthreads();
    if (lead) {
        mbar_expect_tx(&tbar, (unsigned)sizeof(sq));
        tma_load_3d(&sq[0][0][0], &qmap, i0 - kTL_, j0 - kH_, 0, &tbar);
    }
    if (!mbar_wait_bounded(&tbar, 0, err)) return;
    const int tid = ty * kTX_ + tx;
    for (int e = tid; e < kSH_ * kSW_; e += kTX_ * 8) {
        const int r = e / kSW_, c = e % kSW_;
        float p1 = sq[3][r][c];
        if (NP >= 3) p1 += sq[6][r][c];
        sT[r][c] = t_prime(sq[0][r][c], p1, v);
    }
    __syncthreads();
    const int i = i0 + tx;
    if (i >= d.imax) return;
    const float *cxp = xc + kCoefStride * i;
    const bool xint = (i >= 3 && i < d.imax - 3);
#pragma unroll
    for (int h = 0; h < kTY_ / 8; h++) {
        const int ly = ty + 8 * h;
        const int j = j0 + ly;
        if (j >= d.jmax) break;
        const long long fidx = (long long)j * fpitch + i;
        const int sr = ly + kH_, sc = tx + kTL_;
        const float *cyp = yc + kCoefStride * j;
        const bool yint = (j >= 3 && j < d.jmax - 3);
        // x and y derivatives of a tile plane, closures from global memory
        auto ddx = [&](const float (*t)[kSW_], auto glob) -> float {
            if (xint) {
                float r = cxp[4] * (t[sr][sc + 1] - t[sr][sc - 1]);
                r = fmaf(cxp[5], t[sr][sc + 2] - t[sr][sc - 2], r);
                return fmaf(cxp[6], t[sr][sc + 3] - t[sr][sc - 3], r);
            }
            const int o0 = (i < 3) ? -i : (d.imax - 7 - i);
            const float f0 = glob(fidx);
            float r = 0.f;
#pragma unroll
            for (int z = 0; z < 7; z++) r = fmaf(cxp[z], glob(fidx + o0 + z) - f0, r);
            return r;
        };
        auto ddy = [&](const float (*t)[kSW_], auto glob) -> float {
            if (yint) {
                float r = cyp[4] * (t[sr + 1][sc] - t[sr - 1][sc]);
                r = fmaf(cyp[5], t[sr + 2][sc] - t[sr - 2][sc], r);
                return fmaf(cyp[6], t[sr + 3][sc] - t[sr - 3][sc], r);
            }
            const int o0 = (j < 3) ? -j : (d.jmax - 7 - j);
            const float f0 = glob(fidx);
            float r = 0.f;
#pragma unroll
            for (int z = 0; z < 7; z++)
                r = fmaf(cyp[z], glob(fidx + (long long)(o0 + z) * fpitch) - f0, r);
            return r;
        };
        auto gu = [&](long long x) { return q[fplane + x]; };
        auto gv = [&](long long x) { return q[2 * fplane + x]; };
        auto gT = [&](long long x) { return t_prime_at<NP>(q, fplane, x, v); };
        const float ux = ddx(sq[1], gu), uy = ddy(sq[1], gu);
        const float vx = ddx(sq[2], gv), vy = ddy(sq[2], gv);
        const float Tx = ddx(sT, gT), Ty = ddy(sT, gT);
        float mu, kc;
        transport_f32(v.T_b + sT[sr][sc], trf, v, mu, kc);
        const float div = ux + vy;
        const float m23 = (2.0f / 3.0f) * mu, mu2 = 2.0f * mu;
        tau[fidx] = fmaf(mu2, ux, -(m23 * div));
        tau[fplane + fidx] = mu * (uy + vx);
        tau[2 * fplane + fidx] = fmaf(mu2, vy, -(m23 * div));
        tau[3 * fplane + fidx] = kc * Tx;
        tau[4 * fplane + fidx] = kc * Ty;
    }
}

// Resident blocks per SM: 4 with pairs (64 registers), 5 with single FP32
// perturbations (48 registers), 3 with the viscous tile.
template <int NP, bool VISC>
constexpr int split_stage_blocks() { return VISC ? 3 : (NP == 0 ? 5 : kSplitMinBlocks); }

template <int NP, bool FIRST, bool SRC, bool VISC>
__global__ void __launch_bounds__(256, split_stage_blocks<NP, VISC>())
    k_split_stage(const __grid_constant__ CUtensorMap qmap, const __grid_constant__ CUtensorMap vmap,
                  const float *__restrict__ tau, const float *__restrict__ trf, const SplitVisc vis,
                  int *__restrict__ err, Dims d,
                  int fpitch, const float *__restrict__ qin, float *__restrict__ qout,
                  double *__restrict__ W, const float *__restrict__ xc,
                  const float *__restrict__ yc, const float *__restrict__ xcl,
                  const float *__restrict__ ycl, const SplitMean mean,
                  const float *__restrict__ sigx, const float *__restrict__ sigy,
                  const float *__restrict__ src, const double *__restrict__ stage_sin,
                  double alpha, double bdt, int stage)
{
    constexpr int NPL = 4 + NP;
    __shared__ alignas(128) float sq[NPL][kSH][kSW];
    // viscous: the halo tile of tau_xx', tau_xy', tau_yy', k dT'/dx, k dT'/dy
    __shared__ alignas(128) float sv[VISC ? 5 : 1][VISC ? kSH : 1][VISC ? kSW : 4];
    __shared__ alignas(8) unsigned long long tbar;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = blockIdx.x * kTX, j0 = blockIdx.y * kTY;
    const long long fplane = (long long)fpitch * d.jmax;
    const bool lead = (tx == 0 && ty == 0);
    // tile rows ly + kH +- 3 and columns tx + kTL +- 3 stay inside sq for
    // this launch shape; the box's x times 4 bytes is a multiple of 16
    NS_CHECK(err, kChkSplit, blockDim.x == kTX && blockDim.y == 8 && kTY % 8 == 0);
    NS_CHECK(err, kChkSplit, ((i0 - kTL) & 3) == 0 && fpitch >= d.imax && d.imax >= 7 &&
                                 d.jmax >= 7);
    if (lead) mbar_init(&tbar, 1);
    __syncthreads();
    if (lead) {
        // the box (40 x kSH x NPL floats) starts at (i0-4, j0-3, 0); points
        // outside the grid read as zero and are never used
        mbar_expect_tx(&tbar, (unsigned)(sizeof(sq) + (VISC ? sizeof(sv) : 0)));
        tma_load_3d(&sq[0][0][0], &qmap, i0 - kTL, j0 - kH, 0, &tbar);
        if (VISC) tma_load_3d(&sv[0][0][0], &vmap, i0 - kTL, j0 - kH, 0, &tbar);
    }
    // the FP64 accumulators of this thread's two points, requested before
    // the tile so that their latency overlaps the tile load
    double wold[kPT][4];
    if (!FIRST) {
#pragma unroll
        for (int h = 0; h < kPT; h++) {
            const int j = j0 + ty + 8 * h, i = i0 + tx;
            const bool ok = i < d.imax && j < d.jmax;
            const long long didx = (long long)j * d.pitch + i;
#pragma unroll
            for (int k = 0; k < 4; k++) wold[h][k] = ok ? W[k * d.plane + didx] : 0.0;
        }
    }
    if (!mbar_wait_bounded(&tbar, 0, err)) return;
    const int i = i0 + tx;
    if (i >= d.imax) return;
    const float *cxp = xc + kCoefStride * i;
    const float cx4 = cxp[4], cx5 = cxp[5], cx6 = cxp[6];
    // the FP64 coefficients minus their FP32 roundings: without them every
    // derivative is scaled by 1 + O(6e-8) and advection runs that much off
    const float *cxlp = xcl + kCoefStride * i;
    const float clx4 = cxlp[4], clx5 = cxlp[5], clx6 = cxlp[6];
    const bool xint = (i >= 3 && i < d.imax - 3);
#pragma unroll
    for (int h = 0; h < kPT; h++) {
        const int ly = ty + 8 * h;
        const int j = j0 + ly;
        if (j >= d.jmax) break;
        const long long fidx = (long long)j * fpitch + i;
        const long long didx = (long long)j * d.pitch + i;
        const int sr = ly + kH, sc = tx + kTL;
        float q[NPL], gx[NPL], gy[NPL];
        const float *cyp = yc + kCoefStride * j;
        const bool yint = (j >= 3 && j < d.jmax - 3);
        const float *cylp = ycl + kCoefStride * j;
        // With pairs, where the interior stencil applies in both directions
        // (such a point is interior too): du'/dx, dv'/dx and dv'/dy of the
        // hi planes in float-float (the differences exact, each coefficient
        // as hi + lo, the products exact, the sum compensated), for the
        // divergence and the base-flow advection below.
        const bool ffp = NP >= 2 && xint && yint;
        float uxh = 0.f, uxl = 0.f, vxh = 0.f, vxl = 0.f, vyh = 0.f, vyl = 0.f;
        if (ffp) {
            const float chx[3] = {cx4, cx5, cx6}, clx[3] = {clx4, clx5, clx6};
            const float chy[3] = {cyp[4], cyp[5], cyp[6]}, cly[3] = {cylp[4], cylp[5], cylp[6]};
            const float upx[3] = {sq[1][sr][sc + 1], sq[1][sr][sc + 2], sq[1][sr][sc + 3]};
            const float umx[3] = {sq[1][sr][sc - 1], sq[1][sr][sc - 2], sq[1][sr][sc - 3]};
            const float vpx[3] = {sq[2][sr][sc + 1], sq[2][sr][sc + 2], sq[2][sr][sc + 3]};
            const float vmx[3] = {sq[2][sr][sc - 1], sq[2][sr][sc - 2], sq[2][sr][sc - 3]};
            const float vpy[3] = {sq[2][sr + 1][sc], sq[2][sr + 2][sc], sq[2][sr + 3][sc]};
            const float vmy[3] = {sq[2][sr - 1][sc], sq[2][sr - 2][sc], sq[2][sr - 3][sc]};
            drp_ff(upx, umx, chx, clx, uxh, uxl);
            drp_ff(vpx, vmx, chx, clx, vxh, vxl);
            drp_ff(vpy, vmy, chy, cly, vyh, vyl);
        }
#pragma unroll
        for (int k = 0; k < NPL; k++) {
            q[k] = sq[k][sr][sc];
            if (ffp && (k == 1 || k == 2)) {
                gx[k] = k == 1 ? uxh + uxl : vxh + vxl;
            } else if (xint) {
                const float d1 = sq[k][sr][sc + 1] - sq[k][sr][sc - 1];
                const float d2 = sq[k][sr][sc + 2] - sq[k][sr][sc - 2];
                const float d3 = sq[k][sr][sc + 3] - sq[k][sr][sc - 3];
                float r = 0.f;
                if (k < 4) r = fmaf(clx6, d3, fmaf(clx5, d2, clx4 * d1));
                r = fmaf(cx4, d1, r);
                r = fmaf(cx5, d2, r);
                gx[k] = fmaf(cx6, d3, r);
            } else {
                gx[k] = closure_f32(qin + k * fplane + fidx, 1, i, d.imax, cxp);
            }
            if (ffp && k == 2) {
                gy[k] = vyh + vyl;
            } else if (yint) {
                const float d1 = sq[k][sr + 1][sc] - sq[k][sr - 1][sc];
                const float d2 = sq[k][sr + 2][sc] - sq[k][sr - 2][sc];
                const float d3 = sq[k][sr + 3][sc] - sq[k][sr - 3][sc];
                float r = 0.f;
                if (k < 4) r = fmaf(cylp[6], d3, fmaf(cylp[5], d2, cylp[4] * d1));
                r = fmaf(cyp[4], d1, r);
                r = fmaf(cyp[5], d2, r);
                gy[k] = fmaf(cyp[6], d3, r);
            } else {
                gy[k] = closure_f32(qin + k * fplane + fidx, fpitch, j, d.jmax, cyp);
            }
        }
        const bool interior = (i > 0) && (i < d.imax - 1) && (j > 0) && (j < d.jmax - 1);
        if (interior) {
            // Divergence du'/dx + dv'/dy, compensated where the interior
            // stencil applies: for a nearly steady solenoidal field its two
            // O(|u'|) terms cancel, and a plain FP32 rounding of them would
            // be the same every stage and drive p' coherently.
            float div;
            // U_b*du'/dx and U_b*dv'/dx (pairs only, interior stencil) as
            // float-float (ah + al): at a vortex advected by the base flow
            // these dominate the u' and v' right-hand sides, and their FP32
            // rounding, different every stage, was the larger part of the
            // error p' picks up there.
            float ah[3] = {0.f, 0.f, 0.f}, al[3] = {0.f, 0.f, 0.f};
            bool adv_ff = false;
            if (xint && yint) {
                float xh = uxh, xl = uxl, yh = vyh, yl = vyl, sh, se;
                if constexpr (NP < 2) {
                    // single FP32 perturbations: the divergence's own
                    // float-float derivatives
                    const float fpx[3] = {sq[1][sr][sc + 1], sq[1][sr][sc + 2], sq[1][sr][sc + 3]};
                    const float fmx[3] = {sq[1][sr][sc - 1], sq[1][sr][sc - 2], sq[1][sr][sc - 3]};
                    const float fpy[3] = {sq[2][sr + 1][sc], sq[2][sr + 2][sc], sq[2][sr + 3][sc]};
                    const float fmy[3] = {sq[2][sr - 1][sc], sq[2][sr - 2][sc], sq[2][sr - 3][sc]};
                    const float chx[3] = {cx4, cx5, cx6}, clx[3] = {clx4, clx5, clx6};
                    const float chy[3] = {cyp[4], cyp[5], cyp[6]},
                                cly[3] = {cylp[4], cylp[5], cylp[6]};
                    drp_ff(fpx, fmx, chx, clx, xh, xl);
                    drp_ff(fpy, fmy, chy, cly, yh, yl);
                }
                two_sum(xh, yh, sh, se);
                // the lo parts' derivatives are small: plain FP32 is exact enough
                div = sh + (se + (xl + yl));
                if constexpr (NP >= 2) {
                    div += gx[4] + gy[5];
                    // U_b (hi + lo) times d/dx of the hi plane (float-float)
                    // plus that of the lo plane, the product's rounding kept
                    const float ub = mean.u[j], ubl = mean.ulo[j];
                    ah[1] = ub * uxh;
                    al[1] = fmaf(ub, uxh, -ah[1]) + fmaf(ub, uxl + gx[4], ubl * uxh);
                    ah[2] = ub * vxh;
                    al[2] = fmaf(ub, vxh, -ah[2]) + fmaf(ub, vxl + gx[5], ubl * vxh);
                    adv_ff = true;
                }
            } else {
                div = gx[1] + gy[2];
                if (NP >= 2) div += gx[NP >= 2 ? 4 : 0] + gy[NP >= 2 ? 5 : 0];
            }
            // derivatives of the pair variables including their lo parts
#pragma unroll
            for (int k = 1; k <= NP; k++) {
                gx[k] += gx[k + 3];
                gy[k] += gy[k + 3];
            }
            // U = Ub + q'; dUb/dx = 0, v_b = 0, dp_b = 0 (eqeuler.f90:63-92, 1/Re = 0)
            const float rho = mean.rho[j] + q[0];
            const float uu = mean.u[j] + q[1];
            const float vv = q[2];
            const float pp = mean.p + q[3];
            const float rhoy = mean.drho[j] + gy[0];
            const float uy = mean.du[j] + gy[1];
            const float ri = 1.0f / rho;
            // r[k] + rl[k]: rl carries the float-float parts of u' and v'
            float r[4], rl[4] = {0.f, 0.f, 0.f, 0.f};
            // rho*du/dx + rho*dv/dy (eqeuler.f90:63) as rho*div
            float t = uu * gx[0];
            t = fmaf(vv, rhoy, t);
            t = fmaf(rho, div, t);
            r[0] = -t;
            if (adv_ff) {
                // the other terms (u' d/dx, pressure gradient, v' d/dy) in FP32,
                // summed with the advection pair
                float t1 = q[1] * gx[1];
                t1 = fmaf(ri, gx[3], t1);
                t1 = fmaf(vv, uy, t1);
                float t2 = q[1] * gx[2];
                t2 = fmaf(vv, gy[2], t2);
                t2 = fmaf(ri, gy[3], t2);
                float rh, re;
                two_sum(ah[1], al[1] + t1, rh, re);
                r[1] = -rh;
                rl[1] = -re;
                two_sum(ah[2], al[2] + t2, rh, re);
                r[2] = -rh;
                rl[2] = -re;
            } else {
                t = uu * gx[1];
                t = fmaf(ri, gx[3], t);
                t = fmaf(vv, uy, t);
                r[1] = -t;
                t = uu * gx[2];
                t = fmaf(vv, gy[2], t);
                t = fmaf(ri, gy[3], t);
                r[2] = -t;
            }
            // gamma*p*du/dx + gamma*p*dv/dy (eqeuler.f90:80-82) as gamma*p*div
            const float gp = mean.gamma * pp;
            t = uu * gx[3];
            t = fmaf(vv, gy[3], t);
            t = fmaf(gp, div, t);
            if (SRC) t = t - (float)stage_sin[stage] * src[fidx];
            r[3] = -t;
            if (VISC) {
                // eqeuler.f90:68-92: (1/(Re rho)) div tau for u and v,
                // (gamma-1)/Re * Phi + 1/(Re Pr) * div(k grad T) for p
                const long long vpl = fplane;
                auto dxy = [&](int a, int b) -> float {
                    float rx, ry;
                    if (xint) {
                        rx = cx4 * (sv[a][sr][sc + 1] - sv[a][sr][sc - 1]);
                        rx = fmaf(cx5, sv[a][sr][sc + 2] - sv[a][sr][sc - 2], rx);
                        rx = fmaf(cx6, sv[a][sr][sc + 3] - sv[a][sr][sc - 3], rx);
                    } else {
                        rx = closure_f32(tau + a * vpl + fidx, 1, i, d.imax, cxp);
                    }
                    if (yint) {
                        ry = cyp[4] * (sv[b][sr + 1][sc] - sv[b][sr - 1][sc]);
                        ry = fmaf(cyp[5], sv[b][sr + 2][sc] - sv[b][sr - 2][sc], ry);
                        ry = fmaf(cyp[6], sv[b][sr + 3][sc] - sv[b][sr - 3][sc], ry);
                    } else {
                        ry = closure_f32(tau + b * vpl + fidx, fpitch, j, d.jmax, cyp);
                    }
                    return rx + ry;
                };
                const float rv = vis.inv_re * ri;
                rl[1] = fmaf(rv, dxy(0, 1), rl[1]);
                rl[2] = fmaf(rv, dxy(1, 2), rl[2]);
                const float t0 = sv[0][sr][sc], t1 = sv[1][sr][sc], t2 = sv[2][sr][sc];
                float phi = gx[1] * t0;
                phi = fmaf(gx[2], t1, phi);
                phi = fmaf(gy[1], t1, phi);
                phi = fmaf(gy[2], t2, phi);
                r[3] = fmaf(vis.gm1_re, phi, r[3]);
                r[3] = fmaf(vis.inv_re_pr, dxy(3, 4), r[3]);
            }
            // rk_steep (rk.f90:163-164) with the FP64 accumulator carried as
            // w/dt: w~ = alpha*w~ + R, q' += (beta*dt)*w~ (bdt).  R enters FP64
            // exactly and dt only through the FP64 product beta*dt: an FP32
            // dt*R would advance every stage by FP32(dt), whose relative
            // error (up to 2^-24) shifts each wave's phase in proportion to
            // the time run.  u', v' kept as pairs.
#pragma unroll
            for (int k = 0; k < 4; k++) {
                double dr = f2d_exact(r[k]);
                if (NP >= 2 && (k == 1 || k == 2)) dr += f2d_exact(rl[k]);
                const double w = FIRST ? dr : fma(alpha, wold[h][k], dr);
                // stage 5's w is never read: stage 0 sets w~ = R
                if (stage < 5) W[k * d.plane + didx] = w;
                if (is_pair<NP>(k)) {
                    // hi + beta*dt*w~ in FP64, split exactly; the old lo joins in
                    // FP32 (both parts are below an FP32 ulp of hi)
                    float &lo = q[is_pair<NP>(k) ? k + 3 : k];
                    float hi, rem;
                    d2f_split(fma(bdt, w, f2d_exact(q[k])), hi, rem);
                    lo = rem + lo;
                    q[k] = hi;
                } else {
                    q[k] = d2f_rn(fma(bdt, w, f2d_exact(q[k])));
                }
            }
        }
        // bufferxy (rk.f90:77-151): U - Ub = q'
        auto damp = [&](float s) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (is_pair<NP>(k)) pair_scale(q[k], q[is_pair<NP>(k) ? k + 3 : k], s);
                else q[k] *= s;
            }
        };
        if (j < d.D || j >= d.jmax - d.D) damp(sigy[j]);
        if (i < d.D || i >= d.imax - d.D) damp(sigx[i]);
#pragma unroll
        for (int k = 0; k < NPL; k++) qout[k * fplane + fidx] = q[k];
    }
}

// ---------------------------------------------------------------------------
// FP32 filter recurrences (filtering.f90) over q'.  Same three passes and
// chunking as the FP64 kernel (ns_kernels.cu); here one warp stages its 32
// lines through shared memory so that every global access is coalesced.
// ---------------------------------------------------------------------------
// Filter coefficients for the FP32 sweeps, in forms that keep a constant
// field exactly constant: the 13-point filter as
//   v = u0 + sum_s m_s*((u_s - u0) + (u_-s - u0)),  m_s = -sigmaf*df(s)
// (its coefficients sum to 0 up to 3e-17, which is dropped), and the
// boundary filter as
//   v = u0 + sum_{s != 0} b_s*(u_s - u0) + bsum*u0,  bsum = -sigmaf*sum(dfb)
// with bsum the FP64 sum, which carries the reference's REAL(4) coefficient
// sum in y (-8.4e-9) and is ~1e-17 in x.  Rounding the coefficients to FP32
// then changes the filter's response only at nonzero wavenumbers; with the
// plain forms every application scaled the smooth part of q' by 1 + 3e-8.
struct FiltF {
    float m[7];      // m[s], s = 1..6
    float bm1, b[6]; // b(-1), b[s] s = 1..5
    float bsum;
};

// The second differences are formed as (u_s - u0) + (u_-s - u0): for a
// smooth field the two differences are exact (Sterbenz) and small, so the
// rounding is relative to the second difference, not to |u|; summing
// u_s + u_-s first would round at |u|*6e-8, the same pattern every
// application for a steady structure such as a vortex.
__device__ __forceinline__ float pass2_f(const float *w, const FiltF &f)
{
    const float u0 = w[6];
    float acc = f.m[6] * ((w[12] - u0) + (w[0] - u0));
    acc = fmaf(f.m[5], (w[11] - u0) + (w[1] - u0), acc);
    acc = fmaf(f.m[4], (w[10] - u0) + (w[2] - u0), acc);
    acc = fmaf(f.m[3], (w[9] - u0) + (w[3] - u0), acc);
    acc = fmaf(f.m[2], (w[8] - u0) + (w[4] - u0), acc);
    acc = fmaf(f.m[1], w[7] - u0, acc);
    return fmaf(f.m[1], w[5] - u0, u0 + acc);
}

// Boundary filter at window position p: neighbours p-1 (newest) and
// p+1..p+5 (pass 1), or mirrored (pass 3, dir = -1).
template <int DIR>
__device__ __forceinline__ float passb_f(const float *w, int p, const FiltF &f)
{
    const float u0 = w[p];
    float acc = f.bsum * u0;
#pragma unroll
    for (int z = 1; z <= 5; z++) acc = fmaf(f.b[z], w[p + DIR * z] - u0, acc);
    return fmaf(f.bm1, w[p - DIR] - u0, u0 + acc);
}

// The same two forms on hi + lo pairs (u', v'): the differences are
// (h_s - h_0) + (l_s - l_0), the correction acc is FP32 (it is small), and
// the result (h_0 + l_0) + acc is renormalised into a pair.
__device__ __forceinline__ void pass2_p(const float *wh, const float *wl, const FiltF &f,
                                        float &oh, float &ol)
{
    const float h0 = wh[6], l0 = wl[6];
#define NS_DD(t) ((wh[t] - h0) + (wl[t] - l0))
    float acc = f.m[6] * (NS_DD(12) + NS_DD(0));
    acc = fmaf(f.m[5], NS_DD(11) + NS_DD(1), acc);
    acc = fmaf(f.m[4], NS_DD(10) + NS_DD(2), acc);
    acc = fmaf(f.m[3], NS_DD(9) + NS_DD(3), acc);
    acc = fmaf(f.m[2], NS_DD(8) + NS_DD(4), acc);
    acc = fmaf(f.m[1], NS_DD(7), acc);
    acc = fmaf(f.m[1], NS_DD(5), acc);
#undef NS_DD
    oh = h0;
    ol = l0;
    pair_add(oh, ol, acc);
}

template <int DIR>
__device__ __forceinline__ void passb_p(const float *wh, const float *wl, int p, const FiltF &f,
                                        float &oh, float &ol)
{
    const float h0 = wh[p], l0 = wl[p];
    float acc = fmaf(f.bsum, l0, f.bsum * h0);
#pragma unroll
    for (int z = 1; z <= 5; z++)
        acc = fmaf(f.b[z], (wh[p + DIR * z] - h0) + (wl[p + DIR * z] - l0), acc);
    acc = fmaf(f.bm1, (wh[p - DIR] - h0) + (wl[p - DIR] - l0), acc);
    oh = h0;
    ol = l0;
    pair_add(oh, ol, acc);
}

// One filter line along y (stride st) of a single FP32 variable (PAIR =
// false) or of a hi/lo pair (lo at sl).  Steps a .. b-1 of pass 2 with the
// chunking of the FP64 kernel; cr: the FP64 action on the base flow, added
// to every output.
template <bool PAIR>
__device__ __forceinline__ void filter_y_line(const float *__restrict__ s,
                                              const float *__restrict__ sl, float *__restrict__ o,
                                              float *__restrict__ ol, long long st, int n, int a,
                                              int b, bool first, bool last, int q0, const FiltF &f,
                                              const float *__restrict__ cr)
{
    float wh[13], wl[13];
    auto put = [&](int pos, float h, float l) {
        if (PAIR) {
            pair_add(h, l, cr[pos]);
            o[(long long)pos * st] = h;
            ol[(long long)pos * st] = l;
        } else {
            o[(long long)pos * st] = h + cr[pos];
        }
    };
#pragma unroll
    for (int t = 0; t < 13; t++) {
        wh[t] = s[(long long)(q0 - 6 + t) * st];
        wl[t] = PAIR ? sl[(long long)(q0 - 6 + t) * st] : 0.f;
    }
    int q = q0;
    if (first) {
        // pass 1 from the true line start (q0 = 6)
#pragma unroll
        for (int p = 1; p <= 6; p++) {
            if (PAIR) passb_p<1>(wh, wl, p, f, wh[p], wl[p]);
            else wh[p] = passb_f<1>(wh, p, f);
        }
        if (a == 6) {
#pragma unroll
            for (int p = 0; p < 6; p++) put(p, wh[p], wl[p]);
        }
    }
    // loads run eight steps ahead through a register ring (static indices by
    // unrolling); the value appended at step q is position q+7
    float ph[8], pl[8];
#pragma unroll
    for (int t = 0; t < 8; t++) {
        const bool ok = q + 7 + t < n;
        ph[t] = ok ? s[(long long)(q + 7 + t) * st] : 0.f;
        pl[t] = (PAIR && ok) ? sl[(long long)(q + 7 + t) * st] : 0.f;
    }
    auto step = [&](int qq, float nh, float nl) {
        float vh, vl = 0.f;
        if (PAIR) pass2_p(wh, wl, f, vh, vl);
        else vh = pass2_f(wh, f);
        if (qq >= a) put(qq, vh, vl);
#pragma unroll
        for (int u = 0; u < 5; u++) {
            wh[u] = wh[u + 1];
            wl[u] = wl[u + 1];
        }
        wh[5] = vh;
        wl[5] = vl;
#pragma unroll
        for (int u = 6; u < 12; u++) {
            wh[u] = wh[u + 1];
            wl[u] = wl[u + 1];
        }
        wh[12] = nh;
        wl[12] = nl;
    };
    for (; q + 8 <= b; q += 8) {
#pragma unroll
        for (int t = 0; t < 8; t++) {
            const int qq = q + t;
            step(qq, ph[t], pl[t]);
            const bool ok = qq + 15 < n;
            ph[t] = ok ? s[(long long)(qq + 15) * st] : 0.f;
            pl[t] = (PAIR && ok) ? sl[(long long)(qq + 15) * st] : 0.f;
        }
    }
    for (; q < b; q++) {
        const bool ok = q + 7 < n;
        step(q, ok ? s[(long long)(q + 7) * st] : 0.f,
             (PAIR && ok) ? sl[(long long)(q + 7) * st] : 0.f);
    }
    if (last) {
        // pass 3: w[0..11] = positions n-12 .. n-1
#pragma unroll
        for (int x = 10; x >= 5; x--) {
            if (PAIR) passb_p<-1>(wh, wl, x, f, wh[x], wl[x]);
            else wh[x] = passb_f<-1>(wh, x, f);
        }
#pragma unroll
        for (int x = 5; x < 12; x++) put(n - 12 + x, wh[x], wl[x]);
    }
}

// y filter: thread per (column, variable, chunk); lanes on consecutive
// columns, so each step reads and writes one coalesced row segment.
// corr[k*jmax + j] is the FP64 action of the filter on the base flow.
template <int NP>
__global__ void __launch_bounds__(128)
    k_split_filter_y(Dims d, int fpitch, const float *__restrict__ src, float *__restrict__ dst,
                     int chunks, int warm, FiltF f, const float *__restrict__ corr, int *err)
{
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)d.imax * 4 * chunks;
    if (gid >= total) return;
    const int line = (int)(gid % d.imax);
    const int rest = (int)(gid / d.imax);
    const int k = rest % 4, c = rest / 4;
    const int n = d.jmax;
    const long long st = fpitch, fplane = (long long)fpitch * d.jmax;
    const long long base = (long long)k * fplane + line;
    const long long lbase = (long long)(k + 3) * fplane + line;  // lo plane of a pair
    const int len2 = n - 12;
    const int a = 6 + (int)(((long long)c * len2) / chunks);
    const int b = 6 + (int)(((long long)(c + 1) * len2) / chunks);
    const bool exact = (c == 0 || warm < 0 || a - warm <= 6);
    const int q0 = exact ? 6 : a - warm;
    // reads q0-6 .. (ahead, guarded) n-1; writes a .. b-1 and the line ends
    NS_CHECK(err, kChkSplit, k < 4 && c < chunks && n >= 13 && 6 <= a && a <= b && b <= n - 6 &&
                                 q0 >= 6 && q0 <= a);
    const float *cr = corr + (long long)k * d.jmax;
    if (is_pair<NP>(k))
        filter_y_line<true>(src + base, src + lbase, dst + base, dst + lbase, st, n, a, b, exact,
                            c == chunks - 1, q0, f, cr);
    else
        filter_y_line<false>(src + base, nullptr, dst + base, nullptr, st, n, a, b, exact,
                             c == chunks - 1, q0, f, cr);
}

// x filter: each warp owns 32 consecutive rows of one variable and one
// chunk.  The old values a lane appends to its window (position q+7 at step
// q) are staged kSplitXB positions at a time through [32][kSplitXB+1] tiles
// (an odd row stride: column reads are free of bank conflicts): lane x
// copies position q+7+x of each row with cp.async (no registers, no wait),
// the next block's copies issued before the current block is filtered (two
// tiles per plane).  Step t reads column t of its own row and leaves its
// output there; the tile then goes back with coalesced row writes.  Pair
// variables stage their lo parts through a second tile pair.  The tiles set
// the shared memory per warp and with it the resident warps.  Measured on
// 4096^2: blocks of 32 positions for pairs (0.38 ms; 24: 0.41, 16: 0.44) and
// 24 for single FP32 variables (0.18 ms; 32: 0.20, 16: 0.22).
template <int NP>
constexpr int x_block()
{
    return NP ? 32 : 24;
}
// warps per block: 4 for single FP32 variables, 2 when the lo tiles exist
template <int NP>
constexpr int x_warps()
{
    return NP ? 2 : 4;
}

__device__ __forceinline__ void cp_async4(float *dst, const float *src, int src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_addr(dst)),
                 "l"(src), "r"(src_bytes)
                 : "memory");
}

__device__ __forceinline__ void cp_async_commit()
{
    asm volatile("cp.async.commit_group;" ::: "memory");
}

template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <bool PAIR, int XB>
__device__ __forceinline__ void filter_x_rows(const float *__restrict__ sbase,
                                              const float *__restrict__ slbase,
                                              float *__restrict__ obase, float *__restrict__ olbase,
                                              int fpitch, int n, int nrows, int lane, int a, int b,
                                              bool exact, bool first, bool last, int q0,
                                              const FiltF &f, float (*ti)[32][XB + 1],
                                              float (*til)[32][XB + 1])
{
    const bool active = lane < nrows;
    const long long roff = (long long)(active ? lane : 0) * fpitch;
    const float *__restrict__ s = sbase + roff;
    const float *__restrict__ sl = PAIR ? slbase + roff : nullptr;
    // copies of block qb (appended positions qb+7 ..) into tile set `buf`;
    // positions past the row end are zero-filled (0 source bytes)
    auto issue = [&](int buf, int qb) {
        const int pos = qb + 7 + lane;
        const int nb = pos < n ? 4 : 0;
        const int pc = pos < n ? pos : 0;
        if (lane < XB)
            for (int r = 0; r < nrows; r++) {
                cp_async4(&ti[buf][r][lane], sbase + (long long)r * fpitch + pc, nb);
                if (PAIR) cp_async4(&til[buf][r][lane], slbase + (long long)r * fpitch + pc, nb);
            }
        cp_async_commit();
    };
    if (q0 < b) issue(0, q0);
    float wh[13], wl[13];
#pragma unroll
    for (int t = 0; t < 13; t++) {
        wh[t] = s[q0 - 6 + t];
        wl[t] = PAIR ? sl[q0 - 6 + t] : 0.f;
    }
    if (exact) {
#pragma unroll
        for (int p = 1; p <= 6; p++) {
            if (PAIR) passb_p<1>(wh, wl, p, f, wh[p], wl[p]);
            else wh[p] = passb_f<1>(wh, p, f);
        }
        if (first && active)
            for (int p = 0; p < 6; p++) {
                obase[(long long)lane * fpitch + p] = wh[p];
                if (PAIR) olbase[(long long)lane * fpitch + p] = wl[p];
            }
    }
    // Steps q = q0 .. b-1 in blocks of XB: block B covers steps
    // [q0+XB*B, q0+XB*B+XB), appends positions q+7, writes outputs at q.
    int buf = 0;
    for (int qb = q0; qb < b; qb += XB) {
        const bool more = qb + XB < b;
        if (more) {
            issue(buf ^ 1, qb + XB);
            cp_async_wait<1>();  // this block's copies have landed
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();
        const int nstep = min(XB, b - qb);
        float(*tb)[XB + 1] = ti[buf];
        float(*tbl)[XB + 1] = til[PAIR ? buf : 0];
        // one step: output q into the tile column it read, window slides
        auto step = [&](int t) {
            float vh, vl = 0.f;
            if (PAIR) pass2_p(wh, wl, f, vh, vl);
            else vh = pass2_f(wh, f);
            const float nh = tb[lane][t];
            const float nl = PAIR ? tbl[lane][t] : 0.f;
            tb[lane][t] = vh;
            if (PAIR) tbl[lane][t] = vl;
#pragma unroll
            for (int u = 0; u < 5; u++) {
                wh[u] = wh[u + 1];
                wl[u] = wl[u + 1];
            }
            wh[5] = vh;
            wl[5] = vl;
#pragma unroll
            for (int u = 6; u < 12; u++) {
                wh[u] = wh[u + 1];
                wl[u] = wl[u + 1];
            }
            wh[12] = nh;
            wl[12] = nl;
        };
        for (int t = 0; t < nstep; t++) step(t);
        __syncwarp();
        // write outputs q = qb .. qb+nstep-1 that this chunk owns (q >= a)
        for (int r = 0; r < nrows; r++) {
            const int qq = qb + lane;
            if (lane < nstep && qq >= a) {
                obase[(long long)r * fpitch + qq] = tb[r][lane];
                if (PAIR) olbase[(long long)r * fpitch + qq] = tbl[r][lane];
            }
        }
        __syncwarp();
        buf ^= 1;
    }
    if (last && active) {
        // w[0..11] = positions n-12 .. n-1 (pass 3)
#pragma unroll
        for (int x = 10; x >= 5; x--) {
            if (PAIR) passb_p<-1>(wh, wl, x, f, wh[x], wl[x]);
            else wh[x] = passb_f<-1>(wh, x, f);
        }
        for (int x = 5; x < 12; x++) {
            obase[(long long)lane * fpitch + (n - 12 + x)] = wh[x];
            if (PAIR) olbase[(long long)lane * fpitch + (n - 12 + x)] = wl[x];
        }
    }
}

template <int NP>
__device__ __forceinline__ void split_filter_x_body(Dims d, int fpitch, const float *__restrict__ src,
                                                    float *__restrict__ dst, int chunks, int warm,
                                                    const FiltF &f, int *err)
{
    constexpr int kXW = x_warps<NP>();
    constexpr int kXL = NP ? kXW : 1;  // lo tiles only when pairs exist
    constexpr int XB = x_block<NP>();
    __shared__ float tin[kXW][2][32][XB + 1];
    __shared__ float tinl[kXL][2][32][XB + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int rows32 = (d.jmax + 31) / 32;
    const long long gw = (long long)blockIdx.x * kXW + wid;  // global warp
    const long long nw = (long long)rows32 * 4 * chunks;
    if (gw >= nw) return;                                       // whole warp exits together
    const int rg = (int)(gw % rows32);
    const int rest = (int)(gw / rows32);
    const int k = rest % 4, c = rest / 4;
    const int n = d.imax;
    const int row0 = rg * 32;
    const int nrows = min(32, d.jmax - row0);
    const long long fplane = (long long)fpitch * d.jmax;
    const long long roff = (long long)row0 * fpitch;
    const int len2 = n - 12;
    const int a = 6 + (int)(((long long)c * len2) / chunks);
    const int b = 6 + (int)(((long long)(c + 1) * len2) / chunks);
    const bool exact = (c == 0 || warm < 0 || a - warm <= 6);
    const int q0 = exact ? 6 : a - warm;
    // a warp's rows row0 .. row0+nrows-1 (1..32, the tile's rows), its
    // positions q0-6 .. n-1 (staged copies of positions >= n are zero-size)
    NS_CHECK(err, kChkSplit, blockDim.x == 32 * kXW && k < 4 && c < chunks && nrows >= 1 &&
                                 nrows <= 32 && row0 + nrows <= d.jmax);
    NS_CHECK(err, kChkSplit, n >= 13 && 6 <= a && a <= b && b <= n - 6 && q0 >= 6 && q0 <= a &&
                                 fpitch >= n);
    if (is_pair<NP>(k))
        filter_x_rows<true, XB>(src + k * fplane + roff, src + (k + 3) * fplane + roff,
                            dst + k * fplane + roff, dst + (k + 3) * fplane + roff, fpitch, n,
                            nrows, lane, a, b, exact, c == 0, c == chunks - 1, q0, f, tin[wid],
                            tinl[NP ? wid : 0]);
    else
        filter_x_rows<false, XB>(src + k * fplane + roff, nullptr, dst + k * fplane + roff, nullptr,
                             fpitch, n, nrows, lane, a, b, exact, c == 0, c == chunks - 1, q0, f,
                             tin[wid], tinl[0]);
}

// Register budgets measured best: the all-FP32 variant at one block per SM
// minimum (96 registers), the pair variant left to the compiler (111).
__global__ void __launch_bounds__(32 * x_warps<0>(), 1)
    k_split_filter_x_single(Dims d, int fpitch, const float *__restrict__ src,
                            float *__restrict__ dst, int chunks, int warm, FiltF f, int *err)
{
    split_filter_x_body<0>(d, fpitch, src, dst, chunks, warm, f, err);
}

__global__ void __launch_bounds__(32 * x_warps<3>())
    k_split_filter_x_pairs(Dims d, int fpitch, const float *__restrict__ src,
                           float *__restrict__ dst, int chunks, int warm, FiltF f, int *err)
{
    split_filter_x_body<3>(d, fpitch, src, dst, chunks, warm, f, err);
}

// ---------------------------------------------------------------------------
// ccpml (cc.f90:6-68) on q': rho'(1,j) = rhob(j) - rho_b(j), v' = 0,
// p' = 1/gamma - p_b on every edge; extrapolations are the same in q'.  The
// perimeter is small, so values are combined in FP64 (u', v' as hi + lo).
// ---------------------------------------------------------------------------
template <int NP>
__device__ __forceinline__ double bc_get(const float *q, long long P, int k, long long idx)
{
    double v = (double)q[k * P + idx];
    if (is_pair<NP>(k)) v += (double)q[(k + 3) * P + idx];
    return v;
}

template <int NP>
__device__ __forceinline__ void bc_put(float *q, long long P, int k, long long idx, double v)
{
    const float h = (float)v;
    q[k * P + idx] = h;
    if (is_pair<NP>(k)) q[(k + 3) * P + idx] = (float)(v - (double)h);
}

template <int NP>
__global__ void k_split_bc(Dims d, int fpitch, float *__restrict__ q,
                           const float *__restrict__ rho_bc, double p_bc)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const long long P = (long long)fpitch * d.jmax;
    auto colval = [&](int i, int j, double *v) {
        const long long r = (long long)j * fpitch;
        if (i == 0) {
            v[0] = rho_bc[j];
            v[1] = 2.0 * bc_get<NP>(q, P, 1, r + 1) - bc_get<NP>(q, P, 1, r + 2);
            v[2] = 0.0;
            v[3] = p_bc;
        } else {
            const int a = d.imax - 2, b = d.imax - 3;
            for (int k = 0; k < 3; k++) v[k] = 2.0 * bc_get<NP>(q, P, k, r + a) - bc_get<NP>(q, P, k, r + b);
            v[3] = p_bc;
        }
    };
    double v[4];
    if (t > 0 && t < d.jmax - 1) {
        const long long r = (long long)t * fpitch;
        colval(0, t, v);
        for (int k = 0; k < 4; k++) bc_put<NP>(q, P, k, r, v[k]);
        colval(d.imax - 1, t, v);
        for (int k = 0; k < 4; k++) bc_put<NP>(q, P, k, r + d.imax - 1, v[k]);
    }
    if (t < d.imax) {
        const int jt = d.jmax - 1;
        double a[4], b[4];
        if (t == 0 || t == d.imax - 1) {
            colval(t, jt - 1, a);
            colval(t, jt - 2, b);
        } else {
            for (int k = 0; k < 4; k++) {
                a[k] = bc_get<NP>(q, P, k, (long long)(jt - 1) * fpitch + t);
                b[k] = bc_get<NP>(q, P, k, (long long)(jt - 2) * fpitch + t);
            }
        }
        for (int k = 0; k < 3; k++) bc_put<NP>(q, P, k, (long long)jt * fpitch + t, 2.0 * a[k] - b[k]);
        bc_put<NP>(q, P, 3, (long long)jt * fpitch + t, p_bc);
        if (t == 0 || t == d.imax - 1) {
            colval(t, 1, a);
            colval(t, 2, b);
        } else {
            for (int k = 0; k < 4; k++) {
                a[k] = bc_get<NP>(q, P, k, (long long)1 * fpitch + t);
                b[k] = bc_get<NP>(q, P, k, (long long)2 * fpitch + t);
            }
        }
        for (int k = 0; k < 3; k++) bc_put<NP>(q, P, k, t, 2.0 * a[k] - b[k]);
        bc_put<NP>(q, P, 3, t, p_bc);
    }
}

// State conversion: q' = U - Ub (pairs as hi + lo) and U = Ub + q'.
template <int NP>
__global__ void k_split_from_full(Dims d, int fpitch, const double *__restrict__ U,
                                  const double *__restrict__ Ub, float *__restrict__ q)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= d.imax || j >= d.jmax) return;
    const long long P = (long long)fpitch * d.jmax, fi = (long long)j * fpitch + i;
    for (int k = 0; k < 4; k++) {
        const long long di = k * d.plane + (long long)j * d.pitch + i;
        bc_put<NP>(q, P, k, fi, U[di] - Ub[di]);
    }
}

template <int NP>
__global__ void k_split_to_full(Dims d, int fpitch, const float *__restrict__ q,
                                const double *__restrict__ Ub, double *__restrict__ U)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= d.imax || j >= d.jmax) return;
    const long long P = (long long)fpitch * d.jmax, fi = (long long)j * fpitch + i;
    for (int k = 0; k < 4; k++) {
        const long long di = k * d.plane + (long long)j * d.pitch + i;
        U[di] = Ub[di] + bc_get<NP>(q, P, k, fi);
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
static FiltF to_f32(const FilterCoef &c)
{
    // FilterCoef holds m[s] = -sigmaf*df(s), bm1 = -sigmaf*dfb(-1),
    // b[s] = -sigmaf*dfb(s) and b0 = 1 - sigmaf*dfb(0) (ns_api.cu)
    FiltF f;
    for (int s = 0; s < 7; s++) f.m[s] = (float)c.m[s];
    f.bm1 = (float)c.bm1;
    double sum = c.bm1 + (c.b0 - 1.0);
    for (int s = 0; s < 6; s++) {
        f.b[s] = (float)c.b[s];
        if (s >= 1) sum += c.b[s];
    }
    f.bsum = (float)sum;
    return f;
}

template <int NP>
static cudaError_t launch_split_np(ns_ctx *c, int cls, int stage, cudaStream_t s)
{
    const Dims &d = c->d;
    SplitState &sp = c->sp;
    // buffer roles alternate every stage; a step has six stages, so the
    // roles at the start of every step are the same
    float *qa = sp.q[stage & 1], *qb = sp.q[(stage + 1) & 1];
    switch (cls) {
    case NS_KC_SPLIT_STAGE: {
        const dim3 blk(kTX, 8), grd((d.imax + kTX - 1) / kTX, (d.jmax + kTY - 1) / kTY);
        const bool src = sp.src != nullptr;
#define NS_SPL(FIRST, SRC, VISC)                                                                \
    k_split_stage<NP, FIRST, SRC, VISC><<<grd, blk, 0, s>>>(                                    \
        sp.qmap[stage & 1], sp.vmap, sp.tau, sp.trf, sp.vis, c->d_err, d, sp.fpitch, qa, qb,    \
        c->W, sp.xc, sp.yc, sp.xcl, sp.ycl, sp.mean, sp.sigx, sp.sigy, sp.src, c->stage_sin,    \
        c->alpha[stage], c->beta[stage] * c->p.dt, stage)
#define NS_SPL2(VISC)                                                                           \
    if (stage == 0) {                                                                           \
        if (src) NS_SPL(true, true, VISC); else NS_SPL(true, false, VISC);                      \
    } else {                                                                                    \
        if (src) NS_SPL(false, true, VISC); else NS_SPL(false, false, VISC);                    \
    }
        if (c->visc) {
            NS_SPL2(true)
        } else {
            NS_SPL2(false)
        }
#undef NS_SPL2
#undef NS_SPL
        break;
    }
    case NS_KC_SPLIT_VISC: {
        const dim3 blk(kTX, 8), grd((d.imax + kTX - 1) / kTX, (d.jmax + kTY - 1) / kTY);
        k_split_visc<NP><<<grd, blk, 0, s>>>(sp.qmap[stage & 1], c->d_err, d, sp.fpitch, qa,
                                             sp.tau, sp.xc, sp.yc, sp.trf, sp.vis);
        break;
    }
    case NS_KC_SPLIT_FX: {
        const long long warps = (long long)((d.jmax + 31) / 32) * 4 * sp.fx_chunks;
        constexpr int kXW = x_warps<NP>();
        const unsigned nb = (unsigned)((warps + kXW - 1) / kXW);
        if (NP)
            k_split_filter_x_pairs<<<nb, 32 * kXW, 0, s>>>(d, sp.fpitch, qb, qa, sp.fx_chunks,
                                                           sp.warm, to_f32(c->fx), c->d_err);
        else
            k_split_filter_x_single<<<nb, 32 * kXW, 0, s>>>(d, sp.fpitch, qb, qa, sp.fx_chunks,
                                                            sp.warm, to_f32(c->fx), c->d_err);
        break;
    }
    case NS_KC_SPLIT_FY: {
        const long long t = (long long)d.imax * 4 * sp.fy_chunks;
        k_split_filter_y<NP><<<(unsigned)((t + 127) / 128), 128, 0, s>>>(
            d, sp.fpitch, qa, qb, sp.fy_chunks, sp.warm, to_f32(c->fy), sp.ycorr, c->d_err);
        break;
    }
    case NS_KC_SPLIT_BC: {
        const int nt = d.imax > d.jmax ? d.imax : d.jmax;
        k_split_bc<NP><<<(nt + 127) / 128, 128, 0, s>>>(d, sp.fpitch, qb, sp.rho_bc, sp.p_bc);
        break;
    }
    default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_split_kernel(ns_ctx *c, int cls, int stage, cudaStream_t s)
{
    return c->sp.np == 3 ? launch_split_np<3>(c, cls, stage, s)
                         : launch_split_np<0>(c, cls, stage, s);
}

cudaError_t launch_split_from_full(ns_ctx *c, const double *U, cudaStream_t s)
{
    const dim3 blk(32, 8), grd((c->d.imax + 31) / 32, (c->d.jmax + 7) / 8);
    if (c->sp.np == 3)
        k_split_from_full<3><<<grd, blk, 0, s>>>(c->d, c->sp.fpitch, U, c->Ubase, c->sp.q[0]);
    else
        k_split_from_full<0><<<grd, blk, 0, s>>>(c->d, c->sp.fpitch, U, c->Ubase, c->sp.q[0]);
    return cudaGetLastError();
}

cudaError_t launch_split_to_full(ns_ctx *c, double *U, cudaStream_t s)
{
    const dim3 blk(32, 8), grd((c->d.imax + 31) / 32, (c->d.jmax + 7) / 8);
    if (c->sp.np == 3)
        k_split_to_full<3><<<grd, blk, 0, s>>>(c->d, c->sp.fpitch, c->sp.q[0], c->Ubase, U);
    else
        k_split_to_full<0><<<grd, blk, 0, s>>>(c->d, c->sp.fpitch, c->sp.q[0], c->Ubase, U);
    return cudaGetLastError();
}

}  // namespace ns
