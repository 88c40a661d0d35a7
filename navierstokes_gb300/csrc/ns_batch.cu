// ns_batch.cu -- many independent instances of the time step in one
// persistent launch per step.
//
// A parameter sweep advances dozens of uneven-size Euler grids (each one a
// complete rk_euler, rk.f90:12-75, with its own size, source, mean flow and
// time step).  One cooperative, persistent kernel per step runs the six
// stages; each stage has four phases over a work list that spans every
// instance:
//   A  tiles:   FP32/FP64 derivatives from a shared-memory tile, Euler RHS,
//               FP64 LDDRK update, buffer                (rk.f90:52-64)
//   B  x lines: lddfilterx                                (filtering.f90:9-96)
//   C  y lines: lddfiltery                                (filtering.f90:98-190)
//   D  edges:   ccpml                                     (cc.f90:6-68)
// separated by grid-wide barriers.  Every barrier wait is bounded: a block
// that waits too long sets an error word and returns, the others see the
// word and return too, and the host reports NS_ERR_TIMEOUT.
//
// Each instance is written as U = Ub + q' with Ub its base flow (uniform in
// x, v = 0, uniform p); T = float stores q' in FP32 (split precision),
// T = double in FP64.  The arithmetic is that of the single-grid split path
// (ns_split.cu), instance by instance.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "ns_check.cuh"
#include "ns_coef.h"
#include "ns_f32conv.cuh"
#include "ns_internal.cuh"
#include "ns_tma.cuh"

namespace ns {
namespace batch {

struct Inst {
    int imax, jmax, pitch, D;  // pitch in elements of T and of W
    long long q_off;           // plane 0 of the instance in q[0], q[1]
    long long w_off;           // plane 0 in W (FP64)
    long long s_off;           // source field (-1: none)
    int x_off, y_off;          // per-column / per-row table offsets
    int fx_chunks, fy_chunks, warm;
    float dt_f, pmean_f, gamma_f, p_bc_f;
    double dt_d, pmean_d, gamma_d, p_bc_d;
};

struct Args {
    const Inst *inst;
    const int4 *tiles, *fx, *fy;
    const int2 *bc;            // edge items: (instance, first of 32 positions)
    // TMA maps of every instance's halo tile: [(ty16 * n + inst) * 2 + buf],
    // buf 0 for q0 and 1 for q1; box 40 x (TY + 6) x 4 planes
    int ntiles, nfx, nfy, nbc;
    int ninst;                 // instances (the bound of every item's .x)
    const CUtensorMap *qmaps;
    void *q0, *q1;             // T*
    double *W;
    // tables in the state's precision T (xcl, ycl: FP32 low parts, split only)
    const void *xc, *yc, *sigx, *sigy, *rho_bc, *mrho, *mu, *mdrho, *mdu, *corr;
    const float *xcl, *ycl;
    const void *src;           // T*
    const double *stage_sin;   // [inst][8]
    const double *bdt;         // [inst][6]: beta_k * dt, the FP32 instances' update factor
    double alpha[6], beta[6];
    // filter coefficients ([0] = x, [1] = y) in both precisions
    float fm_f[7], fbm1_f[2], fb_f[2][6], fbsum_f[2];
    double fm_d[7], fbm1_d[2], fb_d[2][6], fbsum_d[2];
    unsigned *bar_count, *bar_gen;
    unsigned *work;            // per stage: next x-line item, next y-line item
    int *err;
    unsigned nblocks;          // blocks that take part in each barrier
    long long spin_limit;
    // phase timing (ns_batch_phase_times): block 0 records the global timer
    // at the start and after every barrier (1 + 6*4 stamps); null otherwise
    unsigned long long *stamps;
};

// Tiles of kTX x TY points; their halo box spans kTL columns to the left
// (the TMA box's x times the element size must be a multiple of 16 bytes,
// so 4 columns for FP32 and FP64 alike) and kH rows above and below.
constexpr int kTX = 32, kH = 3, kTL = 4, kWarps = 8;

template <typename T>
__device__ __forceinline__ T pick(float f, double d);
template <>
__device__ __forceinline__ float pick<float>(float f, double) { return f; }
template <>
__device__ __forceinline__ double pick<double>(float, double d) { return d; }

template <typename T>
__device__ __forceinline__ const T *tab(const void *p) { return static_cast<const T *>(p); }

template <typename T>
__device__ __forceinline__ double to_d(T x);
template <>
__device__ __forceinline__ double to_d<double>(double x) { return x; }

template <>
__device__ __forceinline__ double to_d<float>(float x) { return f2d_exact(x); }

template <typename T>
__device__ __forceinline__ T from_d(double x);
template <>
__device__ __forceinline__ double from_d<double>(double x) { return x; }
template <>
__device__ __forceinline__ float from_d<float>(double x) { return d2f_rn(x); }

// Grid-wide barrier with a bounded wait.  Returns false when this or another
// block gave up (the error word is set), after which callers return.
__device__ __forceinline__ bool grid_barrier(const Args &a)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = (*(volatile int *)a.err == 0);
        if (ok) {
            const unsigned g = *(volatile unsigned *)a.bar_gen;
            __threadfence();
            if (atomicAdd(a.bar_count, 1u) == a.nblocks - 1u) {
                atomicExch(a.bar_count, 0u);
                __threadfence();
                atomicAdd(a.bar_gen, 1u);
            } else {
                long long spins = 0;
                while (*(volatile unsigned *)a.bar_gen == g) {
                    if (*(volatile int *)a.err != 0) { ok = 0; break; }
                    if (++spins > a.spin_limit) {
                        atomicCAS(a.err, 0, 1);  // the first failure recorded wins
                        ok = 0;
                        break;
                    }
                    __nanosleep(64);
                }
            }
            __threadfence();
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// ---------------------------------------------------------------------------
// Phase A: one tile of one instance.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// The state buffers are written by other phases of the same launch, so they
// are read through plain (coherent) loads: no __restrict__ / read-only path.
template <int TY>
constexpr int tile_sw()
{
    return kTX + 8;  // columns i0-4 .. i0+35
}
template <int TY>
constexpr int tile_sh()
{
    return TY + 2 * kH;
}

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

// One element global -> shared without registers; 0 source bytes fill zeros.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T *dst, const T *src, bool ok)
{
    const int nb = ok ? (int)sizeof(T) : 0;
    if constexpr (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_u32(dst)), "l"(src),
                     "r"(nb)
                     : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src),
                     "r"(nb)
                     : "memory");
}

// The halo tile of `item` (4 planes, SH x SW, from (i0-4, j0-3)) into sqbuf
// by one TMA load, counted by bar; points outside the instance read as zero.
// Issued by thread 0.
template <typename T, int TY>
__device__ void tile_issue(const Args &a, int4 item, int which, T *sqbuf,
                           unsigned long long *bar)
{
    constexpr int SW = tile_sw<TY>(), SH = tile_sh<TY>();
    NS_CHECK(a.err, kChkBatch, item.x >= 0 && item.x < a.ninst && item.y % kTX == 0 &&
                                   ((item.y - kTL) * (int)sizeof(T)) % 16 == 0);
    const CUtensorMap *map = a.qmaps + ((size_t)(TY == 16) * a.ninst + item.x) * 2 + which;
    mbar_expect_tx(bar, (unsigned)(4 * SH * SW * sizeof(T)));
    tma_load_3d(sqbuf, map, item.y - kTL, item.z - kH, 0, bar);
}

template <int N>
__device__ __forceinline__ void tile_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// One tile of phase A from its staged halo tile (tile_issue, completed).
template <typename T, int TY>
__device__ void stage_tile(const Args &a, int st, int4 item, const T *qin, T *qout,
                           const T *sqbuf)
{
    constexpr int SW = tile_sw<TY>(), SH = tile_sh<TY>();
    const T(*sq)[SH][SW] = reinterpret_cast<const T(*)[SH][SW]>(sqbuf);
    NS_CHECK(a.err, kChkBatch, item.x >= 0 && item.x < a.ninst);
    const Inst in = a.inst[item.x];
    const int i0 = item.y, j0 = item.z;
    // tile rows ly + kH +- 3 < SH and columns tx + kTL +- 3 < SW; closures
    // need lines of at least 7 points
    NS_CHECK(a.err, kChkBatch, blockDim.x == 32 * kWarps && TY % kWarps == 0 && i0 >= 0 &&
                                   i0 < in.imax && j0 >= 0 && j0 < in.jmax && in.imax >= 7 &&
                                   in.jmax >= 7);
    const long long plane = (long long)in.pitch * in.jmax;
    const T *q = qin + in.q_off;
    T *qo = qout + in.q_off;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i = i0 + tx;
    if (i < in.imax) {
        const T *cxp = tab<T>(a.xc) + (long long)kCoefStride * (in.x_off + i);
        const float *cxl = a.xcl + (long long)kCoefStride * (in.x_off + i);
        const bool xint = (i >= 3 && i < in.imax - 3);
        const T ssin = (T)a.stage_sin[item.x * 8 + st];
#pragma unroll
        for (int h = 0; h < TY / kWarps; h++) {
            const int ly = ty + kWarps * h;
            const int j = j0 + ly;
            if (j >= in.jmax) break;
            const long long idx = (long long)j * in.pitch + i;
            const int sr = ly + kH, sc = tx + kTL;
            const T *cyp = tab<T>(a.yc) + (long long)kCoefStride * (in.y_off + j);
            const float *cyl = a.ycl + (long long)kCoefStride * (in.y_off + j);
            const bool yint = (j >= 3 && j < in.jmax - 3);
            T qv[4], gx[4], gy[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                qv[k] = sq[k][sr][sc];
                if (xint) {
                    T r = cxp[4] * (sq[k][sr][sc + 1] - sq[k][sr][sc - 1]);
                    r = fma(cxp[5], sq[k][sr][sc + 2] - sq[k][sr][sc - 2], r);
                    gx[k] = fma(cxp[6], sq[k][sr][sc + 3] - sq[k][sr][sc - 3], r);
                } else {
                    const int o0 = (i < 3) ? -i : (in.imax - 7 - i);
                    const T *g = q + k * plane + idx + o0;
                    const T f0 = (sizeof(T) == 4) ? q[k * plane + idx] : T(0);
                    T r = T(0);
#pragma unroll
                    for (int z = 0; z < 7; z++) r = fma(cxp[z], g[z] - f0, r);
                    gx[k] = r;
                }
                if (yint) {
                    T r = cyp[4] * (sq[k][sr + 1][sc] - sq[k][sr - 1][sc]);
                    r = fma(cyp[5], sq[k][sr + 2][sc] - sq[k][sr - 2][sc], r);
                    gy[k] = fma(cyp[6], sq[k][sr + 3][sc] - sq[k][sr - 3][sc], r);
                } else {
                    const int o0 = (j < 3) ? -j : (in.jmax - 7 - j);
                    const T *g = q + k * plane + idx + (long long)o0 * in.pitch;
                    const T f0 = (sizeof(T) == 4) ? q[k * plane + idx] : T(0);
                    T r = T(0);
#pragma unroll
                    for (int z = 0; z < 7; z++) r = fma(cyp[z], g[(long long)z * in.pitch] - f0, r);
                    gy[k] = r;
                }
            }
            const bool interior = (i > 0) && (i < in.imax - 1) && (j > 0) && (j < in.jmax - 1);
            if (interior) {
                T div = gx[1] + gy[2];
                if constexpr (sizeof(T) == 4) if (xint && yint) {
                    // compensated divergence, as the single-grid split path
                    float xh = 0.f, xl = 0.f, yh = 0.f, yl = 0.f;
#pragma unroll
                    for (int s = 1; s <= 3; s++) {
                        float dh, dl, sh, se;
                        two_sum((float)sq[1][sr][sc + s], -(float)sq[1][sr][sc - s], dh, dl);
                        float ph = cxp[3 + s] * dh;
                        float pl = fmaf(cxp[3 + s], dh, -ph) + fmaf(cxp[3 + s], dl, cxl[3 + s] * dh);
                        two_sum(xh, ph, sh, se);
                        xh = sh;
                        xl += se + pl;
                        two_sum((float)sq[2][sr + s][sc], -(float)sq[2][sr - s][sc], dh, dl);
                        ph = cyp[3 + s] * dh;
                        pl = fmaf(cyp[3 + s], dh, -ph) + fmaf(cyp[3 + s], dl, cyl[3 + s] * dh);
                        two_sum(yh, ph, sh, se);
                        yh = sh;
                        yl += se + pl;
                    }
                    float sh, se;
                    two_sum(xh, yh, sh, se);
                    div = T(sh + (se + (xl + yl)));
                }
                const int yo = in.y_off + j;
                const T rho = tab<T>(a.mrho)[yo] + qv[0];
                const T uu = tab<T>(a.mu)[yo] + qv[1];
                const T vv = qv[2];
                const T pp = pick<T>(in.pmean_f, in.pmean_d) + qv[3];
                const T rhoy = tab<T>(a.mdrho)[yo] + gy[0];
                const T uy = tab<T>(a.mdu)[yo] + gy[1];
                const T ri = T(1) / rho;
                T r[4];
                T t = uu * gx[0];
                t = fma(vv, rhoy, t);
                t = fma(rho, div, t);
                r[0] = -t;
                t = uu * gx[1];
                t = fma(ri, gx[3], t);
                t = fma(vv, uy, t);
                r[1] = -t;
                t = uu * gx[2];
                t = fma(vv, gy[2], t);
                t = fma(ri, gy[3], t);
                r[2] = -t;
                const T gp = pick<T>(in.gamma_f, in.gamma_d) * pp;
                t = uu * gx[3];
                t = fma(vv, gy[3], t);
                t = fma(gp, div, t);
                if (in.s_off >= 0) {
                    const T *src = reinterpret_cast<const T *>(a.src) + in.s_off;
                    t = t - ssin * src[idx];
                }
                r[3] = -t;
                double *Wp = a.W + in.w_off + idx;
                // FP64 instances: w = alpha*w + dt*R, U += beta*w (rk.f90:163-164).
                // FP32 perturbations carry w/dt instead (w~ = alpha*w~ + R,
                // q' += (beta*dt)*w~), so that dt enters only through the FP64
                // product beta*dt and not as FP32(dt)*R, whose rounding of dt
                // would scale every step (ns_split.cu does the same).
                constexpr bool kF32 = std::is_same<T, float>::value;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const double dr =
                        kF32 ? to_d<T>(r[k]) : to_d<T>(pick<T>(in.dt_f, in.dt_d) * r[k]);
                    const double w = (st == 0) ? dr : fma(a.alpha[st], Wp[k * plane], dr);
                    if (st < 5) Wp[k * plane] = w;  // stage 0 sets w (or w~)
                    // beta*dt from the per-instance table, read where it is used
                    const double bw = kF32 ? a.bdt[item.x * 6 + st] : a.beta[st];
                    qv[k] = from_d<T>(fma(bw, w, to_d<T>(qv[k])));
                }
            }
            if (j < in.D || j >= in.jmax - in.D) {
                const T s = tab<T>(a.sigy)[in.y_off + j];
#pragma unroll
                for (int k = 0; k < 4; k++) qv[k] *= s;
            }
            if (i < in.D || i >= in.imax - in.D) {
                const T s = tab<T>(a.sigx)[in.x_off + i];
#pragma unroll
                for (int k = 0; k < 4; k++) qv[k] *= s;
            }
#pragma unroll
            for (int k = 0; k < 4; k++) qo[k * plane + idx] = qv[k];
        }
    }
}

// ---------------------------------------------------------------------------
// Filter recurrences (constant-exact forms of ns_split.cu).
// ---------------------------------------------------------------------------
// Interior filter step.  FP32: the constant-exact form of ns_split.cu.
// FP64: v = c0*u0 + sum_s m_s*(u_s + u_-s), c0 = 1 - sigmaf*df(0) (m[0]),
// the form and operation count of the single-grid FP64 kernel.
template <typename T>
__device__ __forceinline__ T pass2(const T *w, const T *m)
{
    if constexpr (sizeof(T) == 8) {
        T v = m[0] * w[6];
        v = fma(m[6], w[12] + w[0], v);
        v = fma(m[5], w[11] + w[1], v);
        v = fma(m[4], w[10] + w[2], v);
        v = fma(m[3], w[9] + w[3], v);
        v = fma(m[2], w[8] + w[4], v);
        v = fma(m[1], w[7], v);
        return fma(m[1], w[5], v);
    }
    const T u0 = w[6];
    T acc = m[6] * ((w[12] - u0) + (w[0] - u0));
    acc = fma(m[5], (w[11] - u0) + (w[1] - u0), acc);
    acc = fma(m[4], (w[10] - u0) + (w[2] - u0), acc);
    acc = fma(m[3], (w[9] - u0) + (w[3] - u0), acc);
    acc = fma(m[2], (w[8] - u0) + (w[4] - u0), acc);
    acc = fma(m[1], w[7] - u0, acc);
    return fma(m[1], w[5] - u0, u0 + acc);
}

// Boundary filter step (b[0]: FP64 holds 1 - sigmaf*dfb(0) there).
template <typename T, int DIR>
__device__ __forceinline__ T passb(const T *w, int p, T bm1, const T *b, T bsum)
{
    if constexpr (sizeof(T) == 8) {
        T v = b[0] * w[p];
#pragma unroll
        for (int z = 1; z <= 5; z++) v = fma(b[z], w[p + DIR * z], v);
        return fma(bm1, w[p - DIR], v);
    }
    const T u0 = w[p];
    T acc = bsum * u0;
#pragma unroll
    for (int z = 1; z <= 5; z++) acc = fma(b[z], w[p + DIR * z] - u0, acc);
    return fma(bm1, w[p - DIR] - u0, u0 + acc);
}

template <typename T>
struct FCoef {
    const T *m, *b;
    T bm1, bsum;
};
template <typename T>
__device__ __forceinline__ FCoef<T> fcoef(const Args &a, int d);
template <>
__device__ __forceinline__ FCoef<float> fcoef<float>(const Args &a, int d)
{
    return {a.fm_f, a.fb_f[d], a.fbm1_f[d], a.fbsum_f[d]};
}
template <>
__device__ __forceinline__ FCoef<double> fcoef<double>(const Args &a, int d)
{
    return {a.fm_d, a.fb_d[d], a.fbm1_d[d], a.fbsum_d[d]};
}

// Phase C: y lines of 32 consecutive columns (one per lane).
template <typename T>
__device__ void fy_item(const Args &a, int4 item, const T *srcq, T *dstq)
{
    NS_CHECK(a.err, kChkBatch, item.x >= 0 && item.x < a.ninst);
    const Inst in = a.inst[item.x];
    const int k = item.y, col = item.z + (threadIdx.x & 31), c = item.w;
    NS_CHECK(a.err, kChkBatch, k >= 0 && k < 4 && item.z >= 0 && item.z % 32 == 0 &&
                                   item.z < in.imax && c >= 0 && c < in.fy_chunks &&
                                   in.jmax >= 13);
    if (col >= in.imax) return;
    const int n = in.jmax, chunks = in.fy_chunks, warm = in.warm;
    const long long st = in.pitch;
    const long long base = in.q_off + (long long)k * in.pitch * in.jmax + col;
    const T *s = srcq + base;
    T *o = dstq + base;
    const T *cr = tab<T>(a.corr) + 4LL * in.y_off + (long long)k * n;  // [k][j] of this instance
    const FCoef<T> fc = fcoef<T>(a, 1);
    const int len2 = n - 12;
    const int a0 = 6 + (int)(((long long)c * len2) / chunks);
    const int b0 = 6 + (int)(((long long)(c + 1) * len2) / chunks);
    NS_CHECK(a.err, kChkBatch, 6 <= a0 && a0 <= b0 && b0 <= n - 6);
    T w[13];
    int q;
    if (c == 0 || warm < 0 || a0 - warm <= 6) {
#pragma unroll
        for (int t = 0; t < 13; t++) w[t] = s[t * st];
#pragma unroll
        for (int p = 1; p <= 6; p++) w[p] = passb<T, 1>(w, p, fc.bm1, fc.b, fc.bsum);
        if (c == 0)
            for (int p = 0; p < 6; p++) o[p * st] = w[p] + cr[p];
        q = 6;
    } else {
        q = a0 - warm;
#pragma unroll
        for (int t = 0; t < 13; t++) w[t] = s[(long long)(q - 6 + t) * st];
    }
    auto step = [&](int qq, T next) {
        const T v = pass2<T>(w, fc.m);
        if (qq >= a0) o[(long long)qq * st] = v + cr[qq];
#pragma unroll
        for (int u = 0; u < 5; u++) w[u] = w[u + 1];
        w[5] = v;
#pragma unroll
        for (int u = 6; u < 12; u++) w[u] = w[u + 1];
        w[12] = next;
    };
    // blocks of 8 steps, the next block's inputs loaded before this one runs
    T nx[8];
#pragma unroll
    for (int t = 0; t < 8; t++) nx[t] = (q + 7 + t < n) ? s[(long long)(q + 7 + t) * st] : T(0);
    for (; q + 8 <= b0; q += 8) {
        T cur[8];
#pragma unroll
        for (int t = 0; t < 8; t++) {
            cur[t] = nx[t];
            nx[t] = (q + 15 + t < n) ? s[(long long)(q + 15 + t) * st] : T(0);
        }
#pragma unroll
        for (int t = 0; t < 8; t++) step(q + t, cur[t]);
    }
    for (; q < b0; q++) step(q, (q + 7 < n) ? s[(long long)(q + 7) * st] : T(0));
    if (c == chunks - 1) {
#pragma unroll
        for (int x = 10; x >= 5; x--) w[x] = passb<T, -1>(w, x, fc.bm1, fc.b, fc.bsum);
        for (int x = 5; x < 12; x++) o[(long long)(n - 12 + x) * st] = w[x] + cr[n - 12 + x];
    }
}

// Phase B: x lines of 32 consecutive rows, staged through shared memory
// PW positions at a time (coalesced row segments).  The copies go by
// cp.async into two tiles, the next block's in flight while the current
// block is filtered; each step leaves its output in the tile column it read,
// and the tile goes back with row writes.
template <typename T, int PW>
__device__ void fx_item(const Args &a, int4 item, const T *srcq, T *dstq,
                        T (*tbuf)[32][PW + 1])
{
    NS_CHECK(a.err, kChkBatch, item.x >= 0 && item.x < a.ninst);
    const Inst in = a.inst[item.x];
    const int lane = threadIdx.x & 31;
    const int k = item.y, row0 = item.z, c = item.w;
    const int n = in.imax, chunks = in.fx_chunks, warm = in.warm;
    const int nrows = min(32, in.jmax - row0);
    // rows row0 .. row0+nrows-1 (1..32, the tile's rows) of plane k
    NS_CHECK(a.err, kChkBatch, k >= 0 && k < 4 && row0 >= 0 && row0 % 32 == 0 && nrows >= 1 &&
                                   c >= 0 && c < chunks && n >= 13 && in.pitch >= n);
    const long long base = in.q_off + (long long)k * in.pitch * in.jmax + (long long)row0 * in.pitch;
    const T *sb = srcq + base;
    T *ob = dstq + base;
    const bool active = lane < nrows;
    const T *s = sb + (long long)(active ? lane : 0) * in.pitch;
    const int len2 = n - 12;
    const int a0 = 6 + (int)(((long long)c * len2) / chunks);
    const int b0 = 6 + (int)(((long long)(c + 1) * len2) / chunks);
    const bool exact = (c == 0 || warm < 0 || a0 - warm <= 6);
    const int q0 = exact ? 6 : a0 - warm;
    NS_CHECK(a.err, kChkBatch, 6 <= a0 && a0 <= b0 && b0 <= n - 6 && q0 >= 6 && q0 <= a0);
    const FCoef<T> fc = fcoef<T>(a, 0);
    // copies of the block starting at step qb (positions qb+7 ..) into tile buf
    auto issue = [&](int buf, int qb) {
        const int pin = qb + 7;
        for (int r = 0; r < nrows; r++)
            for (int x = lane; x < PW; x += 32) {
                const int pos = pin + x;
                const bool ok = pos < n;
                cp_async_elem(&tbuf[buf][r][x], sb + (long long)r * in.pitch + (ok ? pos : 0), ok);
            }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    if (q0 < b0) issue(0, q0);
    T w[13];
    if (exact) {
#pragma unroll
        for (int t = 0; t < 13; t++) w[t] = s[t];
#pragma unroll
        for (int p = 1; p <= 6; p++) w[p] = passb<T, 1>(w, p, fc.bm1, fc.b, fc.bsum);
        if (c == 0 && active)
            for (int p = 0; p < 6; p++) ob[(long long)lane * in.pitch + p] = w[p];
    } else {
#pragma unroll
        for (int t = 0; t < 13; t++) w[t] = s[q0 - 6 + t];
    }
    int buf = 0;
    for (int qb = q0; qb < b0; qb += PW) {
        if (qb + PW < b0) {
            issue(buf ^ 1, qb + PW);
            tile_wait<1>();  // this block's copies have landed
        } else {
            tile_wait<0>();
        }
        __syncwarp();
        T(*tb)[PW + 1] = tbuf[buf];
        const int nstep = min(PW, b0 - qb);
        auto step = [&](int t) {
            const T v = pass2<T>(w, fc.m);
            const T nxt = tb[lane][t];
            tb[lane][t] = v;
#pragma unroll
            for (int u = 0; u < 5; u++) w[u] = w[u + 1];
            w[5] = v;
#pragma unroll
            for (int u = 6; u < 12; u++) w[u] = w[u + 1];
            w[12] = nxt;
        };
        for (int t = 0; t < nstep; t++) step(t);
        __syncwarp();
        for (int r = 0; r < nrows; r++)
            for (int x = lane; x < PW; x += 32) {
                const int qq = qb + x;
                if (x < nstep && qq >= a0) ob[(long long)r * in.pitch + qq] = tb[r][x];
            }
        __syncwarp();
        buf ^= 1;
    }
    if (c == chunks - 1 && active) {
#pragma unroll
        for (int x = 10; x >= 5; x--) w[x] = passb<T, -1>(w, x, fc.bm1, fc.b, fc.bsum);
        for (int x = 5; x < 12; x++) ob[(long long)lane * in.pitch + (n - 12 + x)] = w[x];
    }
}

// Phase D: ccpml of one instance at positions item.y .. item.y+31 (rows of
// the left and right columns, columns of the top and bottom rows), one warp.
// Every position's values are independent of the others' (the corner
// columns recompute the column values they extrapolate from), so the
// perimeter splits into pieces freely.
template <typename T>
__device__ void bc_item(const Args &a, int2 item, T *qall)
{
    const int inst = item.x;
    NS_CHECK(a.err, kChkBatch, inst >= 0 && inst < a.ninst && item.y >= 0 && item.y % 32 == 0);
    const Inst in = a.inst[inst];
    const long long P = (long long)in.pitch * in.jmax;
    T *q = qall + in.q_off;
    const T pbc = pick<T>(in.p_bc_f, in.p_bc_d);
    const T *rbc = tab<T>(a.rho_bc) + in.y_off;
    auto colval = [&](int i, int j, T *v) {
        const long long r = (long long)j * in.pitch;
        if (i == 0) {
            v[0] = rbc[j];
            v[1] = T(2) * q[P + r + 1] - q[P + r + 2];
            v[2] = T(0);
            v[3] = pbc;
        } else {
            for (int k = 0; k < 3; k++) v[k] = T(2) * q[k * P + r + in.imax - 2] - q[k * P + r + in.imax - 3];
            v[3] = pbc;
        }
    };
    const int nt = max(in.imax, in.jmax);
    {
        const int t = item.y + (threadIdx.x & 31);
        if (t >= nt) return;
        T v[4];
        if (t > 0 && t < in.jmax - 1) {
            const long long r = (long long)t * in.pitch;
            colval(0, t, v);
            for (int k = 0; k < 4; k++) q[k * P + r] = v[k];
            colval(in.imax - 1, t, v);
            for (int k = 0; k < 4; k++) q[k * P + r + in.imax - 1] = v[k];
        }
        if (t < in.imax) {
            const int jt = in.jmax - 1;
            T x[4], y[4];
            if (t == 0 || t == in.imax - 1) {
                colval(t, jt - 1, x);
                colval(t, jt - 2, y);
            } else {
                for (int k = 0; k < 4; k++) {
                    x[k] = q[k * P + (long long)(jt - 1) * in.pitch + t];
                    y[k] = q[k * P + (long long)(jt - 2) * in.pitch + t];
                }
            }
            for (int k = 0; k < 3; k++) q[k * P + (long long)jt * in.pitch + t] = T(2) * x[k] - y[k];
            q[3 * P + (long long)jt * in.pitch + t] = pbc;
            if (t == 0 || t == in.imax - 1) {
                colval(t, 1, x);
                colval(t, 2, y);
            } else {
                for (int k = 0; k < 4; k++) {
                    x[k] = q[k * P + in.pitch + t];
                    y[k] = q[k * P + 2LL * in.pitch + t];
                }
            }
            for (int k = 0; k < 3; k++) q[k * P + t] = T(2) * x[k] - y[k];
            q[3 * P + t] = pbc;
        }
    }
}

// Items handed out one per warp from a counter, largest first (the host
// sorts the lists by cost): the phase ends close to total work / warps
// instead of at the unluckiest warp's share.
template <typename F>
__device__ __forceinline__ void for_items(unsigned *ctr, int n, F &&f)
{
    for (;;) {
        unsigned w = 0;
        if ((threadIdx.x & 31) == 0) w = atomicAdd(ctr, 1u);
        w = __shfl_sync(0xffffffffu, w, 0);
        if ((int)w >= n) break;
        f((int)w);
    }
}

__device__ __forceinline__ void stamp(const Args &a, int slot)
{
    if (a.stamps && blockIdx.x == 0 && threadIdx.x == 0) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        a.stamps[slot] = t;
    }
}

// TY: tile rows of phase A; PW: x-line block width of phase B (its two
// tiles per warp set the shared memory, and with it how many blocks fit on
// an SM).  The autotuner picks the shape.  The FP32 shapes fit 64 registers
// without spilling, so 4 blocks per SM when the shared memory allows.
template <typename T, int TY, int PW>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 1) k_batch_step(Args a)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5;
    // this warp's two x-line tiles of 32 rows
    T(*tx2)[32][PW + 1] = reinterpret_cast<T(*)[32][PW + 1]>(smem) + (size_t)warp * 2;
    const long long nwarps = (long long)gridDim.x * kWarps;
    const long long gw = (long long)blockIdx.x * kWarps + warp;
    // one mbarrier per tile buffer; tuse counts the completed phases of
    // both, buffer 0 in the low half and buffer 1 in the high half
    __shared__ alignas(8) unsigned long long tbar[2];
    unsigned tuse = 0u;
    if (threadIdx.x == 0) {
        mbar_init(&tbar[0], 1);
        mbar_init(&tbar[1], 1);
    }
    __syncthreads();
    stamp(a, 0);
    for (int st = 0; st < 6; st++) {
        T *qa = reinterpret_cast<T *>((st & 1) ? a.q1 : a.q0);
        T *qb = reinterpret_cast<T *>((st & 1) ? a.q0 : a.q1);
        {
            // two tile buffers: the next item's TMA load is in flight while
            // the current item is computed.  The region was last written and
            // read by the generic proxy (the previous phases): fence before
            // the async proxy writes it.
            constexpr size_t kTile = 4 * (size_t)tile_sh<TY>() * tile_sw<TY>();
            T *const buf0 = reinterpret_cast<T *>(smem);
            auto buf = [&](int x) { return buf0 + x * kTile; };
            const int which = st & 1;  // qa is q1 in odd stages
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            int b = 0;
            if (threadIdx.x == 0 && (int)blockIdx.x < a.ntiles)
                tile_issue<T, TY>(a, a.tiles[blockIdx.x], which, buf(0), &tbar[0]);
            for (int it = blockIdx.x; it < a.ntiles; it += gridDim.x) {
                const int nx = it + (int)gridDim.x;
                if (threadIdx.x == 0 && nx < a.ntiles)
                    tile_issue<T, TY>(a, a.tiles[nx], which, buf(b ^ 1), &tbar[b ^ 1]);
                if (!mbar_wait_bounded(&tbar[b], (tuse >> (16 * b)) & 1u, a.err)) return;
                tuse += 1u << (16 * b);
                stage_tile<T, TY>(a, st, a.tiles[it], qa, qb, buf(b));
                __syncthreads();  // buf[b] is refilled two items on
                b ^= 1;
            }
        }
        if (!grid_barrier(a)) return;
        stamp(a, 1 + 4 * st);
        for_items(a.work + 2 * st, a.nfx,
                  [&](int wi) { fx_item<T, PW>(a, a.fx[wi], qb, qa, tx2); });
        if (!grid_barrier(a)) return;
        stamp(a, 2 + 4 * st);
        for_items(a.work + 2 * st + 1, a.nfy, [&](int wi) { fy_item<T>(a, a.fy[wi], qa, qb); });
        if (!grid_barrier(a)) return;
        stamp(a, 3 + 4 * st);
        for (long long wi = gw; wi < a.nbc; wi += nwarps) bc_item<T>(a, a.bc[wi], qb);
        if (a.stamps && !grid_barrier(a)) return;  // timed runs close every phase
        if (!a.stamps && st < 5 && !grid_barrier(a)) return;
        stamp(a, 4 + 4 * st);
    }
}

__global__ void k_batch_sin(const double *wf, const double *dt, int n, int *d_iter, double *ss)
{
    const int t = threadIdx.x;
    const int iter = *d_iter;
    // rk.f90:188: sin(wf*((iter+c_k)*dt)) per instance and stage
    const double ct[6] = {0.0, 0.032918605146, 0.249351723343,
                          0.466911705055, 0.582030414044, 0.847252983783};
    for (int e = t; e < n * 6; e += blockDim.x) {
        const int in = e / 6, k = e % 6;
        ss[in * 8 + k] = sin(wf[in] * (((double)iter + ct[k]) * dt[in]));
    }
    __syncthreads();
    if (t == 0) *d_iter = iter + 1;
}

__global__ void k_batch_set_iter(int *d_iter, int v) { *d_iter = v; }

template <typename T>
__global__ void k_batch_from_full(const double *U, int imax, int jmax, int upitch,
                                  const double *rho, const double *u, double pmean, T *q,
                                  int pitch)
{
    // U: host-uploaded FP64 planes (upitch), q' = U - Ub with Ub(j) = (rho, u, 0, pmean)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= imax || j >= jmax) return;
    const double base[4] = {rho[j], u[j], 0.0, pmean};
    for (int k = 0; k < 4; k++)
        q[(long long)k * pitch * jmax + (long long)j * pitch + i] =
            (T)(U[(long long)k * upitch * jmax + (long long)j * upitch + i] - base[k]);
}

template <typename T>
__global__ void k_batch_to_full(const T *q, int imax, int jmax, int pitch, const double *rho,
                                const double *u, double pmean, double *U, int upitch)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= imax || j >= jmax) return;
    const double base[4] = {rho[j], u[j], 0.0, pmean};
    for (int k = 0; k < 4; k++)
        U[(long long)k * upitch * jmax + (long long)j * upitch + i] =
            base[k] + (double)q[(long long)k * pitch * jmax + (long long)j * pitch + i];
}

}  // namespace batch
}  // namespace ns

// ===========================================================================
// Host side
// ===========================================================================
struct ns_batch {
    int n = 0, dev = 0, precision = NS_PREC_FP64;
    cudaStream_t own = nullptr, stream = nullptr;
    std::vector<ns::batch::Inst> hinst;
    std::vector<double> hrho, hu;                 // per-row base flow, pooled
    std::vector<double> hpmean;
    size_t qsize = 0, wsize = 0;                  // elements
    void *q[2] = {nullptr, nullptr};
    double *W = nullptr, *stage_sin = nullptr, *wf = nullptr, *dtv = nullptr, *bdt = nullptr;
    double *drho = nullptr, *du = nullptr;        // FP64 per-row base flow for conversions
    double *stagebuf = nullptr;                   // FP64 staging planes for host transfers
    size_t stagebuf_elems = 0;
    ns::batch::Inst *inst = nullptr;
    int4 *tiles[2] = {nullptr, nullptr}, *fx = nullptr, *fy = nullptr;
    int ntiles[2] = {0, 0}, nfx = 0, nfy = 0, nbc = 0;
    int2 *bc = nullptr;
    CUtensorMap *qmaps = nullptr;  // [(ty16 * n + inst) * 2 + buf]
    void *xc = nullptr, *yc = nullptr, *sigx = nullptr, *sigy = nullptr, *rho_bc = nullptr,
         *mrho = nullptr, *mu = nullptr, *mdrho = nullptr, *mdu = nullptr, *corr = nullptr;
    float *xcl = nullptr, *ycl = nullptr;
    void *src = nullptr;
    unsigned *bar = nullptr;   // [0] count, [1] generation
    int *err = nullptr;
    int *d_iter = nullptr;
    ns::batch::Args args{};
    int ty = 16, pw = 16, blocks_per_sm = 0, grid = 0;
    size_t smem = 0;
    double tuned_ms = 0.0;
    bool has_src = false, have_state = false;
    bool no_graph = false;    // capture of the cooperative launch unavailable
    cudaGraphExec_t exec = nullptr;
    std::string err_text;
};

namespace {

using namespace ns::coef;

int berr(ns_batch *b, int code, const std::string &msg)
{
    if (b) b->err_text = msg;
    ns::record_error(msg.c_str());
    return code;
}

void coef_table(std::vector<double> &tab, int n, double h, const double *mesh, int D, int mode)
{
    tab.resize((size_t)n * ns::kCoefStride);
    line_table(tab.data(), n, h, mesh, D, mode);
}

double line_deriv(const double *f, int q, int n, const double *c)
{
    if (q >= 3 && q < n - 3)
        return c[4] * (f[q + 1] - f[q - 1]) + c[5] * (f[q + 2] - f[q - 2]) + c[6] * (f[q + 3] - f[q - 3]);
    const int o0 = (q < 3) ? -q : (n - 7 - q);
    double r = 0.0;
    for (int z = 0; z < 7; z++) r += c[z] * f[q + o0 + z];
    return r;
}

template <class T>
int balloc(ns_batch *b, T **p, size_t n)
{
    if (cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        *p = nullptr;
        return berr(b, NS_ERR_OOM, "ns_batch: cudaMalloc failed");
    }
    return NS_OK;
}

// Allocates a device table of v in the state precision (es = 4: FP32, 8:
// FP64) and uploads it synchronously.
int tput(ns_batch *b, void **d, const std::vector<double> &v, size_t es)
{
    if (cudaMalloc(d, std::max<size_t>(v.size(), 1) * es) != cudaSuccess) {
        *d = nullptr;
        return berr(b, NS_ERR_OOM, "ns_batch: cudaMalloc failed");
    }
    cudaError_t e;
    if (es == 4) {
        std::vector<float> f(v.begin(), v.end());
        e = cudaMemcpy(*d, f.data(), f.size() * 4, cudaMemcpyHostToDevice);
    } else {
        e = cudaMemcpy(*d, v.data(), v.size() * 8, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) return berr(b, NS_ERR_CUDA, "ns_batch: table upload failed");
    return NS_OK;
}

template <class T>
int bput(ns_batch *b, T *d, const std::vector<T> &v)
{
    if (v.empty()) return NS_OK;
    if (cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, b->stream) !=
        cudaSuccess)
        return berr(b, NS_ERR_CUDA, "ns_batch: upload failed");
    return NS_OK;
}

void bfree(ns_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    void *ps[] = {b->q[0], b->q[1], b->W, b->stage_sin, b->wf, b->dtv, b->bdt, b->drho, b->du,
                  b->stagebuf, b->inst, b->tiles[0], b->tiles[1], b->fx, b->fy, b->bc,
                  b->xc, b->xcl, b->yc, b->ycl, b->sigx, b->sigy, b->rho_bc, b->mrho, b->mu,
                  b->mdrho, b->mdu, b->corr, b->src, b->bar, b->err, b->d_iter, b->qmaps};
    for (void *p : ps)
        if (p) cudaFree(p);
    if (b->own) cudaStreamDestroy(b->own);
}

using StepKernel = void (*)(ns::batch::Args);

// The step kernel of a shape: precision, tile rows (8, 16) and x-line block
// width (16, 24 or 32 positions for FP32, 16 for FP64).  For FP32 the
// x-line tiles take 35, 51 or 68 KB per block: 4, 4 or 3 blocks fit on an
// SM, and the more shared memory, the less L1 remains for the tile phase's
// table and closure loads.  The autotuner measures which wins.
StepKernel step_kernel(int precision, int ty, int pw)
{
    using ns::batch::k_batch_step;
    if (precision == NS_PREC_SPLIT32) {
        if (ty == 8)
            return pw == 32 ? k_batch_step<float, 8, 32>
                            : pw == 24 ? k_batch_step<float, 8, 24> : k_batch_step<float, 8, 16>;
        return pw == 32 ? k_batch_step<float, 16, 32>
                        : pw == 24 ? k_batch_step<float, 16, 24> : k_batch_step<float, 16, 16>;
    }
    return ty == 8 ? k_batch_step<double, 8, 16> : k_batch_step<double, 16, 16>;
}

cudaError_t launch_step_k(ns_batch *b, cudaStream_t s, unsigned long long *stamps)
{
    ns::batch::Args a = b->args;
    a.stamps = stamps;
    a.tiles = b->tiles[b->ty == 8 ? 0 : 1];
    a.ntiles = b->ntiles[b->ty == 8 ? 0 : 1];
    a.nblocks = (unsigned)b->grid;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)b->grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = b->smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, step_kernel(b->precision, b->ty, b->pw), a);
}

cudaError_t launch_step(ns_batch *b, cudaStream_t s, unsigned long long *stamps = nullptr)
{
    // the per-stage item counters start every step at zero
    cudaError_t me = cudaMemsetAsync(b->bar + 2, 0, 12 * sizeof(unsigned), s);
    if (me != cudaSuccess) return me;
    if (b->has_src) {
        ns::batch::k_batch_sin<<<1, 256, 0, s>>>(b->wf, b->dtv, b->n, b->d_iter, b->stage_sin);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return launch_step_k(b, s, stamps);
}

size_t smem_for(int precision, int ty, int pw)
{
    const size_t es = precision == NS_PREC_SPLIT32 ? 4 : 8;
    const size_t tile = 2 * 4 * (size_t)(ty + 6) * 40 * es;  // two tile buffers
    const size_t fx = (size_t)ns::batch::kWarps * 2 * 32 * (pw + 1) * es;
    return std::max(tile, fx);
}

int occupancy(StepKernel k, size_t smem)
{
    int nb = 0;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, 256, smem);
    return nb;
}

int configure(ns_batch *b, int ty, int pw, int bps)
{
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->dev);
    b->ty = ty;
    b->pw = pw;
    b->smem = smem_for(b->precision, ty, pw);
    const int maxb = occupancy(step_kernel(b->precision, ty, pw), b->smem);
    if (maxb < 1) return berr(b, NS_ERR_CUDA, "ns_batch: the step kernel cannot be resident");
    b->blocks_per_sm = (bps > 0 && bps < maxb) ? bps : maxb;
    b->grid = b->blocks_per_sm * nsm;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    return NS_OK;
}

int ensure_graph(ns_batch *b)
{
    if (b->exec) return NS_OK;
    cudaStream_t cs;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess)
        return berr(b, NS_ERR_CUDA, "ns_batch: stream");
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t le = launch_step(b, cs);
        e = cudaStreamEndCapture(cs, &g);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) {
        b->exec = nullptr;
        cudaGetLastError();
        return berr(b, NS_ERR_CUDA, std::string("ns_batch: graph capture: ") + cudaGetErrorString(e));
    }
    return NS_OK;
}

int check_err(ns_batch *b)
{
    int h = 0;
    if (cudaMemcpyAsync(&h, b->err, sizeof(int), cudaMemcpyDeviceToHost, b->stream) != cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess)
        return berr(b, NS_ERR_CUDA, std::string("ns_batch: ") + cudaGetErrorString(cudaGetLastError()));
    if (h) {
        cudaMemsetAsync(b->err, 0, sizeof(int), b->stream);
        cudaMemsetAsync(b->bar, 0, 2 * sizeof(unsigned), b->stream);
        cudaStreamSynchronize(b->stream);
        if (h & ns::kCheckTag) {
            const int rc = ns::check_error(h);
            b->err_text = ns_last_error(nullptr);
            return rc;
        }
        return berr(b, NS_ERR_TIMEOUT, "ns_batch: a phase barrier of the persistent step kernel timed out");
    }
    return NS_OK;
}

}  // namespace

extern "C" {

int ns_batch_create(const ns_params *const *params, int n, int precision, ns_batch **out)
{
    if (!out || !params || n < 1) return berr(nullptr, NS_ERR_PARAM, "ns_batch_create: bad argument");
    *out = nullptr;
    if (precision == NS_PREC_SPLIT)
        return berr(nullptr, NS_ERR_UNSUPPORTED,
                    "ns_batch_create: the batched path carries single FP32 perturbations: "
                    "use NS_PREC_SPLIT32");
    if (precision != NS_PREC_FP64 && precision != NS_PREC_SPLIT32)
        return berr(nullptr, NS_ERR_PARAM, "ns_batch_create: precision");
    for (int q = 0; q < n; q++) {
        const ns_params *p = params[q];
        if (!p || p->abi_version != NS_ABI_VERSION || !p->inviscid || p->nk != 4 || p->imax < 13 ||
            p->jmax < 13 || p->D < 0 || 2 * p->D > p->imax || 2 * p->D > p->jmax ||
            !(p->dt > 0) || !(p->dm > 0) || !(p->dn > 0) || !p->meshx || !p->meshy ||
            !p->sigmax || !p->sigmay || !p->rhob || !p->Ub ||
            (p->source_mode == NS_SRC_GAUSSIAN && (!p->m || !p->n || !(p->r0 != 0.0))) ||
            (p->source_mode == NS_SRC_FIELD && !p->src_field) || p->device != params[0]->device ||
            p->sigmaf != params[0]->sigmaf)
            return berr(nullptr, NS_ERR_PARAM,
                        "ns_batch_create: instance " + std::to_string(q) +
                            ": each instance must be a valid Euler case (inviscid=1, nk=4) on "
                            "the same device with the same sigmaf");
    }
    ns_batch *b = new (std::nothrow) ns_batch();
    if (!b) return berr(nullptr, NS_ERR_OOM, "ns_batch_create: host allocation");
    b->n = n;
    b->dev = params[0]->device;
    b->precision = precision;
    int rc = NS_OK;
    const size_t es = precision == NS_PREC_SPLIT32 ? 4 : 8;
    std::vector<ns::batch::Inst> hin(n);
    std::vector<double> xcd, ycd;
    std::vector<double> xc, yc, sx, sy, rbc, mrho, mu, mdrho, mdu, corr;
    std::vector<float> xcl, ycl;
    std::vector<double> rhoj, uj, wfv, dtv, bdtv;
    long long qoff = 0, woff = 0, soff = 0;
    int xoff = 0, yoff = 0;
    double sigmaf = params[0]->sigmaf;
    const int warm = warmup(sigmaf, precision == NS_PREC_SPLIT32 ? std::ldexp(1.0, -32)
                                                               : std::ldexp(1.0, -60), 16);
    for (int q = 0; q < n && rc == NS_OK; q++) {
        const ns_params *p = params[q];
        const int imax = p->imax, jmax = p->jmax;
        auto ub = [&](int k, int i, int j) -> double {
            if (p->ub_layout == NS_LAYOUT_ROWS) return p->Ub[k + 4 * (size_t)j];
            return p->ub_layout == NS_LAYOUT_FORTRAN ? p->Ub[k + 4 * ((size_t)i + (size_t)imax * j)]
                                                     : p->Ub[((size_t)k * jmax + j) * imax + i];
        };
        const double pb = ub(3, 0, 0);
        std::vector<double> rj(jmax), uj2(jmax);
        for (int j = 0; j < jmax; j++) {
            rj[j] = ub(0, 0, j);
            uj2[j] = ub(1, 0, j);
            for (int i = 0; i < imax; i++)
                if (ub(0, i, j) != rj[j] || ub(1, i, j) != uj2[j] || ub(2, i, j) != 0.0 || ub(3, i, j) != pb)
                    rc = berr(b, NS_ERR_UNSUPPORTED,
                              "ns_batch_create: instance " + std::to_string(q) +
                                  ": the base flow must be uniform in x with v = 0 and uniform p");
        }
        if (rc != NS_OK) break;
        ns::batch::Inst &in = hin[q];
        in.imax = imax;
        in.jmax = jmax;
        in.D = p->D;
        in.pitch = (imax + 31) / 32 * 32;
        in.q_off = qoff;
        in.w_off = woff;
        qoff += 4LL * in.pitch * jmax;
        woff += 4LL * in.pitch * jmax;
        in.x_off = xoff;
        in.y_off = yoff;
        in.dt_d = p->dt;
        in.pmean_d = pb;
        in.gamma_d = p->gamma;
        in.p_bc_d = 1.0 / p->gamma - pb;
        in.dt_f = (float)in.dt_d;
        in.pmean_f = (float)in.pmean_d;
        in.gamma_f = (float)in.gamma_d;
        in.p_bc_f = (float)in.p_bc_d;
        in.warm = warm;
        if (p->source_mode != NS_SRC_NONE) {
            in.s_off = soff;
            soff += (long long)in.pitch * jmax;
            b->has_src = true;
        } else {
            in.s_off = -1;
        }
        // chunks: items of roughly 256 positions
        auto nchunks = [&](int nn) {
            if (warm < 0) return 1;
            int c = (nn - 12) / 256;
            const int maxc = (nn - 12) / (4 * (warm + 6));
            c = std::min(c, maxc);
            return std::max(c, 1);
        };
        in.fx_chunks = nchunks(imax);
        in.fy_chunks = nchunks(jmax);
        coef_table(xcd, imax, p->dm, p->meshx, p->D, p->metric_mode);
        coef_table(ycd, jmax, p->dn, p->meshy, p->D, p->metric_mode);
        for (double v : xcd) {
            xc.push_back(v);
            xcl.push_back((float)(v - (double)(float)v));
        }
        for (double v : ycd) {
            yc.push_back(v);
            ycl.push_back((float)(v - (double)(float)v));
        }
        for (int i = 0; i < imax; i++) sx.push_back(p->sigmax[i]);
        for (int j = 0; j < jmax; j++) {
            sy.push_back(p->sigmay[j]);
            rbc.push_back(p->rhob[j] - rj[j]);
            mrho.push_back(rj[j]);
            mu.push_back(uj2[j]);
            mdrho.push_back(line_deriv(rj.data(), j, jmax, &ycd[(size_t)j * ns::kCoefStride]));
            mdu.push_back(line_deriv(uj2.data(), j, jmax, &ycd[(size_t)j * ns::kCoefStride]));
            rhoj.push_back(rj[j]);
            uj.push_back(uj2[j]);
        }
        std::vector<double> col(jmax), f(jmax);
        for (int k = 0; k < 4; k++) {
            for (int j = 0; j < jmax; j++) col[j] = k == 0 ? rj[j] : k == 1 ? uj2[j] : k == 2 ? 0.0 : pb;
            f = col;
            serial_filter_line(f.data(), jmax, sigmaf, kDfbY);
            for (int j = 0; j < jmax; j++) corr.push_back(f[j] - col[j]);
        }
        b->hpmean.push_back(pb);
        wfv.push_back(p->wf);
        dtv.push_back(p->dt);
        for (int k = 0; k < 6; k++) bdtv.push_back(kBeta[k] * p->dt);
        xoff += imax;
        yoff += jmax;
    }
    if (rc != NS_OK) {
        delete b;
        return rc;
    }
    b->hinst = hin;
    b->hrho = rhoj;
    b->hu = uj;
    b->qsize = (size_t)qoff;
    b->wsize = (size_t)woff;
    if (cudaSetDevice(b->dev) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return berr(nullptr, NS_ERR_CUDA, "ns_batch_create: device or stream");
    }
    b->stream = b->own;
    // work lists
    std::vector<int4> tiles8, tiles16, fxl, fyl;
    std::vector<int2> bcl;
    for (int q = 0; q < n; q++) {
        const auto &in = hin[q];
        for (int j0 = 0; j0 < in.jmax; j0 += 8)
            for (int i0 = 0; i0 < in.imax; i0 += 32) tiles8.push_back(make_int4(q, i0, j0, 0));
        for (int j0 = 0; j0 < in.jmax; j0 += 16)
            for (int i0 = 0; i0 < in.imax; i0 += 32) tiles16.push_back(make_int4(q, i0, j0, 0));
        for (int k = 0; k < 4; k++) {
            for (int r0 = 0; r0 < in.jmax; r0 += 32)
                for (int c = 0; c < in.fx_chunks; c++) fxl.push_back(make_int4(q, k, r0, c));
            for (int c0 = 0; c0 < in.imax; c0 += 32)
                for (int c = 0; c < in.fy_chunks; c++) fyl.push_back(make_int4(q, k, c0, c));
        }
        // the perimeter in pieces of 32 positions, one warp each
        for (int t0 = 0; t0 < std::max(in.imax, in.jmax); t0 += 32) bcl.push_back(make_int2(q, t0));
    }
    // filter items largest first: a chunk after the first also runs the warm-up
    auto item_cost = [&](const int4 &it, bool along_x) {
        const auto &in = hin[it.x];
        const int n = along_x ? in.imax : in.jmax;
        const int chunks = along_x ? in.fx_chunks : in.fy_chunks;
        return (n - 12) / chunks + (it.w > 0 && in.warm > 0 ? in.warm : 0);
    };
    std::stable_sort(fxl.begin(), fxl.end(), [&](const int4 &p, const int4 &q) {
        return item_cost(p, true) > item_cost(q, true);
    });
    std::stable_sort(fyl.begin(), fyl.end(), [&](const int4 &p, const int4 &q) {
        return item_cost(p, false) > item_cost(q, false);
    });
    b->ntiles[0] = (int)tiles8.size();
    b->ntiles[1] = (int)tiles16.size();
    b->nfx = (int)fxl.size();
    b->nfy = (int)fyl.size();
    b->nbc = (int)bcl.size();
    size_t maxplane = 0;
    for (const auto &in : hin) maxplane = std::max(maxplane, (size_t)in.pitch * in.jmax);
    b->stagebuf_elems = 8 * maxplane;
#define B_TRY(x)                  \
    do {                          \
        rc = (x);                 \
        if (rc != NS_OK) goto fail; \
    } while (0)
    B_TRY(balloc(b, (unsigned char **)&b->q[0], b->qsize * es));
    B_TRY(balloc(b, (unsigned char **)&b->q[1], b->qsize * es));
    B_TRY(balloc(b, &b->W, b->wsize));
    B_TRY(balloc(b, &b->stage_sin, (size_t)8 * n));
    B_TRY(balloc(b, &b->wf, (size_t)n));
    B_TRY(balloc(b, &b->dtv, (size_t)n));
    B_TRY(balloc(b, &b->bdt, (size_t)6 * n));
    B_TRY(balloc(b, &b->drho, rhoj.size()));
    B_TRY(balloc(b, &b->du, uj.size()));
    B_TRY(balloc(b, &b->stagebuf, b->stagebuf_elems));
    B_TRY(balloc(b, &b->inst, (size_t)n));
    B_TRY(balloc(b, &b->tiles[0], tiles8.size()));
    B_TRY(balloc(b, &b->tiles[1], tiles16.size()));
    B_TRY(balloc(b, &b->fx, fxl.size()));
    B_TRY(balloc(b, &b->fy, fyl.size()));
    B_TRY(balloc(b, &b->bc, bcl.size()));
    B_TRY(balloc(b, &b->xcl, xcl.size()));
    B_TRY(balloc(b, &b->ycl, ycl.size()));
    B_TRY(tput(b, &b->xc, xc, es));
    B_TRY(tput(b, &b->yc, yc, es));
    B_TRY(tput(b, &b->sigx, sx, es));
    B_TRY(tput(b, &b->sigy, sy, es));
    B_TRY(tput(b, &b->rho_bc, rbc, es));
    B_TRY(tput(b, &b->mrho, mrho, es));
    B_TRY(tput(b, &b->mu, mu, es));
    B_TRY(tput(b, &b->mdrho, mdrho, es));
    B_TRY(tput(b, &b->mdu, mdu, es));
    B_TRY(tput(b, &b->corr, corr, es));
    B_TRY(balloc(b, (unsigned char **)&b->src, std::max<long long>(soff, 1) * es));
    B_TRY(balloc(b, &b->bar, 2 + 12));
    B_TRY(balloc(b, &b->err, 1));
    B_TRY(balloc(b, &b->d_iter, 1));
    {
        // the halo-tile maps of every instance, buffer and tile height: planes
        // of jmax rows of pitch elements from the instance's plane 0; box
        // 40 x (TY + 6) x 4 from (i0-4, j0-3), zeros outside the instance
        const auto encode = ns::tensor_encoder();
        if (!encode) {
            rc = berr(b, NS_ERR_UNSUPPORTED, "ns_batch_create: cuTensorMapEncodeTiled is unavailable");
            goto fail;
        }
        std::vector<CUtensorMap> maps((size_t)4 * n);
        for (int t16 = 0; t16 < 2; t16++)
            for (int q = 0; q < n; q++)
                for (int bf = 0; bf < 2; bf++) {
                    const auto &in = hin[q];
                    const cuuint64_t dims[3] = {(cuuint64_t)in.imax, (cuuint64_t)in.jmax, 4};
                    const cuuint64_t strides[2] = {(cuuint64_t)in.pitch * es,
                                                   (cuuint64_t)in.pitch * in.jmax * es};
                    const cuuint32_t box[3] = {(cuuint32_t)(ns::batch::kTX + 8),
                                               (cuuint32_t)((t16 ? 16 : 8) + 2 * ns::batch::kH), 4};
                    const cuuint32_t estr[3] = {1u, 1u, 1u};
                    void *base = (unsigned char *)b->q[bf] + (size_t)in.q_off * es;
                    const CUresult r = encode(
                        &maps[((size_t)t16 * n + q) * 2 + bf],
                        es == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                        3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
                    if (r != CUDA_SUCCESS) {
                        rc = berr(b, NS_ERR_CUDA, "ns_batch_create: cuTensorMapEncodeTiled failed");
                        goto fail;
                    }
                }
        rc = balloc(b, &b->qmaps, maps.size());
        if (rc == NS_OK) rc = bput(b, b->qmaps, maps);
        if (rc == NS_OK && cudaStreamSynchronize(b->stream) != cudaSuccess)
            rc = berr(b, NS_ERR_CUDA, "ns_batch_create: tensor map upload");
        if (rc != NS_OK) goto fail;
    }
    if (cudaMemsetAsync(b->q[0], 0, b->qsize * es, b->stream) != cudaSuccess ||
        cudaMemsetAsync(b->q[1], 0, b->qsize * es, b->stream) != cudaSuccess ||
        cudaMemsetAsync(b->W, 0, b->wsize * 8, b->stream) != cudaSuccess ||
        cudaMemsetAsync(b->stage_sin, 0, 8 * n * sizeof(double), b->stream) != cudaSuccess ||
        cudaMemsetAsync(b->bar, 0, 2 * sizeof(unsigned), b->stream) != cudaSuccess ||
        cudaMemsetAsync(b->err, 0, sizeof(int), b->stream) != cudaSuccess ||
        cudaMemsetAsync(b->d_iter, 0, sizeof(int), b->stream) != cudaSuccess) {
        rc = berr(b, NS_ERR_CUDA, "ns_batch_create: memset");
        goto fail;
    }
    B_TRY(bput(b, b->inst, hin));
    B_TRY(bput(b, b->tiles[0], tiles8));
    B_TRY(bput(b, b->tiles[1], tiles16));
    B_TRY(bput(b, b->fx, fxl));
    B_TRY(bput(b, b->fy, fyl));
    B_TRY(bput(b, b->bc, bcl));
    B_TRY(bput(b, b->xcl, xcl));
    B_TRY(bput(b, b->ycl, ycl));
    B_TRY(bput(b, b->drho, rhoj));
    B_TRY(bput(b, b->du, uj));
    B_TRY(bput(b, b->wf, wfv));
    B_TRY(bput(b, b->dtv, dtv));
    B_TRY(bput(b, b->bdt, bdtv));
    if (b->has_src) {
        // spatial source fields (rk.f90:188-189), in the state's precision
        for (int q = 0; q < n; q++) {
            const ns_params *p = params[q];
            const auto &in = hin[q];
            if (in.s_off < 0) continue;
            std::vector<double> fld((size_t)in.pitch * in.jmax, 0.0);
            for (int j = 0; j < in.jmax; j++)
                for (int i = 0; i < in.imax; i++) {
                    double v;
                    if (p->source_mode == NS_SRC_GAUSSIAN) {
                        const double dx = p->m[i] - p->m_pt, dy = p->n[j] - p->n_pt;
                        v = p->amplitude * std::exp(-(std::log(2.0) * (dx * dx + dy * dy) / (p->r0 * p->r0)));
                    } else {
                        v = p->src_field[(size_t)j * in.imax + i];
                    }
                    fld[(size_t)j * in.pitch + i] = v;
                }
            cudaError_t e;
            if (precision == NS_PREC_SPLIT32) {
                std::vector<float> ff(fld.begin(), fld.end());
                e = cudaMemcpy((float *)b->src + in.s_off, ff.data(), ff.size() * 4, cudaMemcpyHostToDevice);
            } else {
                e = cudaMemcpy((double *)b->src + in.s_off, fld.data(), fld.size() * 8, cudaMemcpyHostToDevice);
            }
            if (e != cudaSuccess) {
                rc = berr(b, NS_ERR_CUDA, "ns_batch_create: source upload");
                goto fail;
            }
        }
    }
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) {
        rc = berr(b, NS_ERR_CUDA, "ns_batch_create: setup");
        goto fail;
    }
    {
        ns::batch::Args &a = b->args;
        a.inst = b->inst;
        a.fx = b->fx;
        a.fy = b->fy;
        a.bc = b->bc;
        a.nfx = b->nfx;
        a.nfy = b->nfy;
        a.nbc = b->nbc;
        a.ninst = b->n;
        a.qmaps = b->qmaps;
        a.q0 = b->q[0];
        a.q1 = b->q[1];
        a.W = b->W;
        a.xc = b->xc; a.xcl = b->xcl; a.yc = b->yc; a.ycl = b->ycl;
        a.sigx = b->sigx; a.sigy = b->sigy; a.rho_bc = b->rho_bc;
        a.mrho = b->mrho; a.mu = b->mu; a.mdrho = b->mdrho; a.mdu = b->mdu; a.corr = b->corr;
        a.src = b->src;
        a.stage_sin = b->stage_sin;
        a.bdt = b->bdt;
        for (int k = 0; k < 6; k++) {
            a.alpha[k] = kAlpha[k];
            a.beta[k] = kBeta[k];
        }
        a.fm_d[0] = 1.0 - sigmaf * kDf[0];   // used by the FP64 form only
        for (int s = 1; s <= 6; s++) a.fm_d[s] = -sigmaf * kDf[s];
        const double *dfb[2] = {kDfbX, kDfbY};
        for (int d = 0; d < 2; d++) {
            a.fbm1_d[d] = -sigmaf * dfb[d][0];
            double sum = 0.0;
            for (int z = 0; z < 7; z++) sum += dfb[d][z];
            a.fbsum_d[d] = -sigmaf * sum;
            a.fb_d[d][0] = 1.0 - sigmaf * dfb[d][1];   // used by the FP64 form only
            for (int z = 1; z <= 5; z++) a.fb_d[d][z] = -sigmaf * dfb[d][z + 1];
        }
        for (int s = 0; s < 7; s++) a.fm_f[s] = (float)a.fm_d[s];
        a.fm_f[0] = 0.f;
        for (int d = 0; d < 2; d++) {
            a.fbm1_f[d] = (float)a.fbm1_d[d];
            a.fbsum_f[d] = (float)a.fbsum_d[d];
            for (int z = 0; z < 6; z++) a.fb_f[d][z] = (float)a.fb_d[d][z];
            a.fb_f[d][0] = 0.f;
        }
        a.bar_count = b->bar;
        a.bar_gen = b->bar + 1;
        a.work = b->bar + 2;
        a.err = b->err;
        a.spin_limit = 20000000;  // x 64 ns sleeps: about 1-2 s per barrier
    }
    rc = configure(b, 16, 16, 0);
    if (rc != NS_OK) goto fail;
#undef B_TRY
    *out = b;
    return NS_OK;
fail:
    bfree(b);
    delete b;
    return rc;
}

void ns_batch_destroy(ns_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->dev);
    cudaStreamSynchronize(b->stream);
    bfree(b);
    delete b;
}

// Host state of instance q (layout as ns_set_state) -> q' (FP32 or FP64).
int ns_batch_set_state(ns_batch *b, int q, const double *U, int layout)
{
    if (!b || !U || q < 0 || q >= b->n) return berr(b, NS_ERR_PARAM, "ns_batch_set_state: bad argument");
    cudaSetDevice(b->dev);
    const auto &in = b->hinst[q];
    const size_t row = (size_t)in.imax * 8;
    double *stg = b->stagebuf;                 // 4 FP64 planes with pitch in.pitch
    double *raw = b->stagebuf + 4 * (size_t)in.pitch * in.jmax;
    cudaError_t e;
    ns::Dims d;
    d.imax = in.imax;
    d.jmax = in.jmax;
    d.pitch = in.pitch;
    d.nk = 4;
    d.D = in.D;
    d.plane = (long long)in.pitch * in.jmax;
    if (layout == NS_LAYOUT_SOA) {
        e = cudaMemcpy2DAsync(stg, in.pitch * 8, U, row, row, (size_t)in.jmax * 4,
                              cudaMemcpyHostToDevice, b->stream);
    } else if (layout == NS_LAYOUT_FORTRAN) {
        e = cudaMemcpyAsync(raw, U, (size_t)4 * in.imax * in.jmax * 8, cudaMemcpyHostToDevice, b->stream);
        if (e == cudaSuccess) e = ns::launch_aos_to_soa(raw, stg, d, b->stream);
    } else {
        return berr(b, NS_ERR_PARAM, "ns_batch_set_state: layout");
    }
    const dim3 blk(32, 8), grd((in.imax + 31) / 32, (in.jmax + 7) / 8);
    if (e == cudaSuccess) {
        if (b->precision == NS_PREC_SPLIT32)
            ns::batch::k_batch_from_full<float><<<grd, blk, 0, b->stream>>>(
                stg, in.imax, in.jmax, in.pitch, b->drho + in.y_off, b->du + in.y_off,
                b->hpmean[q], (float *)b->q[0] + in.q_off, in.pitch);
        else
            ns::batch::k_batch_from_full<double><<<grd, blk, 0, b->stream>>>(
                stg, in.imax, in.jmax, in.pitch, b->drho + in.y_off, b->du + in.y_off,
                b->hpmean[q], (double *)b->q[0] + in.q_off, in.pitch);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return berr(b, NS_ERR_CUDA, std::string("ns_batch_set_state: ") + cudaGetErrorString(e));
    b->have_state = true;
    return NS_OK;
}

int ns_batch_get_state(ns_batch *b, int q, double *U, int layout)
{
    if (!b || !U || q < 0 || q >= b->n) return berr(b, NS_ERR_PARAM, "ns_batch_get_state: bad argument");
    cudaSetDevice(b->dev);
    const auto &in = b->hinst[q];
    const size_t row = (size_t)in.imax * 8;
    double *stg = b->stagebuf;
    double *raw = b->stagebuf + 4 * (size_t)in.pitch * in.jmax;
    const dim3 blk(32, 8), grd((in.imax + 31) / 32, (in.jmax + 7) / 8);
    if (b->precision == NS_PREC_SPLIT32)
        ns::batch::k_batch_to_full<float><<<grd, blk, 0, b->stream>>>(
            (float *)b->q[0] + in.q_off, in.imax, in.jmax, in.pitch, b->drho + in.y_off,
            b->du + in.y_off, b->hpmean[q], stg, in.pitch);
    else
        ns::batch::k_batch_to_full<double><<<grd, blk, 0, b->stream>>>(
            (double *)b->q[0] + in.q_off, in.imax, in.jmax, in.pitch, b->drho + in.y_off,
            b->du + in.y_off, b->hpmean[q], stg, in.pitch);
    cudaError_t e = cudaGetLastError();
    ns::Dims d;
    d.imax = in.imax;
    d.jmax = in.jmax;
    d.pitch = in.pitch;
    d.nk = 4;
    d.D = in.D;
    d.plane = (long long)in.pitch * in.jmax;
    if (e == cudaSuccess) {
        if (layout == NS_LAYOUT_SOA) {
            e = cudaMemcpy2DAsync(U, row, stg, in.pitch * 8, row, (size_t)in.jmax * 4,
                                  cudaMemcpyDeviceToHost, b->stream);
        } else if (layout == NS_LAYOUT_FORTRAN) {
            e = ns::launch_soa_to_aos(stg, raw, d, b->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(U, raw, (size_t)4 * in.imax * in.jmax * 8, cudaMemcpyDeviceToHost, b->stream);
        } else {
            return berr(b, NS_ERR_PARAM, "ns_batch_get_state: layout");
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return berr(b, NS_ERR_CUDA, std::string("ns_batch_get_state: ") + cudaGetErrorString(e));
    return NS_OK;
}

int ns_batch_step(ns_batch *b, int iter0, int nsteps)
{
    if (!b || nsteps < 0) return berr(b, NS_ERR_PARAM, "ns_batch_step: bad argument");
    if (!b->have_state) return berr(b, NS_ERR_STATE, "ns_batch_step before ns_batch_set_state");
    cudaSetDevice(b->dev);
    if (!b->no_graph && ensure_graph(b) != NS_OK) b->no_graph = true;  // launch directly
    if (b->has_src) ns::batch::k_batch_set_iter<<<1, 1, 0, b->stream>>>(b->d_iter, iter0);
    for (int s = 0; s < nsteps; s++) {
        const cudaError_t e = b->no_graph ? launch_step(b, b->stream)
                                          : cudaGraphLaunch(b->exec, b->stream);
        if (e != cudaSuccess)
            return berr(b, NS_ERR_CUDA, std::string("ns_batch_step: ") + cudaGetErrorString(e));
    }
    return NS_OK;
}

// One step (advancing the state, launched directly) with the phase stamps on:
// ms[0..3] = the time of phases A..D summed over the six stages, each from
// the barrier before it to the barrier after it (barrier cost included).
int ns_batch_phase_times(ns_batch *b, int iter0, double *ms)
{
    if (!b || !ms) return berr(b, NS_ERR_PARAM, "ns_batch_phase_times: NULL argument");
    if (!b->have_state) return berr(b, NS_ERR_STATE, "ns_batch_phase_times before ns_batch_set_state");
    cudaSetDevice(b->dev);
    constexpr int kStamps = 1 + 6 * 4;
    unsigned long long *d = nullptr, h[kStamps] = {};
    if (cudaMalloc(&d, sizeof h) != cudaSuccess) return berr(b, NS_ERR_OOM, "ns_batch_phase_times");
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof h, b->stream);
    if (e == cudaSuccess && b->has_src) {
        ns::batch::k_batch_set_iter<<<1, 1, 0, b->stream>>>(b->d_iter, iter0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = launch_step(b, b->stream, d);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    cudaFree(d);
    if (e != cudaSuccess)
        return berr(b, NS_ERR_CUDA, std::string("ns_batch_phase_times: ") + cudaGetErrorString(e));
    const int rc = check_err(b);
    if (rc != NS_OK) return rc;
    for (int p = 0; p < 4; p++) ms[p] = 0.0;
    for (int st = 0; st < 6; st++)
        for (int p = 0; p < 4; p++)
            ms[p] += (double)(h[1 + 4 * st + p] - h[4 * st + p]) * 1e-6;
    return NS_OK;
}

int ns_batch_synchronize(ns_batch *b)
{
    if (!b) return berr(nullptr, NS_ERR_PARAM, "ns_batch_synchronize: NULL");
    cudaSetDevice(b->dev);
    if (cudaStreamSynchronize(b->stream) != cudaSuccess)
        return berr(b, NS_ERR_CUDA, std::string("ns_batch_synchronize: ") + cudaGetErrorString(cudaGetLastError()));
    return check_err(b);
}

int ns_batch_set_stream(ns_batch *b, void *stream)
{
    if (!b) return berr(nullptr, NS_ERR_PARAM, "ns_batch_set_stream: NULL");
    b->stream = stream ? (cudaStream_t)stream : b->own;
    return NS_OK;
}

// Tile autotuner: times each tile height (8, 16 rows) and residency (1 block
// per SM up to the maximum) for `reps` steps on the current state, keeps the
// fastest, and leaves the state advanced by the steps it ran.
int ns_batch_autotune(ns_batch *b, int iter0, int reps, int *ty, int *blocks_per_sm, double *ms)
{
    if (!b || reps < 1) return berr(b, NS_ERR_PARAM, "ns_batch_autotune: bad argument");
    if (!b->have_state) return berr(b, NS_ERR_STATE, "ns_batch_autotune before ns_batch_set_state");
    cudaSetDevice(b->dev);
    double best = 1e300;
    int bty = 16, bpw = 16, bbps = 0;
    int it = iter0;
    const bool f32 = b->precision == NS_PREC_SPLIT32;
    for (int t : {8, 16})
    for (int pw : {16, 24, 32}) {
        if (!f32 && pw != 16) continue;  // FP32: 16, 24 or 32; FP64: 16
        const size_t sm = smem_for(b->precision, t, pw);
        const int maxb = occupancy(step_kernel(b->precision, t, pw), sm);
        for (int bps = 1; bps <= maxb; bps++) {
            int rc = configure(b, t, pw, bps);
            if (rc != NS_OK) return rc;
            if (!b->no_graph && ensure_graph(b) != NS_OK) b->no_graph = true;
            auto one = [&]() {
                return b->no_graph ? launch_step(b, b->stream) : cudaGraphLaunch(b->exec, b->stream);
            };
            if (b->has_src) ns::batch::k_batch_set_iter<<<1, 1, 0, b->stream>>>(b->d_iter, it);
            one();  // warm-up
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            cudaEventRecord(e0, b->stream);
            for (int r = 0; r < reps; r++) one();
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            float t_ms = 0.f;
            cudaEventElapsedTime(&t_ms, e0, e1);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            it += reps + 1;
            rc = check_err(b);
            if (rc != NS_OK) return rc;
            if (t_ms / reps < best) {
                best = t_ms / reps;
                bty = t;
                bpw = pw;
                bbps = bps;
            }
        }
    }
    int rc = configure(b, bty, bpw, bbps);
    if (rc != NS_OK) return rc;
    b->tuned_ms = best;
    if (ty) *ty = bty;
    if (blocks_per_sm) *blocks_per_sm = b->blocks_per_sm;
    if (ms) *ms = best;
    return NS_OK;
}

// Test hook for the bounded barrier: the next step waits for `extra` blocks
// that never come, with a spin limit of `spin_limit`; the step must then
// return NS_ERR_TIMEOUT from ns_batch_synchronize and leave the context usable.
int ns_batch_barrier_test(ns_batch *b, int extra, long long spin_limit)
{
    if (!b || extra < 0 || spin_limit < 1) return berr(b, NS_ERR_PARAM, "ns_batch_barrier_test: bad argument");
    cudaSetDevice(b->dev);
    ns::batch::Args saved = b->args;
    b->args.spin_limit = spin_limit;
    const int g = b->grid;
    b->grid = g;
    // launch directly (no graph) with a participant count that cannot be met
    ns::batch::Args a = b->args;
    a.tiles = b->tiles[b->ty == 8 ? 0 : 1];
    a.ntiles = b->ntiles[b->ty == 8 ? 0 : 1];
    a.nblocks = (unsigned)(g + extra);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)g);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = b->smem;
    cfg.stream = b->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, step_kernel(b->precision, b->ty, b->pw), a);
    b->args = saved;
    if (e != cudaSuccess) return berr(b, NS_ERR_CUDA, std::string("ns_batch_barrier_test: ") + cudaGetErrorString(e));
    return ns_batch_synchronize(b);
}

int ns_batch_info(ns_batch *b, int *grid, int *ty, int *blocks_per_sm, int *items)
{
    if (!b) return berr(nullptr, NS_ERR_PARAM, "ns_batch_info: NULL");
    if (grid) *grid = b->grid;
    if (ty) *ty = b->ty;
    if (blocks_per_sm) *blocks_per_sm = b->blocks_per_sm;
    if (items) {
        items[0] = b->ntiles[b->ty == 8 ? 0 : 1];
        items[1] = b->nfx;
        items[2] = b->nfy;
        items[3] = b->n;
    }
    return NS_OK;
}

}  // extern "C"
