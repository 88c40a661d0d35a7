// ns_internal.cuh -- shared definitions of the GB300 time-step library.
//
// Device layout (all FP64 unless noted): every 2-D field is a plane of
// jmax rows of `pitch` doubles (pitch = imax rounded up to 32, so each row
// starts on a 256-byte boundary); variable k of a multi-variable field is
// plane k.  Index (i,j) (0-based; the reference's (i+1,j+1)) is at
// j*pitch + i.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/ns_gb300.h"

namespace ns {

constexpr int kMaxNk = 5;

// Planes of the auxiliary field `aux`.
enum AuxPlane {
    AUX_T = 0,     // T = gamma*p/rho                      (rhs.f90:20)
    AUX_RINV = 1,  // 1/rho
    AUX_TAU1 = 2,  // tau_xx                               (eqeuler.f90:37)
    AUX_TAU2 = 3,  // tau_xy                               (eqeuler.f90:38)
    AUX_TAU3 = 4,  // tau_yy                               (eqeuler.f90:39)
    AUX_KTX = 5,   // k * dT/dx                            (derivs.f90:48-56)
    AUX_KTY = 6,   // k * dT/dy
    AUX_PSID = 7,  // rho*alpha_cond*(dpsi/dx+dpsi/dy)      (derivs.f90:37)
    AUX_COUNT = 8
};

struct Dims {
    int imax, jmax, pitch, nk, D;
    long long plane;  // pitch * jmax
};

// Per-line derivative coefficients: 8 doubles per line position q.  For an
// interior position entries 4..6 hold a_s*metric/h (s = 1..3) and the
// derivative is sum_s c_s*(f[q+s]-f[q-s]); for the three closure positions
// at each end, entries 0..6 hold the 7 one-sided coefficients for offsets
// o0..o0+6 (o0 = -q at the left end, n-7-q at the right end).
constexpr int kCoefStride = 8;
// Points per block of the FP64 filter recurrences (loads issued one block
// ahead).
constexpr int kFilterPf = 8;
// Warps per SM sub-partition of the FP64 filter sweeps (k_filter deals the
// pass-2 work out in equal segments, one per warp).
constexpr int kFilterWarpsPerSmsp = 2;

// ---------------------------------------------------------------------------
// DRP first derivative along a line (diff.f90:40-238 with the metric of
// diff.f90:276-350 folded into the coefficients).
// f points at position q of a line of length n and stride st; c = the 8
// coefficients of position q.
// ---------------------------------------------------------------------------
// Interior 7-point DRP sum c1*(f1-f-1) + c2*(f2-f-2) + c3*(f3-f-3) along
// stride st (global memory or a shared-memory tile: the same operations in
// the same order, so both give identical bits).
template <typename S>
__device__ __forceinline__ double dint(const double *__restrict__ f, S st, double c1, double c2,
                                       double c3)
{
    double r = c1 * (f[st] - f[-st]);
    r = fma(c2, f[2 * st] - f[-2 * st], r);
    r = fma(c3, f[3 * st] - f[-3 * st], r);
    return r;
}

__device__ __forceinline__ double dline(const double *__restrict__ f, long long st, int q,
                                        int n, const double *__restrict__ c)
{
    if (q >= 3 && q < n - 3) return dint(f, st, c[4], c[5], c[6]);
    const int o0 = (q < 3) ? -q : (n - 7 - q);
    const double *g = f + (long long)o0 * st;
    double r = c[0] * g[0];
#pragma unroll
    for (int z = 1; z < 7; z++) r = fma(c[z], g[(long long)z * st], r);
    return r;
}

// Halo tile of the FP64 first-derivative kernel: a block of 32 x 8 points
// reads a box of 40 x 14 doubles per plane starting 4 columns left (the box's
// x coordinate times 8 bytes must be a multiple of 16) and 3 rows below.
constexpr int kFirstBX = 32, kFirstBY = 8;
constexpr int kFirstTileL = 4, kFirstTileW = 40, kFirstTileH = kFirstBY + 6;

// Split-precision stage kernel: blocks of 32 x kSplitTY points (8 thread
// rows, kSplitTY/8 points per thread), at least kSplitMinBlocks resident per
// SM; its TMA box is 40 x (kSplitTY + 6) x planes.
constexpr int kSplitTY = 16, kSplitMinBlocks = 4;

// Transport law mu(T), k(T) (coefficients.f90:27-59) as piecewise
// polynomials in T: T = 2^e (1 + (j + f)/256), e in [kTrEmin, kTrEmin +
// kTrOctaves), j the top 8 fraction bits; piece (e, j) holds kTrDeg+1
// coefficients of mu then of k in u = T - 2^e (1 + j/256) (exact, by
// Sterbenz), Chebyshev interpolants of degree 5 on the piece.  T outside
// that range takes the exp/log path.
constexpr int kTrEmin = -2, kTrOctaves = 5, kTrDeg = 5;
constexpr int kTrPieces = kTrOctaves * 256;
constexpr int kTrStride = 2 * (kTrDeg + 1);  // doubles per piece

// Filter coefficients pre-multiplied by the filter strength.
struct FilterCoef {
    double c0;       // 1 - sigmaf*df(0)
    double m[7];     // m[s] = -sigmaf*df(s), s = 1..6 (m[0] unused)
    double b0;       // 1 - sigmaf*dfb(0)
    double bm1;      // -sigmaf*dfb(-1)
    double b[6];     // b[s] = -sigmaf*dfb(s), s = 1..5 (b[0] unused)
};

struct Physics {
    double gamma, inv_re, inv_re_pr, gm1_re, dt, inv_pe, alpha_cond;
    double Tref, mu0inv, k0inv;
    double A_mi, B_mi, C_mi, D_mi, A_k, B_k, C_k, D_k;
    // D_mi + log(mu0inv), D_k + log(k0inv): mu = exp(A ln x + B/x + C/x^2 + D_mi_s)
    double D_mi_s, D_k_s;
};

struct StageCoef {
    double alpha, beta;
    int stage;
};

// Base flow seen by the split-precision stage (uniform in x, v = 0,
// uniform p): per-row density and velocity, their FP64 DRP y-derivatives
// rounded to FP32, and the constants.
struct SplitMean {
    const float *rho, *u, *drho, *du;
    const float *ulo;  // u_b - FP32(u_b) per row
    float p, gamma;
};

// Constants of the split-precision viscous terms (Navier-Stokes with a
// base flow uniform in x and y, v = 0): T' = T - T_b from rho' and p',
// mu(T) and k(T) from the FP32 copy of the transport table (or, outside it,
// the fit by expf/logf with x = Tref*T), and the factors of
// eqeuler.f90:68-92.
struct SplitVisc {
    float rho_b, p_b, gamma, T_b;     // uniform base flow, T_b = gamma*p_b/rho_b
    float inv_re, gm1_re, inv_re_pr;  // 1/Re, (gamma-1)/Re, 1/(Re*Pr)
    float Tref, A_mi, B_mi, C_mi, D_mi_s, A_k, B_k, C_k, D_k_s;
};

// Device state of the split-precision path (precision = NS_PREC_SPLIT).
struct SplitState {
    int fpitch = 0;                   // FP32 row pitch (elements)
    // variables carried as hi + lo pairs: u', v', p' (3, NS_PREC_SPLIT) or none
    // (0, NS_PREC_SPLIT32); a buffer holds 4 + np FP32 planes: rho', u', v',
    // p', then the lo parts
    int np = 3;
    float *q[2] = {nullptr, nullptr}; // perturbation ping-pong
    CUtensorMap qmap[2];              // TMA maps of q[0], q[1]: (imax, jmax, 4 + np) FP32
    float *xc = nullptr, *yc = nullptr;
    float *xcl = nullptr, *ycl = nullptr;  // FP64 table minus its FP32 rounding
    float *sigx = nullptr, *sigy = nullptr, *src = nullptr;
    float *rho_bc = nullptr;          // rhob(j) - rho_b(j)
    float *ycorr = nullptr;           // [4][jmax]: y filter applied to Ub, minus Ub
    float *mean_buf = nullptr;        // rho, u, drho, du: [4][jmax]
    SplitMean mean{};
    double p_bc = 0.0;                // 1/gamma - p_b
    int warm = 0, fx_chunks = 1, fy_chunks = 1;
    // viscous (Navier-Stokes) only: tau_xx', tau_xy', tau_yy', k dT'/dx,
    // k dT'/dy as FP32 planes, their TMA map (imax, jmax, 5), the transport
    // table rounded to FP32 and the constants
    float *tau = nullptr;
    CUtensorMap vmap;
    float *trf = nullptr;
    SplitVisc vis{};
};

}  // namespace ns

struct ns_ctx {
    ns_params p;
    ns::Dims d;
    int dev = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    // device buffers
    double *U = nullptr, *U2 = nullptr, *W = nullptr;
    double *dudm = nullptr, *dudn = nullptr, *aux = nullptr;
    double *Ubase = nullptr, *src = nullptr;
    double *xcoef = nullptr, *ycoef = nullptr;
    double *sigx = nullptr, *sigy = nullptr, *rhob = nullptr, *psib = nullptr;
    double *stage_sin = nullptr;
    double *trtab = nullptr;  // kTrPieces x kTrStride (viscous); null: exp/log path
    int *d_iter = nullptr;
    unsigned long long *d_count = nullptr;
    int *d_err = nullptr;  // set by a kernel whose TMA wait gave up
    // TMA maps of the FP64 stage kernels (box 40 x 14 x planes): U as
    // (imax, jmax, nk) and the T plane of aux (imax, jmax, 1) for k_first;
    // aux as (imax, jmax, AUX_COUNT) for k_update's derivative planes.
    // Unset in ns_step_noalloc, whose kernels read global memory only.
    bool fp64_maps = false;
    CUtensorMap umap{}, tmap{}, amap{};
    double *probe_buf = nullptr;
    int probe_cap = 0;
    int32_t *probe_idx = nullptr;
    // probe recorder (ns_probes_*): rec_cap records of rec_npts*nk values
    double *rec_buf = nullptr;
    int32_t *rec_idx = nullptr;
    int rec_cap = 0, rec_npts = 0, rec_n = 0;
    // output path (ns_vorticity): metric-free derivative tables, omega plane
    double *vx = nullptr, *vy = nullptr, *omega = nullptr;
    // host-side constants
    ns::Physics phys;
    ns::FilterCoef fx, fy;
    double ct[6], alpha[6], beta[6];
    int warm = 0;       // filter warm-up length (-1: serial sweeps)
    int warm32 = 0;     // its first warm32 steps run in FP32 (ns_coef.h fp64_warmups)
    int nsm = 152;      // multiprocessors of the device
    bool visc = false;
    bool split = false;
    ns::SplitState sp;
    bool have_state = false;
    // captured one-step graph
    cudaGraphExec_t step_exec = nullptr;
    // ns_rk_euler on page-locked host memory (FP64): the step without stage
    // 0's k_prim/k_first, a copy stream and one event per row band
    cudaGraphExec_t tail_exec = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t band_ev[9] = {};
    cudaEvent_t wb_ev[9] = {};  // a row band of the last stage is ready to go home
    cudaStream_t graph_stream = nullptr;
    int launches_per_step = 0;
    std::string err;
};

// Kernel launchers (ns_kernels.cu).  All enqueue on `s` and return the
// launch status.
namespace ns {
constexpr int kMaxStepLaunches = 64;
cudaError_t launch_step(ns_ctx *c, cudaStream_t s);
// The step without stage 0's k_prim and k_first and without the last
// stage's y sweep and ccpml, and those kernels over ranges of rows (FP64
// contexts): ns_rk_euler runs them band by band as the rows arrive from the
// host and as they leave for it.
cudaError_t launch_step_tail(ns_ctx *c, cudaStream_t s);
cudaError_t launch_rows(ns_ctx *c, int cls, int row0, int rows, cudaStream_t s);
// Launch shape of the segmented filter sweeps (ns_kernels.cu): `seg`
// pass-2 positions per warp, `blocks` blocks of 128 threads.
void filter_shape(int nlines, int n, int nk, int warm, int nsm, int kw, long long &seg,
                  unsigned &blocks);
// The same for len2 pass-2 positions per line.
void filter_shape_len(int nlines, int len2, int nk, int warm, int nsm, int kw, long long &seg,
                      unsigned &blocks);
// ns_rk_euler on a page-locked host array runs its last stage's y sweep and
// ccpml in row bands and sends each band home while the next is filtered:
// bands_for gives the number of bands and the pass-2 position bounds
// pb[0..nb] (band b covers pb[b] .. pb[b+1]-1, rows 0..5 belong to band 0
// and the last six rows to band nb-1: band_rows).  (ns_kernels.cu)
constexpr int kMaxBands = 8;
int bands_for(const ns_ctx *c, int *pb);
void band_rows(const Dims &d, const int *pb, int nb, int b, int &r0, int &r1);
cudaError_t launch_filter_y_band(ns_ctx *c, int p0, int p1, cudaStream_t s);
cudaError_t launch_bc_band(ns_ctx *c, const int *pb, int nb, int b, cudaStream_t s);
cudaError_t launch_kernel(ns_ctx *c, int cls, int stage, cudaStream_t s);
int step_sequence(const ns_ctx *c, int *cls, int *stage);
cudaError_t launch_set_iter(int *d_iter, int iter, cudaStream_t s);
cudaError_t launch_aos_to_soa(const double *in, double *out, const Dims &d, cudaStream_t s);
cudaError_t launch_soa_to_aos(const double *in, double *out, const Dims &d, cudaStream_t s);
cudaError_t launch_probes(const double *U, const Dims &d, int np, const int32_t *idx,
                          double *out, cudaStream_t s);
cudaError_t launch_count_nonfinite(const double *U, const Dims &d, unsigned long long *count,
                                   cudaStream_t s);
// Per-line derivative table of kCoefStride doubles per position, 1/h and
// the metric folded in (mesh == nullptr: no metric) (ns_api.cu).
void build_line_coef(std::vector<double> &tab, int n, double h, const double *mesh, int D,
                     int metric_mode);
// Tables of the transport-law exp/log (ns_kernels.cu): filled once per
// device, outside stream capture.
cudaError_t ensure_math_tables(int device);
cudaError_t launch_math_eval(int fn, const double *x, double *y, int n, cudaStream_t s);
// mu(T) and k(T) of the transport law as k_first evaluates them (table or
// exp/log path) (ns_kernels.cu)
cudaError_t launch_transport_eval(const ns_ctx *c, const double *T, double *mu, double *k, int n,
                                  cudaStream_t s);
// The piecewise-polynomial table of mu(T), k(T) for these constants
// (ns_api.cu).
void build_transport_table(std::vector<double> &tab, double Tref, const double *a_mi,
                           const double *a_k);
// NS_LAYOUT_ROWS: rows[k + nk*j] -> every point of row j of plane k (ns_output.cu)
cudaError_t launch_rows_to_planes(const double *rows, double *planes, const Dims &d,
                                  cudaStream_t s);
int count_step_launches(const ns_ctx *c);
// Makes msg the text ns_last_error(NULL) returns (ns_api.cu).
void record_error(const char *msg);
// cuTensorMapEncodeTiled through the runtime's driver entry point, or null
// when it is unavailable (ns_api.cu).
PFN_cuTensorMapEncodeTiled_v12000 tensor_encoder();
// TMA map of `planes` planes of the context's pitch x jmax FP64 layout from
// `base`, box box_w x box_h x planes (ns_api.cu); NS_OK or the error code
// set on the context.
int make_plane_map(ns_ctx *c, CUtensorMap *map, double *base, int planes, int box_w, int box_h);
// NS_ERR_CHECK for an error word a failed index check of the checked build
// left (ns_check.cuh), with the file and line as the error text (ns_api.cu).
int check_error(int word);
// Split-precision path (ns_split.cu).
cudaError_t launch_split_kernel(ns_ctx *c, int cls, int stage, cudaStream_t s);
cudaError_t launch_split_from_full(ns_ctx *c, const double *U, cudaStream_t s);
cudaError_t launch_split_to_full(ns_ctx *c, double *U, cudaStream_t s);
}  // namespace ns
