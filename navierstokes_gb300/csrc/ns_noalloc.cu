// ns_noalloc.cu -- ns_step_noalloc: the time step for callers that cannot
// allocate device memory.
//
// Who needs it: hosts whose device memory is owned by something else -- a
// Fortran or C code running inside a framework that hands out a fixed pool,
// a process under a memory cap where a cudaMalloc failure mid-run is not
// acceptable, or a caller that must not trigger allocator synchronisation
// between its own kernels.  They pass the state U on the device and the
// setup arrays on the host; every work array the step needs lives in the
// file-scope array below, which the module reserves when it is loaded and
// every GPU that loads the library keeps until the process exits.
//
// Limits: the work area is NS_NOALLOC_MAX_BYTES (64 MiB); imax and jmax are
// at most NS_NOALLOC_MAX_LINE.  Larger cases get NS_ERR_PARAM.  All calls
// share the one work area, on every stream: calls that overlap on the GPU
// race and give wrong results; calls from several host threads must be
// serialised by the caller (the host-side tables below are shared too).
// Every region of the work area is written before it is read within a call,
// so the contents a previous call left behind never leak into a result.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "ns_internal.cuh"

namespace {

constexpr size_t kScratchDoubles = NS_NOALLOC_MAX_BYTES / sizeof(double);
constexpr int kMaxDevices = 64;

// The work area.  Host code must not use this name as an address: it is a
// host-side shadow; the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) double g_noalloc_work[kScratchDoubles];

std::mutex g_mu;
double *g_work_ptr[kMaxDevices];       // device address of g_noalloc_work, per device
// host staging for the per-line tables (serialised by g_mu)
double g_hx[ns::kCoefStride * NS_NOALLOC_MAX_LINE];
double g_hy[ns::kCoefStride * NS_NOALLOC_MAX_LINE];
double g_warm_e[4096 + 6];

// Same tables as the context path (ns_api.cu): DRP coefficients
// init.f90:288-338, filters filtering.f90:25-31, :54-66, :114-120,
// LDDRK rk.f90:27-46, constants global.f90:38-39.
const double kA[3] = {0.770882380518, -0.166705904415, 0.0208431427703};
const double kA4[7] = {0.049041958000, -0.46884035700, -0.47476091400, 1.27327473700,
                       -0.51848452600, 0.16613853300,  -0.026369431000};
const double kA4b[7] = {0.026369431000, -0.16613853300, 0.51848452600, -1.27327473700,
                        0.47476091400,  0.46884035700,  -0.049041958000};
const double kA5[7] = {-0.20933762200, -1.08487567600, 2.14777605000, -1.38892832200,
                       0.76894976600,  -0.28181465000, 0.048230454000};
const double kA5b[7] = {-0.048230454000, 0.28181465000,  -0.76894976600, 1.38892832200,
                        -2.14777605000,  1.08487567600, 0.20933762200};
const double kA6[7] = {-2.19228033900, 4.74861140100, -5.10885191500, 4.46156710400,
                       -2.83349874100, 1.12832886100, -0.20387637100};
const double kA6b[7] = {0.20387637100, -1.12832886100, 2.83349874100, -4.46156710400,
                        5.10885191500, -4.74861140100, 2.19228033900};
const double kDf[7] = {0.190899511506,  -0.171503832236, 0.123632891797, -0.069975429105,
                       0.029662754736, -0.008520738659, 0.001254597714};
const double kDfbX[7] = {-0.057717512738, 0.199278374994,  -0.292668277650, 0.244537361546,
                         -0.134605018019, 0.056184263460, -0.015009191593};
const double kDfbY[7] = {(double)-0.057717512738f, (double)0.199278374994f,
                         (double)-0.292668277650f, (double)0.244537361546f,
                         (double)-0.134605018019f, (double)0.056184263460f,
                         (double)-0.015009191593f};
const double kAlpha[6] = {0.0, -0.737101392796, -1.634740794341,
                          -0.744739003780, -1.469897351522, -2.813971388035};
const double kBeta[6] = {0.032918605146, 0.823256998200, 0.381530948900,
                         0.200092213184, 1.718581042715, 0.27};
const double kCt[6] = {0.0, 0.032918605146, 0.249351723343,
                       0.466911705055, 0.582030414044, 0.847252983783};
const double kPe = 1000.0, kAlphaCond = 0.5;

int fail(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char *fmt, ...)
{
    char buf[384];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ns::record_error(buf);
    return code;
}

void fill_coef(double *tab, int n, double h, const double *mesh, int D, int metric_mode)
{
    std::memset(tab, 0, sizeof(double) * ns::kCoefStride * (size_t)n);
    for (int q = 0; q < n; q++) {
        double mt = 1.0;
        if (metric_mode == NS_METRIC_EVERYWHERE || q < D || q >= n - D) mt = mesh[q];
        double *c = tab + (size_t)q * ns::kCoefStride;
        const double *src = nullptr;
        if (q == 0) src = kA6;
        else if (q == 1) src = kA5;
        else if (q == 2) src = kA4;
        else if (q == n - 3) src = kA4b;
        else if (q == n - 2) src = kA5b;
        else if (q == n - 1) src = kA6b;
        if (src)
            for (int z = 0; z < 7; z++) c[z] = src[z] * mt / h;
        else
            for (int s = 0; s < 3; s++) c[4 + s] = kA[s] * mt / h;
    }
}

ns::FilterCoef filter_coef(double sigmaf, const double *dfb)
{
    ns::FilterCoef f;
    std::memset(&f, 0, sizeof f);
    f.c0 = 1.0 - sigmaf * kDf[0];
    for (int s = 1; s <= 6; s++) f.m[s] = -sigmaf * kDf[s];
    f.bm1 = -sigmaf * dfb[0];
    f.b0 = 1.0 - sigmaf * dfb[1];
    for (int s = 1; s <= 5; s++) f.b[s] = -sigmaf * dfb[s + 1];
    return f;
}

// Warm-up of the chunked filter recurrence (same rule as the context path).
int warmup(double sigmaf)
{
    const int kMax = 4096;
    const double thresh = std::ldexp(1.0, -60);
    int worst = 0;
    for (int u = 0; u < 6; u++) {
        std::memset(g_warm_e, 0, sizeof g_warm_e);
        g_warm_e[u] = 1.0;
        int last_big = 0;
        for (int q = 6; q < kMax + 6; q++) {
            double v = 0.0;
            for (int s = 1; s <= 6; s++) v += -sigmaf * kDf[s] * g_warm_e[q - s];
            g_warm_e[q] = v;
            if (std::fabs(v) >= thresh) last_big = q - 5;
        }
        if (last_big >= kMax - 64) return -1;
        if (last_big > worst) worst = last_big;
    }
    const int w = worst + 8;
    return w < 36 ? 36 : w;
}

__global__ void k_gauss_field(double *__restrict__ src, const double *__restrict__ m,
                              const double *__restrict__ n, ns::Dims d, double amplitude,
                              double m_pt, double n_pt, double r0, double ln2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= d.imax || j >= d.jmax) return;
    const double dx = m[i] - m_pt, dy = n[j] - n_pt;
    src[(long long)j * d.pitch + i] = amplitude * exp(-(ln2 * (dx * dx + dy * dy) / (r0 * r0)));
}

inline size_t round32(size_t n) { return (n + 31) / 32 * 32; }

}  // namespace

extern "C" int ns_step_noalloc(const ns_params *p, double *U, int64_t pitch, int iter0,
                               int nsteps, void *stream)
{
    if (!p || !U) return fail(NS_ERR_PARAM, "ns_step_noalloc: NULL argument");
    if (p->abi_version != NS_ABI_VERSION)
        return fail(NS_ERR_PARAM, "ns_step_noalloc: abi_version %d, library is %d",
                    p->abi_version, NS_ABI_VERSION);
    if (p->precision != NS_PREC_FP64)
        return fail(NS_ERR_UNSUPPORTED, "ns_step_noalloc: precision=%d is not available",
                    p->precision);
    if (p->imax < 13 || p->jmax < 13 || (p->nk != 4 && p->nk != 5) || p->D < 0 ||
        2 * p->D > p->imax || 2 * p->D > p->jmax || nsteps < 0 ||
        !(p->dt > 0) || !(p->dm > 0) || !(p->dn > 0) || !(p->gamma > 1.0) ||
        (!p->inviscid && (!(p->Re > 0) || !(p->Pr > 0) || !(p->Tref > 0))) ||
        p->source_mode < NS_SRC_NONE || p->source_mode > NS_SRC_FIELD ||
        (p->metric_mode != NS_METRIC_BANDS && p->metric_mode != NS_METRIC_EVERYWHERE) ||
        (p->ub_layout != NS_LAYOUT_FORTRAN && p->ub_layout != NS_LAYOUT_SOA))
        return fail(NS_ERR_PARAM, "ns_step_noalloc: invalid parameters (imax=%d jmax=%d nk=%d D=%d "
                    "nsteps=%d)", p->imax, p->jmax, p->nk, p->D, nsteps);
    if (!p->meshx || !p->meshy || !p->sigmax || !p->sigmay || !p->rhob || !p->Ub ||
        (p->nk == 5 && !p->psib) ||
        (p->source_mode == NS_SRC_GAUSSIAN && (!p->m || !p->n || !(p->r0 != 0.0))) ||
        (p->source_mode == NS_SRC_FIELD && !p->src_field))
        return fail(NS_ERR_PARAM, "ns_step_noalloc: a required setup array is NULL");
    if (pitch < p->imax || pitch % 32 != 0)
        return fail(NS_ERR_PARAM, "ns_step_noalloc: pitch=%lld must be >= imax and a multiple of 32",
                    (long long)pitch);
    if (p->imax > NS_NOALLOC_MAX_LINE || p->jmax > NS_NOALLOC_MAX_LINE)
        return fail(NS_ERR_PARAM, "ns_step_noalloc: imax=%d jmax=%d exceed NS_NOALLOC_MAX_LINE=%d",
                    p->imax, p->jmax, NS_NOALLOC_MAX_LINE);
    const int nk = p->nk;
    const size_t P = (size_t)pitch * p->jmax;
    const size_t need = 5 * nk * P + ns::AUX_COUNT * P + (p->source_mode ? P : 0) +
                        round32(ns::kCoefStride * (size_t)p->imax) +
                        round32(ns::kCoefStride * (size_t)p->jmax) + 3 * round32(p->imax) +
                        5 * round32(p->jmax) + 64;
    if (need > kScratchDoubles)
        return fail(NS_ERR_PARAM,
                    "ns_step_noalloc: this %dx%d nk=%d case needs %zu bytes of work area; the "
                    "static work area holds %zu (NS_NOALLOC_MAX_BYTES)",
                    p->imax, p->jmax, nk, need * sizeof(double), kScratchDoubles * sizeof(double));
    if (nsteps == 0) return NS_OK;

    std::lock_guard<std::mutex> lock(g_mu);
    const int dev = p->device;
    if (dev < 0 || dev >= kMaxDevices) return fail(NS_ERR_PARAM, "ns_step_noalloc: device=%d", dev);
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return fail(NS_ERR_CUDA, "ns_step_noalloc: cudaSetDevice: %s", cudaGetErrorString(e));
    if (!g_work_ptr[dev]) {
        // once per device, with that device current
        double *ptr = nullptr;
        e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_work);
        if (e != cudaSuccess || !ptr)
            return fail(NS_ERR_CUDA, "ns_step_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        e = ns::ensure_math_tables(dev);
        if (e != cudaSuccess)
            return fail(NS_ERR_CUDA, "ns_step_noalloc: transport-law tables: %s", cudaGetErrorString(e));
        g_work_ptr[dev] = ptr;
    }
    cudaStream_t s = (cudaStream_t)stream;

    // Carve the work area; the context struct only carries pointers here.
    ns_ctx c;
    c.p = *p;
    c.dev = dev;
    c.stream = s;
    ns::Dims &d = c.d;
    d.imax = p->imax;
    d.jmax = p->jmax;
    d.nk = nk;
    d.D = p->D;
    d.pitch = (int)pitch;
    d.plane = (long long)P;
    double *w = g_work_ptr[dev];
    auto take = [&](size_t n) { double *r = w; w += round32(n); return r; };
    c.U = U;
    c.U2 = take(nk * P);
    c.W = take(nk * P);
    c.dudm = take(nk * P);
    c.dudn = take(nk * P);
    c.aux = take(ns::AUX_COUNT * P);
    c.Ubase = take(nk * P);
    c.src = p->source_mode ? take(P) : nullptr;
    c.xcoef = take(ns::kCoefStride * (size_t)p->imax);
    c.ycoef = take(ns::kCoefStride * (size_t)p->jmax);
    c.sigx = take(p->imax);
    c.sigy = take(p->jmax);
    c.rhob = take(p->jmax);
    c.psib = take(p->jmax);
    c.stage_sin = take(8);
    c.d_iter = reinterpret_cast<int *>(take(8));
    double *mx = take(p->imax), *ny = take(p->jmax);
    c.visc = !p->inviscid;

#define NA_CUDA(call)                                                                       \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(NS_ERR_CUDA, "ns_step_noalloc: %s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

    // setup arrays (host -> work area)
    fill_coef(g_hx, p->imax, p->dm, p->meshx, p->D, p->metric_mode);
    fill_coef(g_hy, p->jmax, p->dn, p->meshy, p->D, p->metric_mode);
    NA_CUDA(cudaMemcpyAsync(c.xcoef, g_hx, sizeof(double) * ns::kCoefStride * p->imax,
                            cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(c.ycoef, g_hy, sizeof(double) * ns::kCoefStride * p->jmax,
                            cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(c.sigx, p->sigmax, sizeof(double) * p->imax, cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(c.sigy, p->sigmay, sizeof(double) * p->jmax, cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(c.rhob, p->rhob, sizeof(double) * p->jmax, cudaMemcpyHostToDevice, s));
    if (p->psib)
        NA_CUDA(cudaMemcpyAsync(c.psib, p->psib, sizeof(double) * p->jmax, cudaMemcpyHostToDevice, s));
    else
        NA_CUDA(cudaMemsetAsync(c.psib, 0, sizeof(double) * p->jmax, s));
    const size_t row = sizeof(double) * p->imax;
    if (p->ub_layout == NS_LAYOUT_SOA) {
        NA_CUDA(cudaMemcpy2DAsync(c.Ubase, sizeof(double) * pitch, p->Ub, row, row,
                                  (size_t)p->jmax * nk, cudaMemcpyHostToDevice, s));
    } else {
        NA_CUDA(cudaMemcpyAsync(c.U2, p->Ub, sizeof(double) * nk * p->imax * p->jmax,
                                cudaMemcpyHostToDevice, s));
        NA_CUDA(ns::launch_aos_to_soa(c.U2, c.Ubase, d, s));
    }
    if (p->source_mode == NS_SRC_FIELD) {
        NA_CUDA(cudaMemcpy2DAsync(c.src, sizeof(double) * pitch, p->src_field, row, row,
                                  (size_t)p->jmax, cudaMemcpyHostToDevice, s));
    } else if (p->source_mode == NS_SRC_GAUSSIAN) {
        NA_CUDA(cudaMemcpyAsync(mx, p->m, row, cudaMemcpyHostToDevice, s));
        NA_CUDA(cudaMemcpyAsync(ny, p->n, sizeof(double) * p->jmax, cudaMemcpyHostToDevice, s));
        const dim3 blk(32, 8), grd((p->imax + 31) / 32, (p->jmax + 7) / 8);
        k_gauss_field<<<grd, blk, 0, s>>>(c.src, mx, ny, d, p->amplitude, p->m_pt, p->n_pt, p->r0,
                                          std::log(2.0));
        NA_CUDA(cudaGetLastError());
    }

    // constants (as ns_create)
    ns::Physics &ph = c.phys;
    std::memset(&ph, 0, sizeof ph);
    ph.gamma = p->gamma;
    ph.dt = p->dt;
    ph.inv_pe = 1.0 / kPe;
    ph.alpha_cond = kAlphaCond;
    ph.Tref = p->Tref;
    ph.A_mi = p->A_mi; ph.B_mi = p->B_mi; ph.C_mi = p->C_mi; ph.D_mi = p->D_mi;
    ph.A_k = p->A_k; ph.B_k = p->B_k; ph.C_k = p->C_k; ph.D_k = p->D_k;
    if (c.visc) {
        ph.inv_re = 1.0 / p->Re;
        ph.inv_re_pr = 1.0 / p->Re / p->Pr;
        ph.gm1_re = (p->gamma - 1.0) / p->Re;
        const double Tr = p->Tref;
        const double ak0 = p->A_k * std::log(1.0 * Tr) + p->B_k / Tr + p->C_k / Tr / Tr + p->D_k;
        const double ami0 = p->A_mi * std::log(1.0 * Tr) + p->B_mi / Tr + p->C_mi / Tr / Tr + p->D_mi;
        ph.k0inv = 1.0 / std::exp(ak0);
        ph.mu0inv = 1.0 / std::exp(ami0);
        ph.D_mi_s = p->D_mi - ami0;
        ph.D_k_s = p->D_k - ak0;
    }
    c.fx = filter_coef(p->sigmaf, kDfbX);
    c.fy = filter_coef(p->sigmaf, kDfbY);
    for (int k = 0; k < 6; k++) {
        c.ct[k] = kCt[k];
        c.alpha[k] = kAlpha[k];
        c.beta[k] = kBeta[k];
    }
    c.warm = warmup(p->sigmaf);
    int nsm = 152;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    c.nsm = nsm;

    // the step, kernel by kernel (no graph: instantiating one allocates)
    int cls[ns::kMaxStepLaunches], stage[ns::kMaxStepLaunches];
    const int n = ns::step_sequence(&c, cls, stage);
    if (c.src) NA_CUDA(ns::launch_set_iter(c.d_iter, iter0, s));
    for (int st = 0; st < nsteps; st++)
        for (int q = 0; q < n; q++) NA_CUDA(ns::launch_kernel(&c, cls[q], stage[q], s));
#undef NA_CUDA
    return NS_OK;
}
