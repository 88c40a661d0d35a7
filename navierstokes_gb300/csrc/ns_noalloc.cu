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
#include <vector>

#include "ns_coef.h"
#include "ns_internal.cuh"

namespace {

using namespace ns::coef;

constexpr size_t kScratchDoubles = NS_NOALLOC_MAX_BYTES / sizeof(double);
constexpr int kMaxDevices = 64;

// The work area.  Host code must not use this name as an address: it is a
// host-side shadow; the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) double g_noalloc_work[kScratchDoubles];

std::mutex g_mu;
double *g_work_ptr[kMaxDevices];       // device address of g_noalloc_work, per device
// host staging for the per-line tables and the transport-law table
// (serialised by g_mu)
double g_hx[ns::kCoefStride * NS_NOALLOC_MAX_LINE];
double g_hy[ns::kCoefStride * NS_NOALLOC_MAX_LINE];
double g_tr[ns::kTrPieces * ns::kTrStride];
double g_tr_key[9];                    // Tref and the two fits g_tr was built for
bool g_tr_valid = false;

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

// Puts the calling thread's current device back on every return path.
struct DeviceGuard {
    int prev = -1;
    DeviceGuard() { if (cudaGetDevice(&prev) != cudaSuccess) prev = -1; }
    ~DeviceGuard() { if (prev >= 0) cudaSetDevice(prev); }
};

// The transport-law table of ns_create for these constants, rebuilt only
// when they change (building it takes a few milliseconds).
void transport_table(const ns_params *p)
{
    const double key[9] = {p->Tref, p->A_mi, p->B_mi, p->C_mi, p->D_mi,
                           p->A_k,  p->B_k,  p->C_k,  p->D_k};
    if (g_tr_valid && std::memcmp(key, g_tr_key, sizeof key) == 0) return;
    std::vector<double> tab;
    ns::build_transport_table(tab, p->Tref, key + 1, key + 5);
    std::memcpy(g_tr, tab.data(), sizeof g_tr);
    std::memcpy(g_tr_key, key, sizeof key);
    g_tr_valid = true;
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
    if (pitch < p->imax || pitch % 32 != 0 ||
        pitch > (int64_t)(NS_NOALLOC_MAX_BYTES / sizeof(double)))
        return fail(NS_ERR_PARAM,
                    "ns_step_noalloc: pitch=%lld must be >= imax, a multiple of 32 and at most "
                    "NS_NOALLOC_MAX_BYTES/8", (long long)pitch);
    if (p->imax > NS_NOALLOC_MAX_LINE || p->jmax > NS_NOALLOC_MAX_LINE)
        return fail(NS_ERR_PARAM, "ns_step_noalloc: imax=%d jmax=%d exceed NS_NOALLOC_MAX_LINE=%d",
                    p->imax, p->jmax, NS_NOALLOC_MAX_LINE);
    const int nk = p->nk;
    const size_t P = (size_t)pitch * p->jmax;
    const size_t trn = p->inviscid ? 0 : (size_t)ns::kTrPieces * ns::kTrStride;
    const size_t need = 5 * nk * P + ns::AUX_COUNT * P + (p->source_mode ? P : 0) + trn +
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
    DeviceGuard keep_device;
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
    // Every call copies its setup arrays from host memory the library reuses
    // on the next call, so a captured call would replay stale tables.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(s, &cap);
    if (e != cudaSuccess || cap != cudaStreamCaptureStatusNone)
        return fail(NS_ERR_UNSUPPORTED,
                    "ns_step_noalloc: the stream is capturing (or its capture status is not "
                    "available); the call copies host tables that the next call reuses");

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
    c.trtab = trn ? take(trn) : nullptr;
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
    line_table(g_hx, p->imax, p->dm, p->meshx, p->D, p->metric_mode);
    line_table(g_hy, p->jmax, p->dn, p->meshy, p->D, p->metric_mode);
    if (c.trtab) {
        transport_table(p);
        NA_CUDA(cudaMemcpyAsync(c.trtab, g_tr, sizeof g_tr, cudaMemcpyHostToDevice, s));
    }
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
    c.fx = filter(p->sigmaf, kDfbX);
    c.fy = filter(p->sigmaf, kDfbY);
    for (int k = 0; k < 6; k++) {
        c.ct[k] = kCt[k];
        c.alpha[k] = kAlpha[k];
        c.beta[k] = kBeta[k];
    }
    fp64_warmups(p->sigmaf, c.warm, c.warm32);
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
