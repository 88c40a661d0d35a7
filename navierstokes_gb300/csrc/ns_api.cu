// ns_api.cu -- host side of the C ABI declared in include/ns_gb300.h.
//
// Builds, once per context, everything rk_euler (rk.f90:12-75) reads from
// module `global`: the per-line DRP coefficient tables with 1/dm, 1/dn and
// the metric folded in (diff.f90:40-350, coefficients init.f90:286-338), the
// filter coefficient sets (filtering.f90:25-31, :54-66, :114-120), the
// LDDRK tables (rk.f90:27-46), the transport reference values
// (coefficients.f90:71-80), the buffer arrays and the base flow.  One step
// is captured once as a CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cudaTypedefs.h>
#include <mutex>

#include "ns_check.cuh"
#include "ns_coef.h"
#include "ns_internal.cuh"

#define NS_STR2(x) #x
#define NS_STR1(x) NS_STR2(x)
#define NS_STR_CUDA_VERSION NS_STR1(CUDART_VERSION)

namespace {

using namespace ns::coef;

thread_local std::string g_last_error;

// Per-line derivative table as a vector (ns::coef::line_table).
void build_coef(std::vector<double> &tab, int n, double h, const double *mesh, int D,
                int metric_mode)
{
    tab.resize((size_t)n * ns::kCoefStride);
    line_table(tab.data(), n, h, mesh, D, metric_mode);
}

int set_err(ns_ctx *c, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    g_last_error = buf;
    return code;
}

int cuda_err(ns_ctx *c, cudaError_t e, const char *what)
{
    return set_err(c, NS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define NS_CUDA(c, call)                                          \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return cuda_err((c), e_, #call);   \
    } while (0)


// DRP first derivative of a line with the per-position table (FP64).
double line_derivative(const double *f, int q, int n, const double *c)
{
    if (q >= 3 && q < n - 3)
        return c[4] * (f[q + 1] - f[q - 1]) + c[5] * (f[q + 2] - f[q - 2]) +
               c[6] * (f[q + 3] - f[q - 3]);
    const int o0 = (q < 3) ? -q : (n - 7 - q);
    double r = 0.0;
    for (int z = 0; z < 7; z++) r += c[z] * f[q + o0 + z];
    return r;
}

int choose_chunks(int nlines_total, int n, int warm, int target_threads)
{
    if (warm < 0) return 1;
    const int len2 = n - 12;
    int c = (target_threads + nlines_total - 1) / nlines_total;
    // chunks at least 4x the warm-up long (<= 25% extra work) while that
    // still fills the GPU; when it does not (few, short lines: the filters are
    // then latency-bound), chunks down to the warm-up length
    int maxc = len2 / (4 * (warm + 6));
    if ((long long)maxc * nlines_total < target_threads) maxc = len2 / (warm + 6);
    if (c > maxc) c = maxc;
    if (c < 1) c = 1;
    return c;
}

template <class T>
int dalloc(ns_ctx *c, T **p, size_t count);

template <class T>
int upload_vec(ns_ctx *c, T *dst, const std::vector<T> &v)
{
    cudaError_t e = cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice,
                                    c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "upload");
    return NS_OK;
}

template <class T>
int dalloc(ns_ctx *c, T **p, size_t count)
{
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return set_err(c, NS_ERR_OOM, "cudaMalloc(%zu bytes): %s", count * sizeof(T),
                       cudaGetErrorString(e));
    }
    return NS_OK;
}

void free_all(ns_ctx *c)
{
    {
        ns::SplitState &sp = c->sp;
        float *fb[] = {sp.q[0], sp.q[1], sp.xc, sp.yc, sp.xcl, sp.ycl, sp.sigx, sp.sigy, sp.src,
                       sp.rho_bc, sp.ycorr, sp.mean_buf, sp.tau, sp.trf};
        for (float *b : fb)
            if (b) cudaFree(b);
    }
    if (c->step_exec) cudaGraphExecDestroy(c->step_exec);
    if (c->tail_exec) cudaGraphExecDestroy(c->tail_exec);
    for (cudaEvent_t ev : c->band_ev)
        if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : c->wb_ev)
        if (ev) cudaEventDestroy(ev);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    double *bufs[] = {c->U,    c->U2,   c->W,     c->dudm, c->dudn, c->aux,
                      c->Ubase, c->src, c->xcoef, c->ycoef, c->sigx, c->sigy,
                      c->rhob, c->psib, c->stage_sin, c->trtab, c->probe_buf, c->rec_buf,
                      c->vx, c->vy, c->omega};
    for (double *b : bufs)
        if (b) cudaFree(b);
    if (c->d_iter) cudaFree(c->d_iter);
    if (c->d_count) cudaFree(c->d_count);
    if (c->d_err) cudaFree(c->d_err);
    if (c->probe_idx) cudaFree(c->probe_idx);
    if (c->rec_idx) cudaFree(c->rec_idx);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
}

int validate(const ns_params *p)
{
    if (!p) return set_err(nullptr, NS_ERR_PARAM, "params is NULL");
    if (p->abi_version != NS_ABI_VERSION)
        return set_err(nullptr, NS_ERR_PARAM, "abi_version %d, library is %d", p->abi_version,
                       NS_ABI_VERSION);
    if (p->imax < 13 || p->jmax < 13)
        return set_err(nullptr, NS_ERR_PARAM, "imax=%d jmax=%d: both must be >= 13", p->imax,
                       p->jmax);
    if ((long long)p->imax * p->jmax > (1LL << 31))
        return set_err(nullptr, NS_ERR_PARAM, "grid of %lld points is too large",
                       (long long)p->imax * p->jmax);
    if (p->nk != 4 && p->nk != 5) return set_err(nullptr, NS_ERR_PARAM, "nk=%d: must be 4 or 5", p->nk);
    if (p->D < 0 || 2 * p->D > p->imax || 2 * p->D > p->jmax)
        return set_err(nullptr, NS_ERR_PARAM, "D=%d: need 0 <= 2*D <= min(imax,jmax)", p->D);
    if (p->metric_mode != NS_METRIC_BANDS && p->metric_mode != NS_METRIC_EVERYWHERE)
        return set_err(nullptr, NS_ERR_PARAM, "metric_mode=%d", p->metric_mode);
    if (p->precision != NS_PREC_FP64 && p->precision != NS_PREC_SPLIT &&
        p->precision != NS_PREC_SPLIT32)
        return set_err(nullptr, NS_ERR_UNSUPPORTED, "precision=%d is not available", p->precision);
    if (p->precision != NS_PREC_FP64 && p->nk != 4)
        return set_err(nullptr, NS_ERR_UNSUPPORTED,
                       "split precision carries rho, u, v, p (nk=4); got nk=%d", p->nk);
    if (p->source_mode < NS_SRC_NONE || p->source_mode > NS_SRC_FIELD)
        return set_err(nullptr, NS_ERR_PARAM, "source_mode=%d", p->source_mode);
    if (!(p->dt > 0) || !(p->dm > 0) || !(p->dn > 0) || !(p->gamma > 1.0))
        return set_err(nullptr, NS_ERR_PARAM, "dt, dm, dn must be > 0 and gamma > 1");
    if (!p->inviscid && (!(p->Re > 0) || !(p->Pr > 0) || !(p->Tref > 0)))
        return set_err(nullptr, NS_ERR_PARAM, "viscous case needs Re, Pr, Tref > 0");
    if (!p->meshx || !p->meshy || !p->sigmax || !p->sigmay || !p->rhob || !p->Ub)
        return set_err(nullptr, NS_ERR_PARAM, "meshx, meshy, sigmax, sigmay, rhob, Ub are required");
    if (p->nk == 5 && !p->psib) return set_err(nullptr, NS_ERR_PARAM, "psib is required for nk=5");
    if (p->source_mode == NS_SRC_GAUSSIAN && (!p->m || !p->n || !(p->r0 != 0.0)))
        return set_err(nullptr, NS_ERR_PARAM, "gaussian source needs m, n and r0 != 0");
    if (p->source_mode == NS_SRC_FIELD && !p->src_field)
        return set_err(nullptr, NS_ERR_PARAM, "field source needs src_field");
    if (p->ub_layout != NS_LAYOUT_FORTRAN && p->ub_layout != NS_LAYOUT_SOA &&
        p->ub_layout != NS_LAYOUT_ROWS)
        return set_err(nullptr, NS_ERR_PARAM, "ub_layout=%d", p->ub_layout);
    return NS_OK;
}

// Copies an nk-variable host field in `layout` into device planes.
int upload_field(ns_ctx *c, const double *h, int layout, double *dplanes)
{
    const ns::Dims &d = c->d;
    const size_t row = (size_t)d.imax * sizeof(double);
    if (layout == NS_LAYOUT_SOA) {
        NS_CUDA(c, cudaMemcpy2DAsync(dplanes, d.pitch * sizeof(double), h, row, row,
                                     (size_t)d.jmax * d.nk, cudaMemcpyHostToDevice, c->stream));
    } else if (layout == NS_LAYOUT_ROWS) {
        // rows of a field constant along i, expanded on the device
        double *stage = (dplanes == c->U2) ? c->dudm : c->U2;
        NS_CUDA(c, cudaMemcpyAsync(stage, h, (size_t)d.nk * d.jmax * sizeof(double),
                                   cudaMemcpyHostToDevice, c->stream));
        NS_CUDA(c, ns::launch_rows_to_planes(stage, dplanes, d, c->stream));
    } else if (layout == NS_LAYOUT_FORTRAN) {
        // stage the raw array in the scratch state buffer, then scatter
        double *stage = (dplanes == c->U2) ? c->dudm : c->U2;
        NS_CUDA(c, cudaMemcpyAsync(stage, h, (size_t)d.nk * d.imax * d.jmax * sizeof(double),
                                   cudaMemcpyHostToDevice, c->stream));
        NS_CUDA(c, ns::launch_aos_to_soa(stage, dplanes, d, c->stream));
    } else {
        return set_err(c, NS_ERR_PARAM, "layout=%d", layout);
    }
    return NS_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// TMA map of one perturbation buffer: planes of jmax rows of fpitch floats;
// box 40 x (kSplitTY + 6) x planes (the stage kernel's halo tile)
int make_split_map(ns_ctx *c, CUtensorMap *map, float *base, int planes)
{
    const auto encode = tensor_map_encoder();
    if (!encode) return set_err(c, NS_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is unavailable");
    const ns::Dims &d = c->d;
    const cuuint64_t dims[3] = {(cuuint64_t)d.imax, (cuuint64_t)d.jmax, (cuuint64_t)planes};
    const cuuint64_t strides[2] = {(cuuint64_t)c->sp.fpitch * sizeof(float),
                                   (cuuint64_t)c->sp.fpitch * d.jmax * sizeof(float)};
    const cuuint32_t box[3] = {40u, (cuuint32_t)(ns::kSplitTY + 6), (cuuint32_t)planes};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_err(c, NS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return NS_OK;
}

// TMA map of `depth` planes of pitch x jmax doubles from `base`, box
// box_w x box_h x planes (by default 40 x 14, the halo tile of the FP64
// stage kernels); depth 0 means depth = planes.
static int make_fp64_map(ns_ctx *c, CUtensorMap *map, double *base, int planes,
                         int depth = 0, int box_w = ns::kFirstTileW,
                         int box_h = ns::kFirstTileH)
{
    if (depth == 0) depth = planes;
    const auto encode = tensor_map_encoder();
    if (!encode) return set_err(c, NS_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is unavailable");
    const ns::Dims &d = c->d;
    const cuuint64_t dims[3] = {(cuuint64_t)d.imax, (cuuint64_t)d.jmax, (cuuint64_t)depth};
    const cuuint64_t strides[2] = {(cuuint64_t)d.pitch * sizeof(double),
                                   (cuuint64_t)d.plane * sizeof(double)};
    const cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, (cuuint32_t)planes};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_err(c, NS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return NS_OK;
}

static int make_fp64_maps(ns_ctx *c)
{
    // k_update's box: tau1..k dT/dy (viscous) and psiDiff (nk = 5)
    const int nz = (c->visc ? 5 : 0) + (c->d.nk >= 5 ? 1 : 0);
    int rc = make_fp64_map(c, &c->umap, c->U, c->d.nk);
    if (rc == NS_OK) rc = make_fp64_map(c, &c->tmap, c->aux + (size_t)ns::AUX_T * c->d.plane, 1);
    if (rc == NS_OK && nz > 0) rc = make_fp64_map(c, &c->amap, c->aux, nz, ns::AUX_COUNT);
    c->fp64_maps = (rc == NS_OK);
    return rc;
}

// Split precision: FP64 base flow + FP32 perturbation (ns_split.cu).
int create_split(ns_ctx *c)
{
    const ns_params *p = &c->p;
    const ns::Dims &d = c->d;
    ns::SplitState &sp = c->sp;
    const int imax = d.imax, jmax = d.jmax, nk = d.nk;
    auto ub = [&](int k, int i, int j) -> double {
        if (p->ub_layout == NS_LAYOUT_ROWS) return p->Ub[k + (size_t)nk * j];
        return p->ub_layout == NS_LAYOUT_FORTRAN
                   ? p->Ub[k + (size_t)nk * (i + (size_t)imax * j)]
                   : p->Ub[((size_t)k * jmax + j) * imax + i];
    };
    std::vector<double> rho(jmax), uu(jmax);
    const double pb = ub(3, 0, 0);
    for (int j = 0; j < jmax; j++) {
        rho[j] = ub(0, 0, j);
        uu[j] = ub(1, 0, j);
        for (int i = 0; i < imax; i++) {
            if (ub(0, i, j) != rho[j] || ub(1, i, j) != uu[j] || ub(2, i, j) != 0.0 ||
                ub(3, i, j) != pb)
                return set_err(c, NS_ERR_UNSUPPORTED,
                               "split precision needs a base flow uniform in x with v = 0 and "
                               "uniform p (violated at i=%d j=%d)", i + 1, j + 1);
        }
        // viscous: the base flow must be uniform in y as well, so that its own
        // stresses and heat flux vanish and those of the flow are
        // perturbation-sized
        if (c->visc && (rho[j] != rho[0] || uu[j] != uu[0]))
            return set_err(c, NS_ERR_UNSUPPORTED,
                           "split precision for Navier-Stokes needs a uniform base flow "
                           "(rho and u vary in y at j=%d)", j + 1);
    }
    sp.fpitch = (imax + 31) / 32 * 32;
    const size_t P = (size_t)d.plane, FP = (size_t)sp.fpitch * jmax;
    int rc;
    if ((rc = dalloc(c, &c->U, nk * P)) || (rc = dalloc(c, &c->U2, nk * P)) ||
        (rc = dalloc(c, &c->W, nk * P)) || (rc = dalloc(c, &c->Ubase, nk * P)) ||
        (rc = dalloc(c, &sp.q[0], (size_t)(4 + sp.np) * FP)) ||
        (rc = dalloc(c, &sp.q[1], (size_t)(4 + sp.np) * FP)) ||
        (rc = dalloc(c, &sp.xc, (size_t)ns::kCoefStride * imax)) ||
        (rc = dalloc(c, &sp.yc, (size_t)ns::kCoefStride * jmax)) ||
        (rc = dalloc(c, &sp.xcl, (size_t)ns::kCoefStride * imax)) ||
        (rc = dalloc(c, &sp.ycl, (size_t)ns::kCoefStride * jmax)) ||
        (rc = dalloc(c, &sp.sigx, (size_t)imax)) || (rc = dalloc(c, &sp.sigy, (size_t)jmax)) ||
        (rc = dalloc(c, &sp.rho_bc, (size_t)jmax)) || (rc = dalloc(c, &sp.ycorr, 4 * (size_t)jmax)) ||
        (rc = dalloc(c, &sp.mean_buf, 5 * (size_t)jmax)) ||
        (rc = dalloc(c, &c->stage_sin, 8)) || (rc = dalloc(c, &c->d_iter, 1)) ||
        (rc = dalloc(c, &c->d_count, 1)) || (rc = dalloc(c, &c->d_err, 1)))
        return rc;
    if (p->source_mode != NS_SRC_NONE && (rc = dalloc(c, &sp.src, FP))) return rc;
    if ((rc = make_split_map(c, &sp.qmap[0], sp.q[0], 4 + sp.np)) ||
        (rc = make_split_map(c, &sp.qmap[1], sp.q[1], 4 + sp.np)))
        return rc;
    if (c->visc) {
        // tau', k grad T' planes and the FP32 transport table
        if ((rc = dalloc(c, &sp.tau, 5 * FP)) ||
            (rc = dalloc(c, &sp.trf, (size_t)ns::kTrPieces * ns::kTrStride)) ||
            (rc = make_split_map(c, &sp.vmap, sp.tau, 5)))
            return rc;
        std::vector<double> tab;
        const double ami[4] = {p->A_mi, p->B_mi, p->C_mi, p->D_mi};
        const double ak[4] = {p->A_k, p->B_k, p->C_k, p->D_k};
        ns::build_transport_table(tab, p->Tref, ami, ak);
        std::vector<float> tabf(tab.begin(), tab.end());
        if ((rc = upload_vec(c, sp.trf, tabf))) return rc;
        const cudaError_t me = cudaMemsetAsync(sp.tau, 0, 5 * FP * sizeof(float), c->stream);
        if (me != cudaSuccess) return cuda_err(c, me, "cudaMemset");
        // upload_vec's host vector must outlive the copy
        const cudaError_t se = cudaStreamSynchronize(c->stream);
        if (se != cudaSuccess) return cuda_err(c, se, "split setup");
    }
    cudaError_t e = cudaMemsetAsync(sp.q[0], 0, (4 + sp.np) * FP * sizeof(float), c->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(sp.q[1], 0, (4 + sp.np) * FP * sizeof(float), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->W, 0, nk * P * sizeof(double), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_iter, 0, sizeof(int), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->stage_sin, 0, 8 * sizeof(double), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaMemset");

    std::vector<double> tx, ty;
    build_coef(tx, imax, p->dm, p->meshx, d.D, p->metric_mode);
    build_coef(ty, jmax, p->dn, p->meshy, d.D, p->metric_mode);
    std::vector<float> txf(tx.begin(), tx.end()), tyf(ty.begin(), ty.end());
    std::vector<float> txl(tx.size()), tyl(ty.size());
    for (size_t q = 0; q < tx.size(); q++) txl[q] = (float)(tx[q] - (double)txf[q]);
    for (size_t q = 0; q < ty.size(); q++) tyl[q] = (float)(ty[q] - (double)tyf[q]);
    std::vector<float> sx(p->sigmax, p->sigmax + imax), sy(p->sigmay, p->sigmay + jmax);
    // base-flow quantities (FP64, rounded once)
    std::vector<float> mean(5 * (size_t)jmax), rbc(jmax), corr(4 * (size_t)jmax, 0.f);
    for (int j = 0; j < jmax; j++) {
        mean[j] = (float)rho[j];
        mean[jmax + j] = (float)uu[j];
        mean[2 * jmax + j] = (float)line_derivative(rho.data(), j, jmax, &ty[(size_t)j * ns::kCoefStride]);
        mean[3 * jmax + j] = (float)line_derivative(uu.data(), j, jmax, &ty[(size_t)j * ns::kCoefStride]);
        mean[4 * jmax + j] = (float)(uu[j] - (double)mean[jmax + j]);
        rbc[j] = (float)(p->rhob[j] - rho[j]);
    }
    {
        // action of the y filter (REAL(4) boundary coefficients) on Ub
        std::vector<double> col(jmax), f(jmax);
        for (int k = 0; k < 4; k++) {
            for (int j = 0; j < jmax; j++) col[j] = (k == 0) ? rho[j] : (k == 1) ? uu[j] : (k == 2) ? 0.0 : pb;
            f = col;
            serial_filter_line(f.data(), jmax, p->sigmaf, kDfbY);
            for (int j = 0; j < jmax; j++) corr[(size_t)k * jmax + j] = (float)(f[j] - col[j]);
        }
    }
    if ((rc = upload_vec(c, sp.xc, txf)) || (rc = upload_vec(c, sp.yc, tyf)) ||
        (rc = upload_vec(c, sp.xcl, txl)) || (rc = upload_vec(c, sp.ycl, tyl)) ||
        (rc = upload_vec(c, sp.sigx, sx)) || (rc = upload_vec(c, sp.sigy, sy)) ||
        (rc = upload_vec(c, sp.mean_buf, mean)) || (rc = upload_vec(c, sp.rho_bc, rbc)) ||
        (rc = upload_vec(c, sp.ycorr, corr)))
        return rc;
    std::vector<float> field;
    if (p->source_mode != NS_SRC_NONE) {
        field.assign(FP, 0.f);
        for (int j = 0; j < jmax; j++)
            for (int i = 0; i < imax; i++) {
                double v;
                if (p->source_mode == NS_SRC_GAUSSIAN) {
                    const double dx = p->m[i] - p->m_pt, dy = p->n[j] - p->n_pt;
                    v = p->amplitude * std::exp(-(std::log(2.0) * (dx * dx + dy * dy) / (p->r0 * p->r0)));
                } else {
                    v = p->src_field[(size_t)j * imax + i];
                }
                field[(size_t)j * sp.fpitch + i] = (float)v;
            }
        if ((rc = upload_vec(c, sp.src, field))) return rc;
    }
    if ((rc = upload_field(c, p->Ub, p->ub_layout, c->Ubase))) return rc;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "split setup");
    sp.mean.rho = sp.mean_buf;
    sp.mean.u = sp.mean_buf + jmax;
    sp.mean.drho = sp.mean_buf + 2 * jmax;
    sp.mean.du = sp.mean_buf + 3 * jmax;
    sp.mean.ulo = sp.mean_buf + 4 * jmax;
    sp.mean.p = (float)pb;
    sp.mean.gamma = (float)p->gamma;
    sp.p_bc = 1.0 / p->gamma - pb;
    if (c->visc) {
        // GET_COEFFICIENTS (coefficients.f90:78-79): 1/mu0 and 1/k0 folded into
        // the constant term of the exp/log form
        const double Tr = p->Tref;
        const double ami0 = p->A_mi * std::log(Tr) + p->B_mi / Tr + p->C_mi / Tr / Tr + p->D_mi;
        const double ak0 = p->A_k * std::log(Tr) + p->B_k / Tr + p->C_k / Tr / Tr + p->D_k;
        ns::SplitVisc &v = sp.vis;
        v.rho_b = (float)rho[0];
        v.p_b = (float)pb;
        v.gamma = (float)p->gamma;
        v.T_b = (float)(p->gamma * pb / rho[0]);
        v.inv_re = (float)(1.0 / p->Re);
        v.gm1_re = (float)((p->gamma - 1.0) / p->Re);
        v.inv_re_pr = (float)(1.0 / p->Re / p->Pr);
        v.Tref = (float)Tr;
        v.A_mi = (float)p->A_mi;
        v.B_mi = (float)p->B_mi;
        v.C_mi = (float)p->C_mi;
        v.D_mi_s = (float)(p->D_mi - ami0);
        v.A_k = (float)p->A_k;
        v.B_k = (float)p->B_k;
        v.C_k = (float)p->C_k;
        v.D_k_s = (float)(p->D_k - ak0);
    }
    return NS_OK;
}

}  // namespace

namespace ns {
PFN_cuTensorMapEncodeTiled_v12000 tensor_encoder() { return tensor_map_encoder(); }

int make_plane_map(ns_ctx *c, CUtensorMap *map, double *base, int planes, int box_w, int box_h)
{
    return make_fp64_map(c, map, base, planes, 0, box_w, box_h);
}

int check_error(int word)
{
    static const char *const files[] = {"?", "ns_kernels.cu", "ns_split.cu", "ns_batch.cu",
                                        "ns_adjoint.cu"};
    const int f = (word >> 16) & 0xff, line = word & 0xffff;
    char buf[160];
    snprintf(buf, sizeof buf, "checked build: an index check failed in %s line %d",
             f < 5 ? files[f] : "?", line);
    record_error(buf);
    return NS_ERR_CHECK;
}

void build_line_coef(std::vector<double> &tab, int n, double h, const double *mesh, int D,
                     int metric_mode)
{
    build_coef(tab, n, h, mesh, D, metric_mode);
}

// mu(T) = exp(g_mi(Tref T) - g_mi(Tref)) and k(T) likewise, with
// g(x) = A ln x + B/x + C/x^2 + D (coefficients.f90:27-59; the division by
// mu0 and k0 of coefficients.f90 is the subtraction of g(Tref)).  Each piece
// [t0, t0 + h) is interpolated at the kTrDeg+1 Chebyshev nodes in long
// double; its Chebyshev series is converted to powers of s = (T - t0)/h and
// then of u = T - t0 (h a power of two, so the scaling is exact).  With
// h = t0/256 the interpolation error is far below the rounding of the
// evaluation: for the N2 fit, mu and k evaluated in double are within
// 2.3e-16 relative of the exact law over T in [1/4, 8) (below 1/4 the fit's
// C/x^2 term makes k too steep for degree 5, so the table starts there).
void build_transport_table(std::vector<double> &tab, double Tref, const double *a_mi,
                           const double *a_k)
{
    constexpr int n = kTrDeg + 1;
    tab.assign((size_t)kTrPieces * kTrStride, 0.0);
    const long double pi = 3.141592653589793238462643383279502884L;
    auto g = [](const double *a, long double x) {
        return (long double)a[0] * std::log(x) + (long double)a[1] / x +
               (long double)a[2] / (x * x) + (long double)a[3];
    };
    const long double tr = Tref;
    const long double g0[2] = {g(a_mi, tr), g(a_k, tr)};
    const double *coef[2] = {a_mi, a_k};
    long double th[n], sn[n];
    for (int i = 0; i < n; i++) {
        th[i] = (2 * i + 1) * pi / (2 * n);
        sn[i] = (1.0L - std::cos(th[i])) / 2;  // node in [0, 1]
    }
    // powers of s in T_m(2s - 1): T_0 = 1, T_1 = 2s - 1, T_m+1 = 2(2s-1)T_m - T_m-1
    long double cm[n][n] = {};
    cm[0][0] = 1;
    cm[1][0] = -1;
    cm[1][1] = 2;
    for (int m = 1; m + 1 < n; m++)
        for (int k = 0; k < n; k++)
            cm[m + 1][k] = 2 * (2 * (k > 0 ? cm[m][k - 1] : 0.0L) - cm[m][k]) - cm[m - 1][k];
    for (int piece = 0; piece < kTrPieces; piece++) {
        const int e = kTrEmin + piece / 256, j = piece % 256;
        const long double t0 = std::ldexp(1.0L + j / 256.0L, e);
        const long double h = std::ldexp(1.0L, e - 8);
        for (int f = 0; f < 2; f++) {
            long double v[n], a[n] = {}, b[n] = {};
            for (int i = 0; i < n; i++) v[i] = std::exp(g(coef[f], tr * (t0 + sn[i] * h)) - g0[f]);
            // 2s - 1 = -cos(th_i), so T_m(2s_i - 1) = (-1)^m cos(m th_i)
            for (int m = 0; m < n; m++) {
                long double acc = 0;
                for (int i = 0; i < n; i++) acc += v[i] * std::cos(m * th[i]);
                a[m] = ((m & 1) ? -acc : acc) * (m == 0 ? 1.0L : 2.0L) / n;
            }
            for (int k = 0; k < n; k++)
                for (int m = 0; m < n; m++) b[k] += a[m] * cm[m][k];
            double *out = &tab[(size_t)piece * kTrStride + (size_t)f * n];
            for (int k = 0; k < n; k++) out[k] = (double)std::ldexp(b[k], -k * (e - 8));
        }
    }
}
}  // namespace ns

namespace ns {
void record_error(const char *msg) { g_last_error = msg; }
}  // namespace ns

int ns_pin_host(void *p, size_t bytes)
{
    if (!p || bytes == 0) return set_err(nullptr, NS_ERR_PARAM, "ns_pin_host: bad argument");
    const cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, NS_ERR_CUDA, "ns_pin_host: cudaHostRegister: %s",
                       cudaGetErrorString(e));
    }
    return NS_OK;
}

int ns_unpin_host(void *p)
{
    if (!p) return set_err(nullptr, NS_ERR_PARAM, "ns_unpin_host: NULL");
    const cudaError_t e = cudaHostUnregister(p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, NS_ERR_CUDA, "ns_unpin_host: cudaHostUnregister: %s",
                       cudaGetErrorString(e));
    }
    return NS_OK;
}

int ns_filter_plan(int nlines, int n, int nk, int warm, int nsm, int64_t *seg, int *blocks)
{
    if (nlines < 1 || n < 13 || nk < 1 || nsm < 1 || !seg || !blocks)
        return set_err(nullptr, NS_ERR_PARAM, "ns_filter_plan: bad argument");
    long long s = 0;
    unsigned b = 0;
    ns::filter_shape(nlines, n, nk, warm, nsm, ns::kFilterWarpsPerSmsp, s, b);
    *seg = s;
    *blocks = (int)b;
    return NS_OK;
}

int ns_transport_table(double Tref, const double *fit_mu, const double *fit_k, double *out)
{
    static_assert(NS_TRANSPORT_TABLE_DOUBLES == ns::kTrPieces * ns::kTrStride, "table size");
    if (!fit_mu || !fit_k || !out || !(Tref > 0.0))
        return set_err(nullptr, NS_ERR_PARAM, "ns_transport_table: bad argument");
    std::vector<double> tab;
    ns::build_transport_table(tab, Tref, fit_mu, fit_k);
    std::memcpy(out, tab.data(), tab.size() * sizeof(double));
    return NS_OK;
}

extern "C" {

int ns_abi_version(void) { return NS_ABI_VERSION; }

const char *ns_build_info(void)
{
    return "ns_gb300 FP64 stage kernels, sm_103a, CUDA " NS_STR_CUDA_VERSION;
}

int ns_params_init(ns_params *p)
{
    if (!p) return NS_ERR_PARAM;
    std::memset(p, 0, sizeof *p);
    p->abi_version = NS_ABI_VERSION;
    p->nk = 5;
    p->metric_mode = NS_METRIC_BANDS;
    p->precision = NS_PREC_FP64;
    p->source_mode = NS_SRC_NONE;
    p->ub_layout = NS_LAYOUT_FORTRAN;
    p->gamma = 1.4;           // init.f90:361
    p->Tref = 273.15;         // dados.in &flow Tref
    p->Pr = 0.71;             // dados.in &flow Pr
    p->Re = 10000.0;          // dados.in &flow Re
    p->sigmaf = 0.1;          // dados.in &grid sigmaf
    // SPECIE_N, coefficients.f90:113-123
    p->A_mi = 0.62526577;
    p->B_mi = -31.779652;
    p->C_mi = -1640.7913;
    p->D_mi = 1.7454992;
    p->A_k = 0.85372829;
    p->B_k = 105.18665;
    p->C_k = -12229.753;
    p->D_k = 0.48299104;
    return NS_OK;
}

const char *ns_last_error(const ns_ctx *ctx)
{
    if (ctx && !ctx->err.empty()) return ctx->err.c_str();
    return g_last_error.c_str();
}

int ns_create(const ns_params *p, ns_ctx **out)
{
    if (!out) return set_err(nullptr, NS_ERR_PARAM, "out is NULL");
    *out = nullptr;
    int rc = validate(p);
    if (rc != NS_OK) return rc;

    ns_ctx *c = new (std::nothrow) ns_ctx();
    if (!c) return set_err(nullptr, NS_ERR_OOM, "host allocation failed");
    c->p = *p;
    c->dev = p->device;
    cudaError_t e = cudaSetDevice(c->dev);
    if (e != cudaSuccess) {
        rc = cuda_err(c, e, "cudaSetDevice");
        delete c;
        return rc;
    }
    e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        rc = cuda_err(c, e, "cudaStreamCreate");
        delete c;
        return rc;
    }
    c->stream = c->own_stream;

    ns::Dims &d = c->d;
    d.imax = p->imax;
    d.jmax = p->jmax;
    d.nk = p->nk;
    d.D = p->D;
    d.pitch = (p->imax + 31) / 32 * 32;
    d.plane = (long long)d.pitch * d.jmax;
    c->visc = !p->inviscid;
    const size_t P = (size_t)d.plane, nk = (size_t)d.nk;
    c->split = (p->precision == NS_PREC_SPLIT || p->precision == NS_PREC_SPLIT32);
    c->sp.np = (p->precision == NS_PREC_SPLIT) ? 3 : 0;

#define NS_TRY(x)                     \
    do {                              \
        rc = (x);                     \
        if (rc != NS_OK) goto fail;   \
    } while (0)
    if (c->split) {
        NS_TRY(create_split(c));
        goto constants;
    }
    if (c->visc) {
        const cudaError_t me = ns::ensure_math_tables(c->dev);
        if (me != cudaSuccess) {
            rc = cuda_err(c, me, "transport-law tables");
            goto fail;
        }
    }
    NS_TRY(dalloc(c, &c->U, nk * P));
    NS_TRY(dalloc(c, &c->U2, nk * P));
    NS_TRY(dalloc(c, &c->W, nk * P));
    NS_TRY(dalloc(c, &c->dudm, nk * P));
    NS_TRY(dalloc(c, &c->dudn, nk * P));
    NS_TRY(dalloc(c, &c->aux, (size_t)ns::AUX_COUNT * P));
    NS_TRY(dalloc(c, &c->Ubase, nk * P));
    NS_TRY(dalloc(c, &c->xcoef, (size_t)d.imax * ns::kCoefStride));
    NS_TRY(dalloc(c, &c->ycoef, (size_t)d.jmax * ns::kCoefStride));
    NS_TRY(dalloc(c, &c->sigx, (size_t)d.imax));
    NS_TRY(dalloc(c, &c->sigy, (size_t)d.jmax));
    NS_TRY(dalloc(c, &c->rhob, (size_t)d.jmax));
    NS_TRY(dalloc(c, &c->psib, (size_t)d.jmax));
    NS_TRY(dalloc(c, &c->stage_sin, 8));
    NS_TRY(dalloc(c, &c->d_iter, 1));
    NS_TRY(dalloc(c, &c->d_count, 1));
    NS_TRY(dalloc(c, &c->d_err, 1));
    if (p->source_mode != NS_SRC_NONE) NS_TRY(dalloc(c, &c->src, P));
    if (c->visc) {
        NS_TRY(dalloc(c, &c->trtab, (size_t)ns::kTrPieces * ns::kTrStride));
        std::vector<double> tab;
        const double ami[4] = {p->A_mi, p->B_mi, p->C_mi, p->D_mi};
        const double ak[4] = {p->A_k, p->B_k, p->C_k, p->D_k};
        ns::build_transport_table(tab, p->Tref, ami, ak);
        e = cudaMemcpyAsync(c->trtab, tab.data(), tab.size() * sizeof(double),
                            cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
            rc = cuda_err(c, e, "transport-law table");
            goto fail;
        }
    }
    NS_TRY(make_fp64_maps(c));

    {
        // zero everything so padding and never-written planes are defined
        double *z[] = {c->U, c->U2, c->W, c->dudm, c->dudn, c->Ubase};
        for (double *b : z) {
            e = cudaMemsetAsync(b, 0, nk * P * sizeof(double), c->stream);
            if (e != cudaSuccess) { rc = cuda_err(c, e, "cudaMemset"); goto fail; }
        }
        e = cudaMemsetAsync(c->aux, 0, (size_t)ns::AUX_COUNT * P * sizeof(double), c->stream);
        if (e != cudaSuccess) { rc = cuda_err(c, e, "cudaMemset"); goto fail; }
        e = cudaMemsetAsync(c->stage_sin, 0, 8 * sizeof(double), c->stream);
        if (e != cudaSuccess) { rc = cuda_err(c, e, "cudaMemset"); goto fail; }
        e = cudaMemsetAsync(c->d_iter, 0, sizeof(int), c->stream);
        if (e != cudaSuccess) { rc = cuda_err(c, e, "cudaMemset"); goto fail; }
        e = cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
        if (e != cudaSuccess) { rc = cuda_err(c, e, "cudaMemset"); goto fail; }
    }

    {
        std::vector<double> tx, ty;
        build_coef(tx, d.imax, p->dm, p->meshx, d.D, p->metric_mode);
        build_coef(ty, d.jmax, p->dn, p->meshy, d.D, p->metric_mode);
        e = cudaMemcpyAsync(c->xcoef, tx.data(), tx.size() * 8, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->ycoef, ty.data(), ty.size() * 8, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->sigx, p->sigmax, (size_t)d.imax * 8, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->sigy, p->sigmay, (size_t)d.jmax * 8, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->rhob, p->rhob, (size_t)d.jmax * 8, cudaMemcpyHostToDevice, c->stream);
        std::vector<double> psib(d.jmax, 0.0);
        if (p->psib) std::memcpy(psib.data(), p->psib, (size_t)d.jmax * 8);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->psib, psib.data(), (size_t)d.jmax * 8, cudaMemcpyHostToDevice, c->stream);
        std::vector<double> field;
        if (e == cudaSuccess && p->source_mode != NS_SRC_NONE) {
            // spatial part of s_acou (rk.f90:188-189); the time factor is
            // applied per stage on the device
            field.assign((size_t)d.jmax * d.pitch, 0.0);
            for (int j = 0; j < d.jmax; j++)
                for (int i = 0; i < d.imax; i++) {
                    double v;
                    if (p->source_mode == NS_SRC_GAUSSIAN) {
                        const double dx = p->m[i] - p->m_pt, dy = p->n[j] - p->n_pt;
                        v = p->amplitude *
                            std::exp(-(std::log(2.0) * (dx * dx + dy * dy) / (p->r0 * p->r0)));
                    } else {
                        v = p->src_field[(size_t)j * d.imax + i];
                    }
                    field[(size_t)j * d.pitch + i] = v;
                }
            e = cudaMemcpyAsync(c->src, field.data(), field.size() * 8, cudaMemcpyHostToDevice,
                                c->stream);
        }
        if (e != cudaSuccess) { rc = cuda_err(c, e, "upload setup arrays"); goto fail; }
        rc = upload_field(c, p->Ub, p->ub_layout, c->Ubase);
        if (rc != NS_OK) goto fail;
        // the setup vectors above must stay alive until the copies finish
        e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) { rc = cuda_err(c, e, "setup"); goto fail; }
    }

    // constants
constants:
    {
        ns::Physics &ph = c->phys;
        ph.gamma = p->gamma;
        ph.dt = p->dt;
        ph.inv_pe = 1.0 / kPe;
        ph.alpha_cond = kAlphaCond;
        if (c->visc) {
            ph.inv_re = 1.0 / p->Re;
            ph.inv_re_pr = 1.0 / p->Re / p->Pr;
            ph.gm1_re = (p->gamma - 1.0) / p->Re;
        } else {
            ph.inv_re = ph.inv_re_pr = ph.gm1_re = 0.0;
        }
        ph.Tref = p->Tref;
        ph.A_mi = p->A_mi; ph.B_mi = p->B_mi; ph.C_mi = p->C_mi; ph.D_mi = p->D_mi;
        ph.A_k = p->A_k; ph.B_k = p->B_k; ph.C_k = p->C_k; ph.D_k = p->D_k;
        if (c->visc) {
            // GET_COEFFICIENTS, coefficients.f90:78-79
            const double Tr = p->Tref;
            const double ak0 = p->A_k * std::log(1.0 * Tr) + p->B_k / Tr + p->C_k / Tr / Tr + p->D_k;
            const double ami0 = p->A_mi * std::log(1.0 * Tr) + p->B_mi / Tr + p->C_mi / Tr / Tr + p->D_mi;
            ph.mu0inv = 1.0 / std::exp(ami0);
            ph.k0inv = 1.0 / std::exp(ak0);
            // mu/mu0 = exp(arg(T) - arg(Tref)): the constant term absorbs 1/mu0
            ph.D_mi_s = p->D_mi - ami0;
            ph.D_k_s = p->D_k - ak0;
        }
        c->fx = filter(p->sigmaf, kDfbX);
        c->fy = filter(p->sigmaf, kDfbY);
        for (int k = 0; k < 6; k++) {
            c->ct[k] = kCt[k];
            c->alpha[k] = kAlpha[k];
            c->beta[k] = kBeta[k];
        }
        fp64_warmups(p->sigmaf, c->warm, c->warm32);
        int nsm = 152;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->dev);
        c->nsm = nsm;
        if (c->split) {
            // FP32 filters are bound by memory: aim at 32 resident warps per SM
            ns::SplitState &sp = c->sp;
            // pairs carry ~48 bits: warm-up to 2^-50; single FP32 to 2^-32
            sp.warm = warmup(p->sigmaf, std::ldexp(1.0, sp.np ? -50 : -32), 16);
            const int twarps = nsm * 32;
            const int xgroups = 4 * ((d.jmax + 31) / 32);
            sp.fx_chunks = choose_chunks(xgroups, d.imax, sp.warm, twarps);
            sp.fy_chunks = choose_chunks(d.imax * 4, d.jmax, sp.warm, twarps * 32);
        }
        c->launches_per_step = ns::count_step_launches(c);
    }
#undef NS_TRY
    *out = c;
    return NS_OK;
fail:
    free_all(c);
    {
        std::string msg = c->err;
        delete c;
        g_last_error = msg;
    }
    return rc;
}

void ns_destroy(ns_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->dev);
    cudaStreamSynchronize(ctx->stream);
    free_all(ctx);
    delete ctx;
}

int ns_set_state(ns_ctx *c, const double *U, int layout)
{
    if (!c || !U) return set_err(c, NS_ERR_PARAM, "ns_set_state: NULL argument");
    NS_CUDA(c, cudaSetDevice(c->dev));
    int rc = upload_field(c, U, layout, c->U);
    if (rc != NS_OK) return rc;
    if (c->split) NS_CUDA(c, ns::launch_split_from_full(c, c->U, c->stream));
    NS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->have_state = true;
    return NS_OK;
}

static int check_kernel_err(ns_ctx *c);

int ns_get_state(ns_ctx *c, double *U, int layout)
{
    if (!c || !U) return set_err(c, NS_ERR_PARAM, "ns_get_state: NULL argument");
    if (!c->have_state) return set_err(c, NS_ERR_STATE, "ns_get_state before ns_set_state");
    NS_CUDA(c, cudaSetDevice(c->dev));
    const ns::Dims &d = c->d;
    const size_t row = (size_t)d.imax * sizeof(double);
    if (c->split) NS_CUDA(c, ns::launch_split_to_full(c, c->U, c->stream));
    if (layout == NS_LAYOUT_SOA) {
        NS_CUDA(c, cudaMemcpy2DAsync(U, row, c->U, d.pitch * sizeof(double), row,
                                     (size_t)d.jmax * d.nk, cudaMemcpyDeviceToHost, c->stream));
    } else if (layout == NS_LAYOUT_FORTRAN) {
        NS_CUDA(c, ns::launch_soa_to_aos(c->U, c->U2, d, c->stream));
        NS_CUDA(c, cudaMemcpyAsync(U, c->U2, (size_t)d.nk * d.imax * d.jmax * sizeof(double),
                                   cudaMemcpyDeviceToHost, c->stream));
    } else {
        return set_err(c, NS_ERR_PARAM, "layout=%d", layout);
    }
    NS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_kernel_err(c);
}

// Captures the launches `fn` makes into *exec (once).
static int capture_graph(ns_ctx *c, cudaGraphExec_t *exec,
                         cudaError_t (*fn)(ns_ctx *, cudaStream_t), const char *what)
{
    if (*exec) return NS_OK;
    cudaStream_t cs;
    NS_CUDA(c, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t le = fn(c, cs);
        e = cudaStreamEndCapture(cs, &g);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) {
        *exec = nullptr;
        cudaGetLastError();
        return cuda_err(c, e, what);
    }
    return NS_OK;
}

static int ensure_graph(ns_ctx *c)
{
    return capture_graph(c, &c->step_exec, ns::launch_step, "capture of the step graph");
}

int ns_step(ns_ctx *c, int iter0, int nsteps)
{
    if (!c) return set_err(nullptr, NS_ERR_PARAM, "ns_step: NULL context");
    if (nsteps < 0) return set_err(c, NS_ERR_PARAM, "nsteps=%d", nsteps);
    if (!c->have_state) return set_err(c, NS_ERR_STATE, "ns_step before ns_set_state");
    if (nsteps == 0) return NS_OK;
    NS_CUDA(c, cudaSetDevice(c->dev));
    int rc = ensure_graph(c);
    if (rc != NS_OK) return rc;
    if (c->src || c->sp.src) NS_CUDA(c, ns::launch_set_iter(c->d_iter, iter0, c->stream));
    for (int s = 0; s < nsteps; s++) NS_CUDA(c, cudaGraphLaunch(c->step_exec, c->stream));
    return NS_OK;
}

// A stage kernel whose TMA wait gave up leaves the error word set; it is
// reported (and cleared) at the next synchronisation.
static int check_kernel_err(ns_ctx *c)
{
    if (!c->d_err) return NS_OK;
    int h = 0;
    NS_CUDA(c, cudaMemcpyAsync(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    NS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (!h) return NS_OK;
    NS_CUDA(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
    NS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (h & ns::kCheckTag) return ns::check_error(h);
    return set_err(c, NS_ERR_TIMEOUT, "a stage kernel timed out waiting for its TMA tile");
}

int ns_synchronize(ns_ctx *c)
{
    if (!c) return set_err(nullptr, NS_ERR_PARAM, "ns_synchronize: NULL context");
    NS_CUDA(c, cudaSetDevice(c->dev));
    NS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_kernel_err(c);
}

// FP64 ns_rk_euler on page-locked host memory.  The host array is copied
// band by band (row bands, in U's own layout) by a copy engine into U2;
// each band is converted to planes as it lands, and stage 0's k_prim and
// k_first run on the bands already converted (k_first of band b once band
// b+1 holds its 3-row halo), so the transfer overlaps that work.  The rest
// of the step but the last stage's y sweep and ccpml is a second captured
// graph; those two run in row bands, and each finished band goes back to the
// host array by a copy engine while the next one is filtered.
static int rk_euler_banded(ns_ctx *c, double *U, int iter)
{
    const ns::Dims &d = c->d;
    int rc = capture_graph(c, &c->tail_exec, ns::launch_step_tail, "capture of the step tail");
    if (rc != NS_OK) return rc;
    if (!c->copy_stream) {
        NS_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        for (cudaEvent_t &ev : c->band_ev)
            NS_CUDA(c, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        for (cudaEvent_t &ev : c->wb_ev)
            NS_CUDA(c, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }
    constexpr int kMaxBands = ns::kMaxBands;
    const int nb = std::max(1, std::min(kMaxBands, d.jmax / 64));
    const int rows = ((d.jmax + nb - 1) / nb + 7) / 8 * 8;
    // the copies into U2 wait for earlier work on the context's stream
    static_assert(sizeof(c->band_ev) / sizeof(c->band_ev[0]) > kMaxBands, "band events");
    NS_CUDA(c, cudaEventRecord(c->band_ev[kMaxBands], c->stream));
    NS_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->band_ev[kMaxBands], 0));
    const size_t row_elems = (size_t)d.nk * d.imax;
    int r0[kMaxBands], nr[kMaxBands], n = 0;
    for (int j = 0; j < d.jmax; j += rows, n++) {
        r0[n] = j;
        nr[n] = std::min(rows, d.jmax - j);
        NS_CUDA(c, cudaMemcpyAsync(c->U2 + row_elems * j, U + row_elems * j,
                                   row_elems * nr[n] * sizeof(double), cudaMemcpyHostToDevice,
                                   c->copy_stream));
        NS_CUDA(c, cudaEventRecord(c->band_ev[n], c->copy_stream));
    }
    if (c->src) NS_CUDA(c, ns::launch_set_iter(c->d_iter, iter, c->stream));
    for (int b = 0; b < n; b++) {
        NS_CUDA(c, cudaStreamWaitEvent(c->stream, c->band_ev[b], 0));
        ns::Dims db = d;
        db.jmax = nr[b];
        NS_CUDA(c, ns::launch_aos_to_soa(c->U2 + row_elems * r0[b], c->U + (size_t)r0[b] * d.pitch,
                                         db, c->stream));
        if (c->visc) NS_CUDA(c, ns::launch_rows(c, NS_KC_PRIM, r0[b], nr[b], c->stream));
        if (b > 0) NS_CUDA(c, ns::launch_rows(c, NS_KC_FIRST, r0[b - 1], nr[b - 1], c->stream));
    }
    NS_CUDA(c, ns::launch_rows(c, NS_KC_FIRST, r0[n - 1], nr[n - 1], c->stream));
    c->have_state = true;
    NS_CUDA(c, cudaGraphLaunch(c->tail_exec, c->stream));
    // The last stage's y sweep and ccpml band by band.  Each finished band is
    // converted to U's own layout in the dudm planes (free once the last
    // stage's k_update has run) and sent home by a copy engine while the next
    // band is filtered.  The bands' pieces start their warm-ups at other
    // points than the whole sweep's, so on grids with more than one band the
    // result differs from ns_step's at the rounding level.
    int pb[ns::kMaxBands + 1];
    const int nwb = ns::bands_for(c, pb);
    double *stage_aos = c->dudm;
    for (int b = 0; b < nwb; b++) {
        NS_CUDA(c, ns::launch_filter_y_band(c, pb[b], pb[b + 1], c->stream));
        NS_CUDA(c, ns::launch_bc_band(c, pb, nwb, b, c->stream));
        int q0, q1;
        ns::band_rows(d, pb, nwb, b, q0, q1);
        ns::Dims db = d;
        db.jmax = q1 - q0;
        NS_CUDA(c, ns::launch_soa_to_aos(c->U + (size_t)q0 * d.pitch, stage_aos + row_elems * q0, db,
                                         c->stream));
        NS_CUDA(c, cudaEventRecord(c->wb_ev[b], c->stream));
        NS_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->wb_ev[b], 0));
        NS_CUDA(c, cudaMemcpyAsync(U + row_elems * q0, stage_aos + row_elems * q0,
                                   row_elems * (q1 - q0) * sizeof(double), cudaMemcpyDeviceToHost,
                                   c->copy_stream));
    }
    NS_CUDA(c, cudaEventRecord(c->wb_ev[ns::kMaxBands], c->copy_stream));
    NS_CUDA(c, cudaStreamWaitEvent(c->stream, c->wb_ev[ns::kMaxBands], 0));
    NS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_kernel_err(c);
}

int ns_rk_euler(ns_ctx *c, double *U, double t, int iter, int nk)
{
    (void)t;
    if (!c || !U) return set_err(c, NS_ERR_PARAM, "ns_rk_euler: NULL argument");
    if (nk != c->d.nk) return set_err(c, NS_ERR_PARAM, "nk=%d, context has %d", nk, c->d.nk);
    NS_CUDA(c, cudaSetDevice(c->dev));
    // Page-locked host memory that the device can address (every pinned
    // allocation under unified addressing): the layout kernels read U from
    // the host and write it back directly, one pass each way, with no
    // staging copy.  Any other host memory goes through set/get state.
    cudaPointerAttributes at{};
    void *dev_view = nullptr;
    if (cudaPointerGetAttributes(&at, U) == cudaSuccess && at.type == cudaMemoryTypeHost &&
        at.devicePointer)
        dev_view = at.devicePointer;
    else
        cudaGetLastError();
    if (!dev_view) {
        int rc = ns_set_state(c, U, NS_LAYOUT_FORTRAN);
        if (rc == NS_OK) rc = ns_step(c, iter, 1);
        if (rc == NS_OK) rc = ns_get_state(c, U, NS_LAYOUT_FORTRAN);
        return rc;
    }
    double *hv = static_cast<double *>(dev_view);
    if (!c->split) return rk_euler_banded(c, U, iter);
    NS_CUDA(c, ns::launch_aos_to_soa(hv, c->U, c->d, c->stream));
    if (c->split) NS_CUDA(c, ns::launch_split_from_full(c, c->U, c->stream));
    c->have_state = true;
    const int rc = ns_step(c, iter, 1);
    if (rc != NS_OK) return rc;
    if (c->split) NS_CUDA(c, ns::launch_split_to_full(c, c->U, c->stream));
    NS_CUDA(c, ns::launch_soa_to_aos(c->U, hv, c->d, c->stream));
    NS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_kernel_err(c);
}

int ns_get_probes(ns_ctx *c, int np, const int32_t *pi, const int32_t *pj, double *out)
{
    if (!c || np < 0 || (np > 0 && (!pi || !pj || !out)))
        return set_err(c, NS_ERR_PARAM, "ns_get_probes: bad argument");
    if (np == 0) return NS_OK;
    if (!c->have_state) return set_err(c, NS_ERR_STATE, "ns_get_probes before ns_set_state");
    std::vector<int32_t> idx(2 * (size_t)np);
    for (int q = 0; q < np; q++) {
        if (pi[q] < 1 || pi[q] > c->d.imax || pj[q] < 1 || pj[q] > c->d.jmax)
            return set_err(c, NS_ERR_PARAM, "probe %d at (%d,%d) is outside the grid", q, pi[q], pj[q]);
        idx[2 * q] = pi[q];
        idx[2 * q + 1] = pj[q];
    }
    NS_CUDA(c, cudaSetDevice(c->dev));
    if (np > c->probe_cap) {
        if (c->probe_buf) cudaFree(c->probe_buf);
        if (c->probe_idx) cudaFree(c->probe_idx);
        c->probe_buf = nullptr;
        c->probe_idx = nullptr;
        c->probe_cap = 0;
        int rc = dalloc(c, &c->probe_buf, (size_t)np * c->d.nk);
        if (rc == NS_OK) rc = dalloc(c, &c->probe_idx, 2 * (size_t)np);
        if (rc != NS_OK) return rc;
        c->probe_cap = np;
    }
    NS_CUDA(c, cudaMemcpyAsync(c->probe_idx, idx.data(), idx.size() * sizeof(int32_t),
                               cudaMemcpyHostToDevice, c->stream));
    if (c->split) NS_CUDA(c, ns::launch_split_to_full(c, c->U, c->stream));
    NS_CUDA(c, ns::launch_probes(c->U, c->d, np, c->probe_idx, c->probe_buf, c->stream));
    NS_CUDA(c, cudaMemcpyAsync(out, c->probe_buf, (size_t)np * c->d.nk * sizeof(double),
                               cudaMemcpyDeviceToHost, c->stream));
    NS_CUDA(c, cudaStreamSynchronize(c->stream));
    return NS_OK;
}

int ns_check_finite(ns_ctx *c, int64_t *nonfinite)
{
    if (!c) return set_err(nullptr, NS_ERR_PARAM, "ns_check_finite: NULL context");
    if (!c->have_state) return set_err(c, NS_ERR_STATE, "ns_check_finite before ns_set_state");
    NS_CUDA(c, cudaSetDevice(c->dev));
    unsigned long long h = 0;
    NS_CUDA(c, cudaMemsetAsync(c->d_count, 0, sizeof(unsigned long long), c->stream));
    if (c->split) NS_CUDA(c, ns::launch_split_to_full(c, c->U, c->stream));
    NS_CUDA(c, ns::launch_count_nonfinite(c->U, c->d, c->d_count, c->stream));
    NS_CUDA(c, cudaMemcpyAsync(&h, c->d_count, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    NS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (nonfinite) *nonfinite = (int64_t)h;
    if (h) return set_err(c, NS_ERR_NONFINITE, "%llu non-finite values in the state", h);
    return NS_OK;
}

int ns_set_stream(ns_ctx *c, void *stream)
{
    if (!c) return set_err(nullptr, NS_ERR_PARAM, "ns_set_stream: NULL context");
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return NS_OK;
}

int ns_get_stream(ns_ctx *c, void **stream)
{
    if (!c || !stream) return set_err(c, NS_ERR_PARAM, "ns_get_stream: NULL argument");
    *stream = (void *)c->stream;
    return NS_OK;
}

int ns_state_device(ns_ctx *c, void **dptr, int64_t *pitch)
{
    if (!c || !dptr || !pitch) return set_err(c, NS_ERR_PARAM, "ns_state_device: NULL argument");
    *dptr = (void *)c->U;
    *pitch = c->d.pitch;
    return NS_OK;
}

int ns_step_launches(ns_ctx *c, int *launches)
{
    if (!c || !launches) return set_err(c, NS_ERR_PARAM, "ns_step_launches: NULL argument");
    *launches = c->launches_per_step;
    return NS_OK;
}

int ns_coef_table(int which, double *out)
{
    if (!out) return 0;
    const double *const tabs[13] = {kA, kA4, kA5, kA6, kA4b, kA5b, kA6b, nullptr,
                                    kDfbX, kDfbY, kAlpha, kBeta, kCt};
    const int lens[13] = {3, 7, 7, 7, 7, 7, 7, 13, 7, 7, 6, 6, 6};
    if (which < 0 || which > 12) return 0;
    if (which == 7) {
        for (int s = -6; s <= 6; s++) out[s + 6] = kDf[s < 0 ? -s : s];
    } else {
        for (int z = 0; z < lens[which]; z++) out[z] = tabs[which][z];
    }
    return lens[which];
}

int ns_filter_warmup(ns_ctx *c, int *warmup)
{
    if (!c || !warmup) return set_err(c, NS_ERR_PARAM, "ns_filter_warmup: NULL argument");
    *warmup = c->warm;
    return NS_OK;
}

int ns_time_kernels(ns_ctx *c, int iter0, int reps, double *ms, int *launches)
{
    if (!c || !ms || !launches || reps < 1)
        return set_err(c, NS_ERR_PARAM, "ns_time_kernels: bad argument");
    if (!c->have_state) return set_err(c, NS_ERR_STATE, "ns_time_kernels before ns_set_state");
    NS_CUDA(c, cudaSetDevice(c->dev));
    int cls[ns::kMaxStepLaunches], stage[ns::kMaxStepLaunches];
    const int n = ns::step_sequence(c, cls, stage);
    std::vector<cudaEvent_t> ev(n + 1);
    for (auto &e : ev) NS_CUDA(c, cudaEventCreate(&e));
    std::vector<double> tot(NS_KC_COUNT, 0.0);
    for (int k = 0; k < NS_KC_COUNT; k++) launches[k] = 0;
    for (int q = 0; q < n; q++) launches[cls[q]]++;
    int rc = NS_OK;
    if (c->src || c->sp.src) {
        cudaError_t e = ns::launch_set_iter(c->d_iter, iter0, c->stream);
        if (e != cudaSuccess) rc = cuda_err(c, e, "set iter");
    }
    for (int r = 0; r < reps && rc == NS_OK; r++) {
        cudaError_t e = cudaEventRecord(ev[0], c->stream);
        for (int q = 0; q < n && e == cudaSuccess; q++) {
            e = ns::launch_kernel(c, cls[q], stage[q], c->stream);
            if (e == cudaSuccess) e = cudaEventRecord(ev[q + 1], c->stream);
        }
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[n]);
        for (int q = 0; q < n && e == cudaSuccess; q++) {
            float t = 0.f;
            e = cudaEventElapsedTime(&t, ev[q], ev[q + 1]);
            tot[cls[q]] += t;
        }
        if (e != cudaSuccess) rc = cuda_err(c, e, "ns_time_kernels");
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (int k = 0; k < NS_KC_COUNT; k++)
        ms[k] = launches[k] ? tot[k] / ((double)reps * launches[k]) : 0.0;
    return rc;
}

const char *ns_kernel_name(int k)
{
    static const char *names[NS_KC_COUNT] = {
        "k_stage_sin",   "k_prim",          "k_first",          "k_update",
        "k_filter_x",    "k_filter_y",      "k_bc",             "k_split_stage",
        "k_split_filter_x", "k_split_filter_y", "k_split_bc", "k_split_visc"};
    return (k >= 0 && k < NS_KC_COUNT) ? names[k] : "";
}

}  // extern "C"
