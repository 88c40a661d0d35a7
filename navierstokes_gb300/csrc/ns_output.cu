// ns_output.cu -- the device side of the program around the step:
//   * fields constant along i expanded on the device from their rows
//     (Ub and the initial U = Ub of init.f90:376-396);
//   * the vorticity of the output path, outt.f90:43-49, with the DRP
//     derivatives of diffall.f90:5-380, which apply no metric;
//   * the contorno_<n>.dat writer (outt.f90:40-55);
//   * the probe recorder of the time loop (euler.f90:152-157).
#include <algorithm>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#include "ns_internal.cuh"

namespace ns {

__global__ void __launch_bounds__(512)
    k_rows_to_planes(const double *__restrict__ rows, double *__restrict__ planes, Dims d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.imax) return;
    for (int j = blockIdx.y * blockDim.y + threadIdx.y; j < d.jmax; j += gridDim.y * blockDim.y)
        for (int k = 0; k < d.nk; k++)
            planes[k * d.plane + (long long)j * d.pitch + i] = rows[k + (long long)d.nk * j];
}

cudaError_t launch_rows_to_planes(const double *rows, double *planes, const Dims &d,
                                  cudaStream_t s)
{
    const dim3 blk(128, 4);
    const dim3 grd((d.imax + 127) / 128, std::min((d.jmax + 3) / 4, 4096));
    k_rows_to_planes<<<grd, blk, 0, s>>>(rows, planes, d);
    return cudaGetLastError();
}

// omega = dv/dx - du/dy at every point: dUcdm(3) - dUcdn(2) of outt.f90:47
// with vx, vy the per-position tables of 1/dm, 1/dn times the DRP weights.
__global__ void __launch_bounds__(256)
    k_vorticity(Dims d, const double *__restrict__ U, const double *__restrict__ vx,
                const double *__restrict__ vy, double *__restrict__ om)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= d.imax || j >= d.jmax) return;
    const long long idx = (long long)j * d.pitch + i;
    const double dvdx = dline(U + 2 * d.plane + idx, 1, i, d.imax, vx + kCoefStride * i);
    const double dudy = dline(U + d.plane + idx, d.pitch, j, d.jmax, vy + kCoefStride * j);
    om[idx] = dvdx - dudy;
}

}  // namespace ns

namespace {

int oerr(ns_ctx *c, int code, const std::string &m)
{
    if (c) c->err = m;
    ns::record_error(m.c_str());
    return code;
}

#define O_CUDA(c, call)                                                                          \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return oerr((c), NS_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_));      \
    } while (0)

int upload(ns_ctx *c, double **dst, const std::vector<double> &v)
{
    O_CUDA(c, cudaMalloc(dst, v.size() * sizeof(double)));
    O_CUDA(c, cudaMemcpyAsync(*dst, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice,
                              c->stream));
    return NS_OK;
}

// omega plane on the device from the current state
int vorticity_device(ns_ctx *c)
{
    const ns::Dims &d = c->d;
    if (!c->vx) {
        // diffall.f90: dudx / dx4 / dx5 / dx6 with dm, dn and no metric
        std::vector<double> tx, ty;
        ns::build_line_coef(tx, d.imax, c->p.dm, nullptr, 0, NS_METRIC_BANDS);
        ns::build_line_coef(ty, d.jmax, c->p.dn, nullptr, 0, NS_METRIC_BANDS);
        int rc;
        if ((rc = upload(c, &c->vx, tx)) || (rc = upload(c, &c->vy, ty))) return rc;
        O_CUDA(c, cudaMalloc(&c->omega, (size_t)d.plane * sizeof(double)));
    }
    if (c->split) O_CUDA(c, ns::launch_split_to_full(c, c->U, c->stream));
    const dim3 blk(32, 8), grd((d.imax + 31) / 32, (d.jmax + 7) / 8);
    ns::k_vorticity<<<grd, blk, 0, c->stream>>>(d, c->U, c->vx, c->vy, c->omega);
    O_CUDA(c, cudaGetLastError());
    return NS_OK;
}

}  // namespace

extern "C" {

int ns_vorticity(ns_ctx *c, double *omega)
{
    if (!c || !omega) return oerr(c, NS_ERR_PARAM, "ns_vorticity: NULL argument");
    if (!c->have_state) return oerr(c, NS_ERR_STATE, "ns_vorticity before ns_set_state");
    O_CUDA(c, cudaSetDevice(c->dev));
    int rc = vorticity_device(c);
    if (rc != NS_OK) return rc;
    const ns::Dims &d = c->d;
    const size_t row = (size_t)d.imax * sizeof(double);
    O_CUDA(c, cudaMemcpy2DAsync(omega, row, c->omega, d.pitch * sizeof(double), row,
                                (size_t)d.jmax, cudaMemcpyDeviceToHost, c->stream));
    O_CUDA(c, cudaStreamSynchronize(c->stream));
    return NS_OK;
}

int ns_write_contorno(ns_ctx *c, const char *path, const double *m, const double *n)
{
    if (!c || !path || !m || !n) return oerr(c, NS_ERR_PARAM, "ns_write_contorno: NULL argument");
    const ns::Dims &d = c->d;
    const int imax = d.imax, jmax = d.jmax, nk = d.nk;
    std::vector<double> U((size_t)nk * imax * jmax), om((size_t)imax * jmax);
    int rc = ns_vorticity(c, om.data());
    if (rc != NS_OK) return rc;
    if ((rc = ns_get_state(c, U.data(), NS_LAYOUT_FORTRAN)) != NS_OK) return rc;
    std::FILE *f = std::fopen(path, "w");
    if (!f) return oerr(c, NS_ERR_PARAM, std::string("cannot open ") + path);
    // records of column i: j = 1..jmax, then an empty record (outt.f90:44-50)
    const int nval = (nk >= 5) ? 8 : 7;
    const size_t rec_len = (size_t)nval * 26 + 1;
    auto format_columns = [&](int i0, int i1, std::string &out) {
        out.resize((size_t)(i1 - i0) * ((size_t)jmax * rec_len + 1));
        char *p = &out[0];
        for (int i = i0; i < i1; i++) {
            for (int j = 0; j < jmax; j++) {
                const double *u = &U[(size_t)nk * ((size_t)i + (size_t)imax * j)];
                double v[8] = {m[i], n[j], u[0], u[1], u[2], u[3], om[(size_t)i + (size_t)imax * j],
                               nk >= 5 ? u[4] : 0.0};
                for (int q = 0; q < nval; q++) {
                    *p++ = ' ';
                    ns_format_real(v[q], p, 26);
                    p += 25;
                }
                *p++ = '\n';
            }
            *p++ = '\n';
        }
        out.resize((size_t)(p - &out[0]));
    };
    const int nthr = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const int cols = 8;
    std::vector<std::string> bufs(nthr);
    bool ok = true;
    for (int i0 = 0; i0 < imax && ok; i0 += nthr * cols) {
        std::vector<std::thread> th;
        for (int t = 0; t < nthr; t++) {
            const int a = i0 + t * cols, b = std::min(imax, a + cols);
            if (a >= b) {
                bufs[t].clear();
                continue;
            }
            th.emplace_back(format_columns, a, b, std::ref(bufs[t]));
        }
        for (auto &x : th) x.join();
        for (int t = 0; t < nthr && ok; t++)
            ok = std::fwrite(bufs[t].data(), 1, bufs[t].size(), f) == bufs[t].size();
    }
    if (std::fclose(f) != 0) ok = false;
    if (!ok) return oerr(c, NS_ERR_PARAM, std::string("write to ") + path + " failed");
    return NS_OK;
}

int ns_probes_arm(ns_ctx *c, int npts, const int32_t *pi, const int32_t *pj, int capacity)
{
    if (!c || npts < 1 || !pi || !pj || capacity < 1)
        return oerr(c, NS_ERR_PARAM, "ns_probes_arm: bad argument");
    std::vector<int32_t> idx(2 * (size_t)npts);
    for (int q = 0; q < npts; q++) {
        if (pi[q] < 1 || pi[q] > c->d.imax || pj[q] < 1 || pj[q] > c->d.jmax)
            return oerr(c, NS_ERR_PARAM, "probe " + std::to_string(q) + " lies outside the grid");
        idx[2 * q] = pi[q];
        idx[2 * q + 1] = pj[q];
    }
    O_CUDA(c, cudaSetDevice(c->dev));
    O_CUDA(c, cudaStreamSynchronize(c->stream));
    if (c->rec_buf) cudaFree(c->rec_buf);
    if (c->rec_idx) cudaFree(c->rec_idx);
    c->rec_buf = nullptr;
    c->rec_idx = nullptr;
    c->rec_cap = c->rec_npts = c->rec_n = 0;
    O_CUDA(c, cudaMalloc(&c->rec_buf, (size_t)capacity * npts * c->d.nk * sizeof(double)));
    O_CUDA(c, cudaMalloc(&c->rec_idx, idx.size() * sizeof(int32_t)));
    O_CUDA(c, cudaMemcpy(c->rec_idx, idx.data(), idx.size() * sizeof(int32_t),
                         cudaMemcpyHostToDevice));
    c->rec_cap = capacity;
    c->rec_npts = npts;
    return NS_OK;
}

int ns_probes_capture(ns_ctx *c)
{
    if (!c) return oerr(c, NS_ERR_PARAM, "ns_probes_capture: NULL context");
    if (!c->rec_cap) return oerr(c, NS_ERR_STATE, "ns_probes_capture before ns_probes_arm");
    if (!c->have_state) return oerr(c, NS_ERR_STATE, "ns_probes_capture before ns_set_state");
    if (c->rec_n >= c->rec_cap) return oerr(c, NS_ERR_STATE, "probe recorder is full");
    O_CUDA(c, cudaSetDevice(c->dev));
    if (c->split) O_CUDA(c, ns::launch_split_to_full(c, c->U, c->stream));
    double *slot = c->rec_buf + (size_t)c->rec_n * c->rec_npts * c->d.nk;
    O_CUDA(c, ns::launch_probes(c->U, c->d, c->rec_npts, c->rec_idx, slot, c->stream));
    c->rec_n++;
    return NS_OK;
}

int ns_probes_drain(ns_ctx *c, double *out, int *nrec)
{
    if (!c || !nrec || (c->rec_n > 0 && !out))
        return oerr(c, NS_ERR_PARAM, "ns_probes_drain: NULL argument");
    O_CUDA(c, cudaSetDevice(c->dev));
    if (c->rec_n > 0)
        O_CUDA(c, cudaMemcpyAsync(out, c->rec_buf,
                                  (size_t)c->rec_n * c->rec_npts * c->d.nk * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream));
    O_CUDA(c, cudaStreamSynchronize(c->stream));
    *nrec = c->rec_n;
    c->rec_n = 0;
    return NS_OK;
}

}  // extern "C"
