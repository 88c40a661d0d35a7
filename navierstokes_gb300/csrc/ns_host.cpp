// ns_host.cpp -- the program around the step, on the host: the dados.in
// reader (init_read, init.f90:10-52), the grid and base-flow setup
// (init_dados, init.f90:56-210; init_variables, init.f90:341-404), the
// list-directed number layout of the reference's output files, and the time
// loop of euler.f90:123-169 with its probe files and field dumps.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "ns_gb300.h"

namespace ns {
void record_error(const char *msg);
}

namespace {

int fail(int code, const std::string &msg)
{
    ns::record_error(msg.c_str());
    return code;
}

// ---------------------------------------------------------------------------
// Namelist groups of init.f90:18-23.  The second `namelist /grid/`
// statement continues group grid, so both &grid groups accept all twelve
// names.
// ---------------------------------------------------------------------------
struct Var {
    const char *name;  // lower case
    char type;         // 'i' int32, 'r' REAL(8)
    size_t off;
};

#define NS_IV(nm, field) Var{nm, 'i', offsetof(ns_dados, field)}
#define NS_RV(nm, field) Var{nm, 'r', offsetof(ns_dados, field)}
#define NS_RA(nm, field, k) Var{nm, 'r', offsetof(ns_dados, field) + (k) * sizeof(double)}

const Var kGrid[] = {NS_IV("imax", imax), NS_IV("jmax", jmax), NS_IV("maxit", maxit),
                     NS_RV("dt", dt),     NS_RV("sigmaf", sigmaf), NS_IV("cgd", cgd),
                     NS_IV("cfd", cfd),   NS_IV("ctd", ctd),   NS_IV("d", D),
                     NS_RV("c1b", c1b),   NS_RV("c2b", c2b),   NS_RV("c3b", c3b)};
const Var kFreq[] = {NS_RV("r0_acous", r0_acous),     NS_RV("amplitude", amplitude),
                     NS_RV("m_pt_acous", m_pt_acous), NS_RV("n_pt_acous", n_pt_acous),
                     NS_RV("wfi", wfi),               NS_RV("wff", wff),
                     NS_RV("wf", wf),                 NS_IV("iterw", iterw),
                     NS_RA("pxfft1", pxfft, 0),       NS_RA("pxfft2", pxfft, 1),
                     NS_RA("pxfft3", pxfft, 2),       NS_RA("pxfft4", pxfft, 3),
                     NS_RA("pxfft5", pxfft, 4)};
const Var kFreeadm[] = {NS_RV("mmin", mmin),      NS_RV("mmax", mmax),      NS_RV("nmin", nmin),
                        NS_RV("nmax", nmax),      NS_RA("pxr1", pxr, 0),    NS_RA("pyr1", pyr, 0),
                        NS_RA("pxr2", pxr, 1),    NS_RA("pyr2", pyr, 1),    NS_RA("pxr3", pxr, 2),
                        NS_RA("pyr3", pyr, 2)};
const Var kFlow[] = {NS_RV("u1", U1), NS_RV("u2", U2), NS_RV("re", Re),    NS_RV("pr", Pr),
                     NS_RV("t1", T1), NS_RV("t2", T2), NS_RV("tref", Tref)};
const Var kMpi[] = {NS_IV("num_procs_x", num_procs_x), NS_IV("num_procs_y", num_procs_y)};

#undef NS_IV
#undef NS_RV
#undef NS_RA

bool is_ident_char(char c)
{
    return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || (c >= '0' && c <= '9') || c == '_';
}

char lower(char c) { return (c >= 'A' && c <= 'Z') ? (char)(c - 'A' + 'a') : c; }

class NamelistReader {
  public:
    explicit NamelistReader(const std::string &text) : t_(text) {}

    // read (unit, nml=<name>): finds the next "&name" (or "$name") from the
    // current position, then reads name = value items up to '/', &end or $end.
    int read_group(const char *name, const Var *vars, size_t nvars, ns_dados *out)
    {
        for (;;) {
            skip(false);
            if (pos_ >= t_.size())
                return error(std::string("namelist group &") + name + " not found");
            const char c = t_[pos_];
            if ((c == '&' || c == '$') && ident_at(pos_ + 1, name)) {
                pos_ += 1 + std::strlen(name);
                break;
            }
            next_line();
        }
        for (;;) {
            skip(true);
            if (pos_ >= t_.size())
                return error(std::string("namelist group &") + name + " has no terminator");
            const char c = t_[pos_];
            if (c == '/') {
                pos_++;
                return NS_OK;
            }
            if (c == '&' || c == '$') {
                if (ident_at(pos_ + 1, "end")) {
                    pos_ += 4;
                    return NS_OK;
                }
                return error(std::string("group start inside namelist group &") + name);
            }
            std::string id;
            while (pos_ < t_.size() && is_ident_char(t_[pos_])) id += lower(t_[pos_++]);
            if (id.empty())
                return error(std::string("unexpected character '") + c + "' in &" + name);
            const Var *v = nullptr;
            for (size_t q = 0; q < nvars; q++)
                if (id == vars[q].name) v = &vars[q];
            if (!v) return error("variable '" + id + "' is not in namelist group &" + name);
            skip(false);
            if (pos_ >= t_.size() || t_[pos_] != '=')
                return error("expected '=' after '" + id + "' in &" + name);
            pos_++;
            skip(false);
            std::string tok;
            while (pos_ < t_.size()) {
                const char d = t_[pos_];
                if (d == ' ' || d == '\t' || d == '\r' || d == '\n' || d == ',' || d == '/' ||
                    d == '!')
                    break;
                tok += d;
                pos_++;
            }
            int rc = store(v, tok, out);
            if (rc != NS_OK) return rc;
        }
    }

  private:
    const std::string &t_;
    size_t pos_ = 0;

    int line() const { return 1 + (int)std::count(t_.begin(), t_.begin() + (long)pos_, '\n'); }

    int error(const std::string &m) const
    {
        return fail(NS_ERR_PARAM, "dados.in line " + std::to_string(line()) + ": " + m);
    }

    void next_line()
    {
        while (pos_ < t_.size() && t_[pos_] != '\n') pos_++;
        if (pos_ < t_.size()) pos_++;
    }

    // blanks, '!' comments and (between items) commas
    void skip(bool commas)
    {
        while (pos_ < t_.size()) {
            const char c = t_[pos_];
            if (c == '!') {
                while (pos_ < t_.size() && t_[pos_] != '\n') pos_++;
            } else if (c == ' ' || c == '\t' || c == '\r' || c == '\n' || (commas && c == ',')) {
                pos_++;
            } else {
                break;
            }
        }
    }

    bool ident_at(size_t p, const char *name) const
    {
        const size_t len = std::strlen(name);
        if (p + len > t_.size()) return false;
        for (size_t q = 0; q < len; q++)
            if (lower(t_[p + q]) != name[q]) return false;
        return p + len == t_.size() || !is_ident_char(t_[p + len]);
    }

    int store(const Var *v, const std::string &tok, ns_dados *out) const
    {
        if (tok.empty()) return error(std::string("no value for '") + v->name + "'");
        char *base = reinterpret_cast<char *>(out) + v->off;
        char *end = nullptr;
        if (v->type == 'i') {
            const long x = std::strtol(tok.c_str(), &end, 10);
            if (*end != '\0' || x < -2147483647L || x > 2147483647L)
                return error("'" + tok + "' is not an integer value for '" + v->name + "'");
            const int32_t y = (int32_t)x;
            std::memcpy(base, &y, sizeof y);
        } else {
            std::string s = tok;
            for (char &c : s)
                if (c == 'd' || c == 'D') c = 'e';
            const double x = std::strtod(s.c_str(), &end);
            if (*end != '\0' || s.find_first_of("xXpP") != std::string::npos)
                return error("'" + tok + "' is not a real value for '" + v->name + "'");
            std::memcpy(base, &x, sizeof x);
        }
        return NS_OK;
    }
};

// ---------------------------------------------------------------------------
// List-directed REAL(8) items.
// ---------------------------------------------------------------------------
void put_field(const char *body, char *buf)
{
    // right-justified in 25 columns
    const int len = (int)std::strlen(body);
    const int pad = std::max(0, 25 - len);
    std::memset(buf, ' ', (size_t)pad);
    std::memcpy(buf + pad, body, (size_t)std::min(len, 25));
    buf[25] = '\0';
}

std::string join(const char *dir, const std::string &file)
{
    if (!dir || !*dir) return file;
    std::string d(dir);
    if (d.back() != '/') d += '/';
    return d + file;
}

// One list-directed record: a blank, then the items separated by blanks.
void write_record(std::FILE *f, const double *v, int n)
{
    char line[27 * 16 + 2];
    char *p = line;
    for (int q = 0; q < n; q++) {
        *p++ = ' ';
        ns_format_real(v[q], p, 26);
        p += 25;
    }
    *p++ = '\n';
    std::fwrite(line, 1, (size_t)(p - line), f);
}

}  // namespace

extern "C" {

int ns_parse_dados(const char *text, ns_dados *out)
{
    if (!text || !out) return fail(NS_ERR_PARAM, "ns_parse_dados: NULL argument");
    ns_dados d;
    std::memset(&d, 0, sizeof d);
    const std::string s(text);
    NamelistReader r(s);
    int rc;
    if ((rc = r.read_group("grid", kGrid, sizeof kGrid / sizeof kGrid[0], &d)) ||
        (rc = r.read_group("freq", kFreq, sizeof kFreq / sizeof kFreq[0], &d)) ||
        (rc = r.read_group("freeadm", kFreeadm, sizeof kFreeadm / sizeof kFreeadm[0], &d)) ||
        (rc = r.read_group("flow", kFlow, sizeof kFlow / sizeof kFlow[0], &d)) ||
        (rc = r.read_group("grid", kGrid, sizeof kGrid / sizeof kGrid[0], &d)) ||
        (rc = r.read_group("mpi", kMpi, sizeof kMpi / sizeof kMpi[0], &d)))
        return rc;
    *out = d;
    return NS_OK;
}

int ns_read_dados(const char *path, ns_dados *out)
{
    if (!path || !out) return fail(NS_ERR_PARAM, "ns_read_dados: NULL argument");
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(NS_ERR_PARAM, std::string("cannot open ") + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ns_parse_dados(ss.str().c_str(), out);
}

// init_dados, init.f90:56-210
int ns_dados_grid(const ns_dados *d, int quirk_buffer, double *m, double *n, double *meshx,
                  double *meshy, double *sigmax, double *sigmay, double *dm_dn, int32_t *probe_ij)
{
    if (!d || !m || !n || !meshx || !meshy || !sigmax || !sigmay)
        return fail(NS_ERR_PARAM, "ns_dados_grid: NULL argument");
    const int imax = d->imax, jmax = d->jmax, D = d->D;
    if (imax < 2 || jmax < 2 || D < 0 || !(d->mmax > d->mmin) || !(d->nmax > d->nmin))
        return fail(NS_ERR_PARAM, "ns_dados_grid: need imax, jmax >= 2, D >= 0, mmax > mmin, "
                                  "nmax > nmin");
    const double mmin = d->mmin, mmax = d->mmax, nmin = d->nmin, nmax = d->nmax;
    // real(imax-1) is a default (single precision) REAL: exact here
    const double dm = (mmax - mmin) / (double)(float)(imax - 1);
    const double dn = (nmax - nmin) / (double)(float)(jmax - 1);
    if (probe_ij) {
        // init.f90:80-85
        for (int q = 0; q < 3; q++) {
            probe_ij[2 * q] = (int32_t)(-mmin / dm + d->pxr[q] / dm + 1);
            probe_ij[2 * q + 1] = (int32_t)(-nmin / dn + d->pyr[q] / dn + 1);
        }
    }
    const double Dx = dm * D, Dy = dn * D;
    const double xli = mmin + Dx, xld = mmax - Dx, yli = nmin + Dy, yls = nmax - Dy;
    for (int i = 1; i <= imax; i++) m[i - 1] = mmin + (double)(float)(i - 1) * dm;
    for (int j = 1; j <= jmax; j++) n[j - 1] = nmin + (double)(float)(j - 1) * dn;
    const double Aa = 2.0, alpham = 2.0;
    for (int i = 1; i <= imax; i++) {
        meshx[i - 1] = 1.0;
        if (i >= 1 && i <= D + 1)
            meshx[i - 1] = 1.0 / (1.0 + Aa * std::pow(std::fabs((m[i - 1] - xli) / Dx), alpham));
        if (i >= imax - D && i <= imax)
            meshx[i - 1] = 1.0 / (1.0 + Aa * std::pow(std::fabs((m[i - 1] - xld) / Dx), alpham));
    }
    for (int j = 1; j <= jmax; j++) {
        meshy[j - 1] = 1.0;
        if (j >= 1 && j <= D + 1)
            meshy[j - 1] = 1.0 / (1.0 + Aa * std::pow(std::fabs((n[j - 1] - yli) / Dy), alpham));
        if (j >= jmax - D + 1 && j <= jmax)
            meshy[j - 1] = 1.0 / (1.0 + Aa * std::pow(std::fabs((n[j - 1] - yls) / Dy), alpham));
    }
    // imaxpml/jmaxpml are never assigned in the reference (global.f90:86)
    const int imaxpml = quirk_buffer ? 0 : D, jmaxpml = quirk_buffer ? 0 : D;
    const double c1b = d->c1b, c2b = d->c2b;
    auto prof = [&](double x) {
        return (1.0 - c1b * x * x) * (1.0 - (1.0 - std::exp(c2b * x * x)) / (1.0 - std::exp(c2b)));
    };
    for (int i = 1; i <= imax; i++) {
        sigmax[i - 1] = 0.0;
        if (i >= 1 && i <= imaxpml) sigmax[i - 1] = prof((m[i - 1] - xli) / (mmin - xli));
        if (i >= imax - D + 1 && i <= imax) sigmax[i - 1] = prof((m[i - 1] - xld) / (mmax - xld));
    }
    for (int j = 1; j <= jmax; j++) {
        sigmay[j - 1] = 0.0;
        if (j >= 1 && j <= jmaxpml) sigmay[j - 1] = prof((n[j - 1] - yli) / (nmin - yli));
        if (j >= jmax - D + 1 && j <= jmax) sigmay[j - 1] = prof((n[j - 1] - yls) / (nmax - yls));
    }
    if (dm_dn) {
        dm_dn[0] = dm;
        dm_dn[1] = dn;
    }
    return NS_OK;
}

// init_variables, init.f90:351-373
int ns_dados_profiles(const ns_dados *d, const double *n, double *uba, double *Tb, double *rhob,
                      double *psib)
{
    if (!d || !n || !uba || !Tb || !rhob || !psib)
        return fail(NS_ERR_PARAM, "ns_dados_profiles: NULL argument");
    const double u1b = d->U1, u2b = d->U2, T1 = d->T1, T2 = d->T2;
    if (u1b == u2b) return fail(NS_ERR_PARAM, "ns_dados_profiles: U1 == U2");
    const double deltamx = 0.4, gamma = 1.4, psi1 = 1.0, psi2 = 0.0;
    for (int j = 0; j < d->jmax; j++) {
        uba[j] = 0.5 * (u1b + u2b + (u1b - u2b) * std::tanh(2.0 * n[j] / deltamx));
        Tb[j] = T1 * (uba[j] - u2b) / (u1b - u2b) + T2 * (u1b - uba[j]) / (u1b - u2b) +
                (gamma - 1.0) / 2.0 * (u1b - uba[j]) * (uba[j] - u2b);
        rhob[j] = 1.0 / (Tb[j]);
        psib[j] = 0.5 * (psi1 + psi2 + (psi1 - psi2) * std::tanh(2.0 * n[j] / deltamx));
    }
    return NS_OK;
}

int ns_create_dados(const ns_dados *d, int nk, int device, int quirk_buffer, ns_ctx **out)
{
    if (!d || !out) return fail(NS_ERR_PARAM, "ns_create_dados: NULL argument");
    *out = nullptr;
    if (nk != 4 && nk != 5) return fail(NS_ERR_PARAM, "ns_create_dados: nk must be 4 or 5");
    if (d->imax < 2 || d->jmax < 2) return fail(NS_ERR_PARAM, "ns_create_dados: bad grid size");
    const int imax = d->imax, jmax = d->jmax;
    std::vector<double> m(imax), n(jmax), mx(imax), my(jmax), sx(imax), sy(jmax), hh(2);
    int rc = ns_dados_grid(d, quirk_buffer, m.data(), n.data(), mx.data(), my.data(), sx.data(),
                           sy.data(), hh.data(), nullptr);
    if (rc != NS_OK) return rc;
    std::vector<double> uba(jmax), Tb(jmax), rhob(jmax), psib(jmax);
    if ((rc = ns_dados_profiles(d, n.data(), uba.data(), Tb.data(), rhob.data(), psib.data())))
        return rc;
    const double gamma = 1.4;  // init.f90:361
    std::vector<double> rows((size_t)nk * jmax);
    for (int j = 0; j < jmax; j++) {
        double *r = &rows[(size_t)nk * j];
        r[0] = rhob[j];
        r[1] = uba[j];
        r[2] = 0.0;
        r[3] = 1.0 / gamma;
        if (nk == 5) r[4] = psib[j];
    }
    ns_params p;
    ns_params_init(&p);
    p.imax = imax;
    p.jmax = jmax;
    p.nk = nk;
    p.D = d->D;
    p.inviscid = 0;
    p.metric_mode = NS_METRIC_BANDS;
    p.precision = NS_PREC_FP64;
    p.source_mode = NS_SRC_GAUSSIAN;
    p.device = device;
    p.ub_layout = NS_LAYOUT_ROWS;
    p.dt = d->dt;
    p.dm = hh[0];
    p.dn = hh[1];
    p.sigmaf = d->sigmaf;
    p.gamma = gamma;
    p.Re = d->Re;
    p.Pr = d->Pr;
    p.Tref = d->Tref;
    p.amplitude = d->amplitude;
    p.wf = d->wf;
    p.m_pt = d->m_pt_acous;
    p.n_pt = d->n_pt_acous;
    p.r0 = d->r0_acous;
    p.m = m.data();
    p.n = n.data();
    p.meshx = mx.data();
    p.meshy = my.data();
    p.sigmax = sx.data();
    p.sigmay = sy.data();
    p.rhob = rhob.data();
    p.psib = psib.data();
    p.Ub = rows.data();
    ns_ctx *c = nullptr;
    if ((rc = ns_create(&p, &c)) != NS_OK) return rc;
    if ((rc = ns_set_state(c, rows.data(), NS_LAYOUT_ROWS)) != NS_OK) {
        ns_destroy(c);
        return rc;
    }
    *out = c;
    return NS_OK;
}

int ns_format_real(double x, char *buf, int len)
{
    if (!buf || len < 26) return -1;
    char body[48];
    if (std::isnan(x)) {
        put_field("NaN", buf);
        return 25;
    }
    if (std::isinf(x)) {
        put_field(x > 0 ? "Infinity" : "-Infinity", buf);
        return 25;
    }
    const bool neg = std::signbit(x);
    const double a = std::fabs(x);
    int e10 = 0;
    char mant[40];
    if (a != 0.0) {
        // 17 significant digits, rounded once; the exponent of the rounded value
        std::snprintf(mant, sizeof mant, "%.16e", a);
        const char *ep = std::strchr(mant, 'e');
        e10 = std::atoi(ep + 1);
    }
    if (a == 0.0 || (e10 >= -1 && e10 <= 16)) {
        // F20.(16-e10) then five blanks (the exponent field's width)
        const int dec = (a == 0.0) ? 16 : 16 - e10;
        std::snprintf(body, sizeof body, "%s%.*f%s", neg ? "-" : "", dec, a, dec == 0 ? "." : "");
        const int blen = (int)std::strlen(body);
        const int pad = std::max(0, 20 - blen);
        std::memset(buf, ' ', (size_t)pad);
        std::memcpy(buf + pad, body, (size_t)std::min(blen, 20));
        std::memset(buf + 20, ' ', 5);
        buf[25] = '\0';
        return 25;
    }
    // E25.17E3: d.dddddddddddddddd E sxxx
    char digits[24];
    std::snprintf(digits, sizeof digits, "%.*s", 18, mant);  // "d.dddddddddddddddd"
    std::snprintf(body, sizeof body, "%s%sE%c%03d", neg ? "-" : "", digits, e10 < 0 ? '-' : '+',
                  std::abs(e10));
    put_field(body, buf);
    return 25;
}

int ns_run_euler(const char *dados_path, const char *outdir, int nk, int device, int maxit,
                 int flags)
{
    ns_dados d;
    int rc = ns_read_dados(dados_path ? dados_path : "dados.in", &d);
    if (rc != NS_OK) return rc;
    const bool quiet = (flags & NS_RUN_QUIET) != 0;
    const bool fields = (flags & NS_RUN_NO_CONTORNO) == 0;
    const int imax = d.imax, jmax = d.jmax;
    if (imax < 13 || jmax < 13) return fail(NS_ERR_PARAM, "ns_run_euler: grid too small");
    std::vector<double> m(imax), n(jmax), mx(imax), my(jmax), sx(imax), sy(jmax), hh(2);
    int32_t pij[6];
    if ((rc = ns_dados_grid(&d, 1, m.data(), n.data(), mx.data(), my.data(), sx.data(), sy.data(),
                            hh.data(), pij)))
        return rc;
    for (int q = 0; q < 3; q++)
        if (pij[2 * q] < 1 || pij[2 * q] > imax || pij[2 * q + 1] < 1 || pij[2 * q + 1] > jmax)
            return fail(NS_ERR_PARAM, "ns_run_euler: probe point " + std::to_string(q + 1) +
                                          " lies outside the grid");
    if (!quiet) {
        // euler.f90:78-85, init.f90:71-72
        const double tr = d.Tref;
        char f[32];
        ns_format_real(tr, f, 32);
        std::printf(" Tref%s\n \n NAVIER STOKES MPI - Master process:\n"
                    "  FORTRAN90 serial version\n \n"
                    "  A program to solve the Non Linear Navier Stokes equations.\n \n", f);
        ns_format_real(hh[0], f, 32);
        std::printf(" dx=%s\n", f);
        ns_format_real(hh[1], f, 32);
        std::printf(" dy=%s\n", f);
    }
    ns_ctx *c = nullptr;
    if ((rc = ns_create_dados(&d, nk, device, 1, &c)) != NS_OK) return rc;
    const int32_t pi[3] = {pij[0], pij[2], pij[4]}, pj[3] = {pij[1], pij[3], pij[5]};
    const int cap = 512;
    std::FILE *pf[3] = {nullptr, nullptr, nullptr};
    std::vector<double> rec((size_t)cap * 3 * nk), tq;
    auto finish = [&](int code) {
        for (std::FILE *f : pf)
            if (f) std::fclose(f);
        ns_destroy(c);
        return code;
    };
    auto drain = [&]() -> int {
        int nrec = 0;
        int r = ns_probes_drain(c, rec.data(), &nrec);
        if (r != NS_OK) return r;
        for (int q = 0; q < nrec; q++)
            for (int k = 0; k < 3; k++) {
                // write(1000+k,*) t, U(1..4,px,py)  (euler.f90:153-155)
                double v[5];
                v[0] = tq[(size_t)q];
                for (int z = 0; z < 4; z++) v[z + 1] = rec[((size_t)q * 3 + k) * nk + z];
                write_record(pf[k], v, 5);
            }
        tq.clear();
        return NS_OK;
    };
    if ((rc = ns_probes_arm(c, 3, pi, pj, cap)) != NS_OK) return finish(rc);
    for (int k = 0; k < 3; k++) {
        const std::string path = join(outdir, "temp" + std::to_string(k + 1) + "_D60.dat");
        pf[k] = std::fopen(path.c_str(), "w");
        if (!pf[k]) return finish(fail(NS_ERR_PARAM, "cannot open " + path));
    }
    const int last = maxit >= 0 ? maxit : d.maxit;
    int cg = 0, ct = 0, icount = 0;
    // CPU_TIME in the reference; the work here runs on the GPU, so the
    // elapsed time is wall-clock
    const auto t0 = std::chrono::steady_clock::now();
    for (int iter = 0; iter <= last; iter++) {
        const double t = (iter + 1) * d.dt;  // euler.f90:126
        if ((rc = ns_step(c, iter, 1)) != NS_OK) return finish(rc);
        if (cg == d.cgd) {
            // euler.f90:133-149
            if (fields) {
                const std::string path = join(outdir, "contorno_" + std::to_string(icount) + ".dat");
                if ((rc = ns_write_contorno(c, path.c_str(), m.data(), n.data())) != NS_OK)
                    return finish(rc);
            }
            if (!quiet) {
                std::vector<double> u1(nk);
                if ((rc = ns_get_probes(c, 1, &pi[0], &pj[0], u1.data())) != NS_OK)
                    return finish(rc);
                const double v[3] = {t, u1[1], u1[3]};
                write_record(stdout, v, 3);
                const double secs =
                    std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                char f[32];
                ns_format_real(secs, f, 32);
                std::printf(" Tempo :%s segundos\n", f);
                std::fflush(stdout);
            }
            icount = icount + 1;
            cg = 0;
        }
        if (ct == d.ctd) {
            // euler.f90:152-157
            if ((int)tq.size() == cap && (rc = drain()) != NS_OK) return finish(rc);
            if ((rc = ns_probes_capture(c)) != NS_OK) return finish(rc);
            tq.push_back(t);
            ct = 0;
        }
        cg = cg + 1;
        ct = ct + 1;
    }
    if ((rc = drain()) != NS_OK) return finish(rc);
    if (!quiet) std::printf(" \n  Euler_MPI:\n  Normal end of execution.\n \n");
    return finish(NS_OK);
}

}  // extern "C"
