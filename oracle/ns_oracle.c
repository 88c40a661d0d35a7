/*
 * ns_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY) for the LDDRK
 * time-step hot path of mathe1s/NavierStokes.
 *
 * A plain-C FP64 restatement of the Fortran, statement by statement, in the
 * reference's array layout U(nk,imax,jmax) (column-major, variable fastest).
 * Every function cites the reference file:line it follows.  Only the loop
 * nesting of independent outputs is reordered for cache locality and OpenMP;
 * the arithmetic of every element (operand order, per-term divisions, the
 * in-place filter recurrences, the REAL(4) y-boundary filter coefficients)
 * is the reference's.  Build with -ffp-contract=off so no FMA is formed.
 *
 * Used only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
 * Parity unpinned by reference-produced vectors (the reference has no tests
 * and cannot be built here); pinned by the known-answer tests in tests/.
 */
#include "ns_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------------- */
/* Coefficient tables                                                       */
/* ---------------------------------------------------------------------- */

/* DRP first-derivative coefficients, init.f90:288-338 (index 1-based). */
static const double a_dudx[4] = {0.0, 0.770882380518, -0.166705904415,
                                 0.0208431427703};
static const double a_dudx4[8] = {0.0, 0.049041958000, -0.46884035700,
                                  -0.47476091400, 1.27327473700,
                                  -0.51848452600, 0.16613853300,
                                  -0.026369431000};
static const double a_dudx4b[8] = {0.0, 0.026369431000, -0.16613853300,
                                   0.51848452600, -1.27327473700,
                                   0.47476091400, 0.46884035700,
                                   -0.049041958000};
static const double a_dudx5[8] = {0.0, -0.20933762200, -1.08487567600,
                                  2.14777605000, -1.38892832200,
                                  0.76894976600, -0.28181465000,
                                  0.048230454000};
static const double a_dudx5b[8] = {0.0, -0.048230454000, 0.28181465000,
                                   -0.76894976600, 1.38892832200,
                                   -2.14777605000, 1.08487567600,
                                   0.20933762200};
static const double a_dudx6[8] = {0.0, -2.19228033900, 4.74861140100,
                                  -5.10885191500, 4.46156710400,
                                  -2.83349874100, 1.12832886100,
                                  -0.20387637100};
static const double a_dudx6b[8] = {0.0, 0.20387637100, -1.12832886100,
                                   2.83349874100, -4.46156710400,
                                   5.10885191500, -4.74861140100,
                                   2.19228033900};

/* 13-point selective filter, filtering.f90:54-66 (index s+6). */
static const double df13[13] = {
    0.001254597714, -0.008520738659, 0.029662754736, -0.069975429105,
    0.123632891797, -0.171503832236, 0.190899511506, -0.171503832236,
    0.123632891797, -0.069975429105, 0.029662754736, -0.008520738659,
    0.001254597714};
/* 7-point boundary filter dfb(-1:5) in x, REAL(8) literals (filtering.f90:25-31). */
static const double dfbx[7] = {-0.057717512738, 0.199278374994,
                               -0.292668277650, 0.244537361546,
                               -0.134605018019, 0.056184263460,
                               -0.015009191593};
/* Same coefficients in y, but written as default-REAL literals
 * (filtering.f90:114-120): each is rounded to REAL(4) then widened. */
static const double dfby[7] = {(double)-0.057717512738f,
                               (double)0.199278374994f,
                               (double)-0.292668277650f,
                               (double)0.244537361546f,
                               (double)-0.134605018019f,
                               (double)0.056184263460f,
                               (double)-0.015009191593f};

/* LDDRK 6-stage coefficients (rk.f90:27-46). */
static const double alphat[6] = {0.0, -0.737101392796, -1.634740794341,
                                 -0.744739003780, -1.469897351522,
                                 -2.813971388035};
static const double betat[6] = {0.032918605146, 0.823256998200,
                                0.381530948900, 0.200092213184,
                                1.718581042715, 0.27};
static const double ctk[6] = {0.0, 0.032918605146, 0.249351723343,
                              0.466911705055, 0.582030414044,
                              0.847252983783};

/* Svehla N2 fit (coefficients.f90:113-123, SPECIE_N). */
static const double A_MI = 0.62526577, B_MI = -31.779652, C_MI = -1640.7913,
                    D_MI = 1.7454992;
static const double A_K = 0.85372829, B_K = 105.18665, C_K = -12229.753,
                    D_K = 0.48299104;
/* global.f90:38-39 */
static const double Pe = 1000.0, alpha_cond = 0.5;

/* ---------------------------------------------------------------------- */
/* Context                                                                  */
/* ---------------------------------------------------------------------- */

struct ora_ctx {
    ora_params p;
    double MI0, K0;
    /* module work arrays (global.f90, allocated in init.f90:224-416) */
    double *dUdm, *dUdn, *dudt, *w;                 /* (nk,imax,jmax) */
    double *TEMP, *MI, *K1;                         /* (imax,jmax) */
    double *DTEMPDM, *DTEMPDN, *D2TEMPDM, *D2TEMPDN; /* (1,imax,jmax) */
    double *psiDiff, *D2psiFDM, *D2psiFDN;          /* (1,imax,jmax) */
    double *TAU, *DTAUDM, *DTAUDN;                  /* (3,imax,jmax) */
    double *s_acou;                                 /* (imax,jmax) */
};

#define IMAX (c->p.imax)
#define JMAX (c->p.jmax)
/* 1-based access into an (nn,imax,jmax) array */
#define A3(a, nn, k, i, j) \
    (a)[((size_t)(k)-1) + (size_t)(nn) * (((size_t)(i)-1) + (size_t)IMAX * ((size_t)(j)-1))]
#define A2(a, i, j) (a)[((size_t)(i)-1) + (size_t)IMAX * ((size_t)(j)-1)]

void ora_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int ora_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int ora_coeffs(int which, double *out)
{
    int i;
    switch (which) {
    case 0: for (i = 0; i < 3; i++) out[i] = a_dudx[i + 1]; return 3;
    case 1: for (i = 0; i < 7; i++) out[i] = a_dudx4[i + 1]; return 7;
    case 2: for (i = 0; i < 7; i++) out[i] = a_dudx5[i + 1]; return 7;
    case 3: for (i = 0; i < 7; i++) out[i] = a_dudx6[i + 1]; return 7;
    case 4: for (i = 0; i < 7; i++) out[i] = a_dudx4b[i + 1]; return 7;
    case 5: for (i = 0; i < 7; i++) out[i] = a_dudx5b[i + 1]; return 7;
    case 6: for (i = 0; i < 7; i++) out[i] = a_dudx6b[i + 1]; return 7;
    case 7: for (i = 0; i < 13; i++) out[i] = df13[i]; return 13;
    case 8: for (i = 0; i < 7; i++) out[i] = dfbx[i]; return 7;
    case 9: for (i = 0; i < 7; i++) out[i] = dfby[i]; return 7;
    case 10: for (i = 0; i < 6; i++) out[i] = alphat[i]; return 6;
    case 11: for (i = 0; i < 6; i++) out[i] = betat[i]; return 6;
    case 12: for (i = 0; i < 6; i++) out[i] = ctk[i]; return 6;
    default: return 0;
    }
}

/* GET_COEFFICIENTS, coefficients.f90:71-80 */
void ora_transport_ref(double Tref, double *mu0, double *k0)
{
    *k0 = exp(A_K * log(1.0 * Tref) + B_K / Tref + C_K / Tref / Tref + D_K);
    *mu0 = exp(A_MI * log(1.0 * Tref) + B_MI / Tref + C_MI / Tref / Tref + D_MI);
}

/* MOLECULAR_MI and k_coefficient at one point, coefficients.f90:27-59 */
void ora_transport(double Tref, double T, double *mu, double *k)
{
    double MI0, K0;
    ora_transport_ref(Tref, &MI0, &K0);
    *mu = 1.0 / MI0 * (exp(A_MI * log(Tref * T) + B_MI / Tref / T +
                           C_MI / Tref / T / Tref / T + D_MI));
    *k = 1.0 / K0 * (exp(A_K * log(Tref * T) + B_K / Tref / T +
                         C_K / Tref / Tref / T / T + D_K));
}

ora_ctx *ora_create(const ora_params *p)
{
    ora_ctx *c;
    size_t np, nk;
    if (!p || p->imax < 13 || p->jmax < 13 || (p->nk != 4 && p->nk != 5))
        return NULL;
    c = (ora_ctx *)calloc(1, sizeof(*c));
    if (!c) return NULL;
    c->p = *p;
    np = (size_t)p->imax * p->jmax;
    nk = (size_t)p->nk;
    c->dUdm = calloc(nk * np, 8);
    c->dUdn = calloc(nk * np, 8);
    c->dudt = calloc(nk * np, 8);
    c->w = calloc(nk * np, 8);
    c->TEMP = calloc(np, 8);
    c->MI = calloc(np, 8);
    c->K1 = calloc(np, 8);
    c->DTEMPDM = calloc(np, 8);
    c->DTEMPDN = calloc(np, 8);
    c->D2TEMPDM = calloc(np, 8);
    c->D2TEMPDN = calloc(np, 8);
    c->psiDiff = calloc(np, 8);
    c->D2psiFDM = calloc(np, 8);
    c->D2psiFDN = calloc(np, 8);
    c->TAU = calloc(3 * np, 8);
    c->DTAUDM = calloc(3 * np, 8);
    c->DTAUDN = calloc(3 * np, 8);
    c->s_acou = calloc(np, 8);
    if (!c->dUdm || !c->dUdn || !c->dudt || !c->w || !c->TEMP || !c->MI ||
        !c->K1 || !c->DTEMPDM || !c->DTEMPDN || !c->D2TEMPDM ||
        !c->D2TEMPDN || !c->psiDiff || !c->D2psiFDM || !c->D2psiFDN ||
        !c->TAU || !c->DTAUDM || !c->DTAUDN || !c->s_acou) {
        ora_destroy(c);
        return NULL;
    }
    ora_transport_ref(p->Tref, &c->MI0, &c->K0);
    return c;
}

void ora_destroy(ora_ctx *c)
{
    if (!c) return;
    free(c->dUdm); free(c->dUdn); free(c->dudt); free(c->w);
    free(c->TEMP); free(c->MI); free(c->K1);
    free(c->DTEMPDM); free(c->DTEMPDN); free(c->D2TEMPDM); free(c->D2TEMPDN);
    free(c->psiDiff); free(c->D2psiFDM); free(c->D2psiFDN);
    free(c->TAU); free(c->DTAUDM); free(c->DTAUDN); free(c->s_acou);
    free(c);
}

/* ---------------------------------------------------------------------- */
/* DRP derivatives (diff.f90)                                               */
/* ---------------------------------------------------------------------- */

/* metricsX, diff.f90:315-350: the six band tests, applied in order (a point
 * in two bands is multiplied twice, as in the reference). */
static double metric_x(const ora_ctx *c, int i, int j, double du)
{
    const int D = c->p.D, imax = IMAX, jmax = JMAX;
    const double mx = c->p.meshx[i - 1];
    if (c->p.metric_mode == 1) return du * mx;
    if ((i >= 1) && (i <= D) && (j >= D + 1) && (j <= jmax - D)) du = du * mx;
    if ((i >= imax - D + 1) && (i <= imax) && (j >= D + 1) && (j <= jmax - D)) du = du * mx;
    if ((i >= 1) && (i <= D) && (j >= jmax - D + 1) && (j <= jmax)) du = du * mx;
    if ((i >= 1) && (i <= D) && (j >= 1) && (j <= D)) du = du * mx;
    if ((i >= imax - D + 1) && (i <= imax) && (j >= 1) && (j <= D)) du = du * mx;
    if ((i >= imax - D + 1) && (i <= imax) && (j >= jmax - D + 1) && (j <= jmax)) du = du * mx;
    return du;
}

/* metricsY, diff.f90:276-311 */
static double metric_y(const ora_ctx *c, int i, int j, double du)
{
    const int D = c->p.D, imax = IMAX, jmax = JMAX;
    const double my = c->p.meshy[j - 1];
    if (c->p.metric_mode == 1) return du * my;
    if ((i >= D + 1) && (i <= imax - D) && (j >= 1) && (j <= D)) du = du * my;
    if ((i >= D + 1) && (i <= imax - D) && (j >= jmax - D + 1) && (j <= jmax)) du = du * my;
    if ((i >= 1) && (i <= D) && (j >= jmax - D + 1) && (j <= jmax)) du = du * my;
    if ((i >= 1) && (i <= D) && (j >= 1) && (j <= D)) du = du * my;
    if ((i >= imax - D + 1) && (i <= imax) && (j >= 1) && (j <= D)) du = du * my;
    if ((i >= imax - D + 1) && (i <= imax) && (j >= jmax - D + 1) && (j <= jmax)) du = du * my;
    return du;
}

/* One x-derivative value at (k,i,j): deropm's dispatch (diff.f90:18-35) to
 * dx6 (:101), dx5 (:75), dx4 (:49), dudx (:40), dx4I (:62), dx5I (:88),
 * dx6I (:114).  Each term is divided by dm separately, summed left to right. */
static double dx_point(const ora_ctx *c, const double *u, int nn, int k, int i, int j)
{
    const double dm = c->p.dm;
    const int imax = IMAX;
#define UX(ii) A3(u, nn, k, (ii), j)
    if (i == 1)
        return (a_dudx6[1] * UX(i + 1 - 1)) / dm + (a_dudx6[2] * UX(i + 2 - 1)) / dm +
               (a_dudx6[3] * UX(i + 3 - 1)) / dm + (a_dudx6[4] * UX(i + 4 - 1)) / dm +
               (a_dudx6[5] * UX(i + 5 - 1)) / dm + (a_dudx6[6] * UX(i + 6 - 1)) / dm +
               (a_dudx6[7] * UX(i + 7 - 1)) / dm;
    if (i == 2)
        return (a_dudx5[1] * UX(i + 1 - 2)) / dm + (a_dudx5[2] * UX(i + 2 - 2)) / dm +
               (a_dudx5[3] * UX(i + 3 - 2)) / dm + (a_dudx5[4] * UX(i + 4 - 2)) / dm +
               (a_dudx5[5] * UX(i + 5 - 2)) / dm + (a_dudx5[6] * UX(i + 6 - 2)) / dm +
               (a_dudx5[7] * UX(i + 7 - 2)) / dm;
    if (i == 3)
        return (a_dudx4[1] * UX(i + 1 - 3)) / dm + (a_dudx4[2] * UX(i + 2 - 3)) / dm +
               (a_dudx4[3] * UX(i + 3 - 3)) / dm + (a_dudx4[4] * UX(i + 4 - 3)) / dm +
               (a_dudx4[5] * UX(i + 5 - 3)) / dm + (a_dudx4[6] * UX(i + 6 - 3)) / dm +
               (a_dudx4[7] * UX(i + 7 - 3)) / dm;
    if (i == imax - 2)
        return (a_dudx4b[7] * UX(i + 7 - 5)) / dm + (a_dudx4b[6] * UX(i + 6 - 5)) / dm +
               (a_dudx4b[5] * UX(i + 5 - 5)) / dm + (a_dudx4b[4] * UX(i + 4 - 5)) / dm +
               (a_dudx4b[3] * UX(i + 3 - 5)) / dm + (a_dudx4b[2] * UX(i + 2 - 5)) / dm +
               (a_dudx4b[1] * UX(i + 1 - 5)) / dm;
    if (i == imax - 1)
        return (a_dudx5b[7] * UX(i + 7 - 6)) / dm + (a_dudx5b[6] * UX(i + 6 - 6)) / dm +
               (a_dudx5b[5] * UX(i + 5 - 6)) / dm + (a_dudx5b[4] * UX(i + 4 - 6)) / dm +
               (a_dudx5b[3] * UX(i + 3 - 6)) / dm + (a_dudx5b[2] * UX(i + 2 - 6)) / dm +
               (a_dudx5b[1] * UX(i + 1 - 6)) / dm;
    if (i == imax)
        return (a_dudx6b[7] * UX(i + 7 - 7)) / dm + (a_dudx6b[6] * UX(i + 6 - 7)) / dm +
               (a_dudx6b[5] * UX(i + 5 - 7)) / dm + (a_dudx6b[4] * UX(i + 4 - 7)) / dm +
               (a_dudx6b[3] * UX(i + 3 - 7)) / dm + (a_dudx6b[2] * UX(i + 2 - 7)) / dm +
               (a_dudx6b[1] * UX(i + 1 - 7)) / dm;
    return (a_dudx[1] * (UX(i + 1) - UX(i - 1))) / dm +
           (a_dudx[2] * (UX(i + 2) - UX(i - 2))) / dm +
           (a_dudx[3] * (UX(i + 3) - UX(i - 3))) / dm;
#undef UX
}

/* One y-derivative value: deropn (diff.f90:127-151) -> dy6 (:214), dy5
 * (:188), dy4 (:162), dudy (:153), dy4I (:175), dy5I (:201), dy6I (:227).
 * The dy* closures are written a*u/dn, i.e. (a*u)/dn. */
static double dy_point(const ora_ctx *c, const double *u, int nn, int k, int i, int j)
{
    const double dn = c->p.dn;
    const int jmax = JMAX;
#define UY(jj) A3(u, nn, k, i, (jj))
    if (j == 1)
        return a_dudx6[1] * UY(j + 1 - 1) / dn + a_dudx6[2] * UY(j + 2 - 1) / dn +
               a_dudx6[3] * UY(j + 3 - 1) / dn + a_dudx6[4] * UY(j + 4 - 1) / dn +
               a_dudx6[5] * UY(j + 5 - 1) / dn + a_dudx6[6] * UY(j + 6 - 1) / dn +
               a_dudx6[7] * UY(j + 7 - 1) / dn;
    if (j == 2)
        return a_dudx5[1] * UY(j + 1 - 2) / dn + a_dudx5[2] * UY(j + 2 - 2) / dn +
               a_dudx5[3] * UY(j + 3 - 2) / dn + a_dudx5[4] * UY(j + 4 - 2) / dn +
               a_dudx5[5] * UY(j + 5 - 2) / dn + a_dudx5[6] * UY(j + 6 - 2) / dn +
               a_dudx5[7] * UY(j + 7 - 2) / dn;
    if (j == 3)
        return a_dudx4[1] * UY(j + 1 - 3) / dn + a_dudx4[2] * UY(j + 2 - 3) / dn +
               a_dudx4[3] * UY(j + 3 - 3) / dn + a_dudx4[4] * UY(j + 4 - 3) / dn +
               a_dudx4[5] * UY(j + 5 - 3) / dn + a_dudx4[6] * UY(j + 6 - 3) / dn +
               a_dudx4[7] * UY(j + 7 - 3) / dn;
    if (j == jmax - 2)
        return a_dudx4b[7] * UY(j + 7 - 5) / dn + a_dudx4b[6] * UY(j + 6 - 5) / dn +
               a_dudx4b[5] * UY(j + 5 - 5) / dn + a_dudx4b[4] * UY(j + 4 - 5) / dn +
               a_dudx4b[3] * UY(j + 3 - 5) / dn + a_dudx4b[2] * UY(j + 2 - 5) / dn +
               a_dudx4b[1] * UY(j + 1 - 5) / dn;
    if (j == jmax - 1)
        return a_dudx5b[7] * UY(j + 7 - 6) / dn + a_dudx5b[6] * UY(j + 6 - 6) / dn +
               a_dudx5b[5] * UY(j + 5 - 6) / dn + a_dudx5b[4] * UY(j + 4 - 6) / dn +
               a_dudx5b[3] * UY(j + 3 - 6) / dn + a_dudx5b[2] * UY(j + 2 - 6) / dn +
               a_dudx5b[1] * UY(j + 1 - 6) / dn;
    if (j == jmax)
        return a_dudx6b[7] * UY(j + 7 - 7) / dn + a_dudx6b[6] * UY(j + 6 - 7) / dn +
               a_dudx6b[5] * UY(j + 5 - 7) / dn + a_dudx6b[4] * UY(j + 4 - 7) / dn +
               a_dudx6b[3] * UY(j + 3 - 7) / dn + a_dudx6b[2] * UY(j + 2 - 7) / dn +
               a_dudx6b[1] * UY(j + 1 - 7) / dn;
    return (a_dudx[1] * (UY(j + 1) - UY(j - 1))) / dn +
           (a_dudx[2] * (UY(j + 2) - UY(j - 2))) / dn +
           (a_dudx[3] * (UY(j + 3) - UY(j - 3))) / dn;
#undef UY
}

/* deropm + metricsX (diff.f90:6-38, 315-350) on an (nn,imax,jmax) array. */
void ora_deropm(const ora_ctx *c, double *dU, const double *U, int nn)
{
    int j;
#pragma omp parallel for schedule(static)
    for (j = 1; j <= JMAX; j++) {
        int i, k;
        for (i = 1; i <= IMAX; i++)
            for (k = 1; k <= nn; k++)
                A3(dU, nn, k, i, j) = metric_x(c, i, j, dx_point(c, U, nn, k, i, j));
    }
}

/* deropn + metricsY (diff.f90:127-151, 276-311). */
void ora_deropn(const ora_ctx *c, double *dU, const double *U, int nn)
{
    int j;
#pragma omp parallel for schedule(static)
    for (j = 1; j <= JMAX; j++) {
        int i, k;
        for (i = 1; i <= IMAX; i++)
            for (k = 1; k <= nn; k++)
                A3(dU, nn, k, i, j) = metric_y(c, i, j, dy_point(c, U, nn, k, i, j));
    }
}

/* ---------------------------------------------------------------------- */
/* Right-hand side (rhs.f90, derivs.f90, eqeuler.f90, coefficients.f90)     */
/* ---------------------------------------------------------------------- */

/* acousticfont, rk.f90:171-193 */
static void acousticfont(ora_ctx *c, double ct, int iter)
{
    const ora_params *p = &c->p;
    int j;
    if (p->source_mode == 1) {
#pragma omp parallel for schedule(static)
        for (j = 1; j <= JMAX; j++) {
            int i;
            for (i = 1; i <= IMAX; i++) {
                double dx = p->m[i - 1] - p->m_pt, dy = p->n[j - 1] - p->n_pt;
                A2(c->s_acou, i, j) =
                    p->amplitude * sin(p->wf * ((iter + ct) * p->dt)) *
                    exp(-(log(2.0) * (dx * dx + dy * dy) / (p->r0 * p->r0)));
            }
        }
    } else if (p->source_mode == 2) {
        const double sv = sin(p->wf * ((iter + ct) * p->dt));
#pragma omp parallel for schedule(static)
        for (j = 1; j <= JMAX; j++) {
            int i;
            for (i = 1; i <= IMAX; i++)
                A2(c->s_acou, i, j) = sv * p->src_field[(size_t)(i - 1) + (size_t)IMAX * (j - 1)];
        }
    }
}

/* rhs_euler, rhs.f90:10-46, with deriv/kdT (derivs.f90:9-56), TAU_IJ and
 * EULERNONLINEAR (eqeuler.f90:28-99).  s_acou must already be set. */
static void rhs_euler(ora_ctx *c, double *dUdt, const double *U)
{
    const ora_params *p = &c->p;
    const int nk = p->nk, visc = !p->inviscid;
    const double gamma = p->gamma, Tref = p->Tref;
    const double MI0 = c->MI0, K0 = c->K0;
    int j;

    if (visc) {
        /* TEMP = gamma*p/rho (rhs.f90:20); MOLECULAR_MI, K_COEFFICIENT
         * (coefficients.f90:27-59) */
#pragma omp parallel for schedule(static)
        for (j = 1; j <= JMAX; j++) {
            int i;
            for (i = 1; i <= IMAX; i++) {
                double T = (gamma) * (A3(U, nk, 4, i, j)) / (A3(U, nk, 1, i, j));
                A2(c->TEMP, i, j) = T;
                A2(c->MI, i, j) = 1.0 / MI0 * (exp(A_MI * log(Tref * T) + B_MI / Tref / T +
                                                   C_MI / Tref / T / Tref / T + D_MI));
                A2(c->K1, i, j) = 1.0 / K0 * (exp(A_K * log(Tref * T) + B_K / Tref / T +
                                                  C_K / Tref / Tref / T / T + D_K));
            }
        }
    }

    /* deriv (derivs.f90:9-45) */
    ora_deropm(c, c->dUdm, U, nk);
    ora_deropn(c, c->dUdn, U, nk);
    if (visc) {
        ora_deropm(c, c->DTEMPDM, c->TEMP, 1);
        ora_deropn(c, c->DTEMPDN, c->TEMP, 1);
        /* kdT, derivs.f90:48-56 */
#pragma omp parallel for schedule(static)
        for (j = 1; j <= JMAX; j++) {
            int i;
            for (i = 1; i <= IMAX; i++) {
                A2(c->DTEMPDN, i, j) = A2(c->DTEMPDN, i, j) * A2(c->K1, i, j);
                A2(c->DTEMPDM, i, j) = A2(c->DTEMPDM, i, j) * A2(c->K1, i, j);
            }
        }
        ora_deropm(c, c->D2TEMPDM, c->DTEMPDM, 1);
        ora_deropn(c, c->D2TEMPDN, c->DTEMPDN, 1);
    }
    if (nk >= 5) {
        /* psiDiff = rho*alpha_cond*(dpsi/dx + dpsi/dy), derivs.f90:35-39 */
#pragma omp parallel for schedule(static)
        for (j = 1; j <= JMAX; j++) {
            int i;
            for (i = 1; i <= IMAX; i++)
                A2(c->psiDiff, i, j) = A3(U, nk, 1, i, j) * alpha_cond *
                                       (A3(c->dUdm, nk, 5, i, j) + A3(c->dUdn, nk, 5, i, j));
        }
        ora_deropm(c, c->D2psiFDM, c->psiDiff, 1);
        ora_deropn(c, c->D2psiFDN, c->psiDiff, 1);
    }

    if (visc) {
        /* TAU_IJ, eqeuler.f90:28-47 */
#pragma omp parallel for schedule(static)
        for (j = 1; j <= JMAX; j++) {
            int i;
            for (i = 1; i <= IMAX; i++) {
                const double mi = A2(c->MI, i, j);
                const double dm2 = A3(c->dUdm, nk, 2, i, j), dn3 = A3(c->dUdn, nk, 3, i, j);
                const double dn2 = A3(c->dUdn, nk, 2, i, j), dm3 = A3(c->dUdm, nk, 3, i, j);
                A3(c->TAU, 3, 1, i, j) = -(2.0 / 3.0 * (mi) * (dm2 + dn3)) + 2.0 * (mi) * (dm2);
                A3(c->TAU, 3, 2, i, j) = (mi) * (dn2 + dm3);
                A3(c->TAU, 3, 3, i, j) = -(2.0 / 3.0 * (mi) * (dm2 + dn3)) + 2.0 * (mi) * (dn3);
            }
        }
        ora_deropm(c, c->DTAUDM, c->TAU, 3);
        ora_deropn(c, c->DTAUDN, c->TAU, 3);
    }

    /* EULERNONLINEAR, eqeuler.f90:53-99 */
    {
        const double Re = p->Re, Pr = p->Pr;
#pragma omp parallel for schedule(static)
        for (j = 1; j <= JMAX; j++) {
            int i;
            for (i = 1; i <= IMAX; i++) {
                const double U1 = A3(U, nk, 1, i, j), U2 = A3(U, nk, 2, i, j);
                const double U3 = A3(U, nk, 3, i, j), U4 = A3(U, nk, 4, i, j);
                const double *dm = &A3(c->dUdm, nk, 1, i, j);
                const double *dn = &A3(c->dUdn, nk, 1, i, j);
                const double s = p->source_mode ? A2(c->s_acou, i, j) : 0.0;
                double r2, r3, r4;
                A3(dUdt, nk, 1, i, j) = -(U2 * (dm[0]) + U1 * (dm[1]) + U3 * (dn[0]) + U1 * (dn[2]));
                if (visc) {
                    const double *tm = &A3(c->DTAUDM, 3, 1, i, j);
                    const double *tn = &A3(c->DTAUDN, 3, 1, i, j);
                    const double *ta = &A3(c->TAU, 3, 1, i, j);
                    r2 = -(U2 * (dm[1]) + 1.0 / U1 * dm[3] + U3 * (dn[1]) -
                           1.0 / Re / (U1) * (tm[0] + tn[1]));
                    r3 = -(U2 * (dm[2]) + U3 * (dn[2]) + 1.0 / U1 * (dn[3]) -
                           1.0 / Re / (U1) * (tm[1] + tn[2]));
                    r4 = -(gamma * U4 * (dm[1]) + U2 * (dm[3]) + gamma * U4 * (dn[2]) +
                           U3 * (dn[3]) - s -
                           (gamma - 1.0) / Re * (+(dm[1]) * ta[0] + (dm[2]) * ta[1] +
                                                 (dn[1]) * ta[1] + (dn[2]) * ta[2]) -
                           1.0 / Re / Pr * (A2(c->D2TEMPDM, i, j) + A2(c->D2TEMPDN, i, j)));
                } else {
                    /* 1/Re = 0: the viscous, dissipation and heat-flux terms
                     * are exactly zero and are not formed. */
                    r2 = -(U2 * (dm[1]) + 1.0 / U1 * dm[3] + U3 * (dn[1]));
                    r3 = -(U2 * (dm[2]) + U3 * (dn[2]) + 1.0 / U1 * (dn[3]));
                    r4 = -(gamma * U4 * (dm[1]) + U2 * (dm[3]) + gamma * U4 * (dn[2]) +
                           U3 * (dn[3]) - s);
                }
                A3(dUdt, nk, 2, i, j) = r2;
                A3(dUdt, nk, 3, i, j) = r3;
                A3(dUdt, nk, 4, i, j) = r4;
                if (nk >= 5)
                    A3(dUdt, nk, 5, i, j) =
                        -(U2 * dm[4] + U3 * dn[4] -
                          1.0 / Pe / U1 * (A2(c->D2psiFDM, i, j) + A2(c->D2psiFDN, i, j)));
            }
        }
    }
}

void ora_rhs(ora_ctx *c, double *dUdt, const double *U, int iter, double ct)
{
    if (c->p.source_mode) acousticfont(c, ct, iter);
    rhs_euler(c, dUdt, U);
}

/* ---------------------------------------------------------------------- */
/* Stage update, buffer, filters, boundary conditions                       */
/* ---------------------------------------------------------------------- */

/* rk_steep, rk.f90:153-169 (interior points only) */
static void rk_steep(ora_ctx *c, double alpha, double beta, double *U)
{
    const int nk = c->p.nk;
    const double dt = c->p.dt;
    int j;
#pragma omp parallel for schedule(static)
    for (j = 2; j <= JMAX - 1; j++) {
        int i, k;
        for (i = 2; i <= IMAX - 1; i++)
            for (k = 1; k <= nk; k++) {
                A3(c->w, nk, k, i, j) = alpha * A3(c->w, nk, k, i, j) + dt * A3(c->dudt, nk, k, i, j);
                A3(U, nk, k, i, j) = A3(U, nk, k, i, j) + beta * A3(c->w, nk, k, i, j);
            }
    }
}

/* bufferxy / bufferx / buffery, rk.f90:77-151 */
void ora_bufferxy(const ora_ctx *c, double *U)
{
    const int nk = c->p.nk, D = c->p.D, imax = IMAX, jmax = JMAX;
    const double *Ub = c->p.Ub;
    int j;
#pragma omp parallel for schedule(static)
    for (j = 1; j <= jmax; j++) {
        int i, k;
        for (i = 1; i <= imax; i++) {
            const double sy = c->p.sigmay[j - 1], sx = c->p.sigmax[i - 1];
            if ((i >= 1) && (i <= imax)) {
                if ((j >= 1) && (j <= D))
                    for (k = 1; k <= nk; k++)
                        A3(U, nk, k, i, j) = A3(Ub, nk, k, i, j) + sy * (A3(U, nk, k, i, j) - A3(Ub, nk, k, i, j));
                if ((j >= jmax - D + 1) && (j <= jmax))
                    for (k = 1; k <= nk; k++)
                        A3(U, nk, k, i, j) = A3(Ub, nk, k, i, j) + sy * (A3(U, nk, k, i, j) - A3(Ub, nk, k, i, j));
            }
            if ((j >= 1) && (j <= jmax)) {
                if ((i >= 1) && (i <= D))
                    for (k = 1; k <= nk; k++)
                        A3(U, nk, k, i, j) = A3(Ub, nk, k, i, j) + sx * (A3(U, nk, k, i, j) - A3(Ub, nk, k, i, j));
                if ((i >= imax - D + 1) && (i <= imax))
                    for (k = 1; k <= nk; k++)
                        A3(U, nk, k, i, j) = A3(Ub, nk, k, i, j) + sx * (A3(U, nk, k, i, j) - A3(Ub, nk, k, i, j));
            }
        }
    }
}

/* lddfilterx, filtering.f90:9-96: three in-place sweeps along i of every
 * line (k,j): ascending boundary pass i=2..7, ascending interior pass
 * i=7..imax-6, descending boundary pass i=imax-1..imax-6. */
void ora_filterx(const ora_ctx *c, double *U, int nk)
{
    const int imax = IMAX, jmax = JMAX;
    const double sigmaf = c->p.sigmaf;
    int j;
#pragma omp parallel for schedule(static)
    for (j = 1; j <= jmax; j++) {
        int k, i, s;
        double Du;
        for (k = 1; k <= nk; k++) {
            for (i = 2; i <= 7; i++) {
                Du = 0.0;
                for (s = -1; s <= 5; s++) Du = Du + dfbx[s + 1] * A3(U, nk, k, i + s, j);
                A3(U, nk, k, i, j) = A3(U, nk, k, i, j) - sigmaf * Du;
            }
            for (i = 7; i <= imax - 6; i++) {
                Du = 0.0;
                for (s = -6; s <= 6; s++) Du = Du + df13[s + 6] * A3(U, nk, k, i + s, j);
                A3(U, nk, k, i, j) = A3(U, nk, k, i, j) - sigmaf * Du;
            }
            for (i = imax - 1; i >= imax - 6; i--) {
                Du = 0.0;
                for (s = -1; s <= 5; s++) Du = Du + dfbx[s + 1] * A3(U, nk, k, i - s, j);
                A3(U, nk, k, i, j) = A3(U, nk, k, i, j) - sigmaf * Du;
            }
        }
    }
}

/* lddfiltery, filtering.f90:98-190: the same sweeps along j of every line
 * (k,i), with the REAL(4)-rounded boundary coefficients.  Lines are
 * processed in blocks of i for locality; each line's recurrence is the
 * reference's. */
void ora_filtery(const ora_ctx *c, double *U, int nk)
{
    const int imax = IMAX, jmax = JMAX;
    const double sigmaf = c->p.sigmaf;
    const int IB = 64;
    int ib;
#pragma omp parallel for schedule(static)
    for (ib = 1; ib <= imax; ib += IB) {
        const int ie = (ib + IB - 1 < imax) ? ib + IB - 1 : imax;
        int k, i, j, s;
        double Du;
        for (k = 1; k <= nk; k++) {
            for (j = 2; j <= 7; j++)
                for (i = ib; i <= ie; i++) {
                    Du = 0.0;
                    for (s = -1; s <= 5; s++) Du = Du + dfby[s + 1] * A3(U, nk, k, i, j + s);
                    A3(U, nk, k, i, j) = A3(U, nk, k, i, j) - sigmaf * Du;
                }
            for (j = 7; j <= jmax - 6; j++)
                for (i = ib; i <= ie; i++) {
                    Du = 0.0;
                    for (s = -6; s <= 6; s++) Du = Du + df13[s + 6] * A3(U, nk, k, i, j + s);
                    A3(U, nk, k, i, j) = A3(U, nk, k, i, j) - sigmaf * Du;
                }
            for (j = jmax - 1; j >= jmax - 6; j--)
                for (i = ib; i <= ie; i++) {
                    Du = 0.0;
                    for (s = -1; s <= 5; s++) Du = Du + dfby[s + 1] * A3(U, nk, k, i, j - s);
                    A3(U, nk, k, i, j) = A3(U, nk, k, i, j) - sigmaf * Du;
                }
        }
    }
}

/* ccpml, cc.f90:6-68: left, right, top, bottom, in that order. */
void ora_ccpml(const ora_ctx *c, double *U)
{
    const int nk = c->p.nk, imax = IMAX, jmax = JMAX;
    const double gamma = c->p.gamma;
    int i, j;
    for (j = 1; j <= jmax; j++) {          /* inflow, cc.f90:23-27 */
        A3(U, nk, 1, 1, j) = c->p.rhob[j - 1];
        A3(U, nk, 2, 1, j) = 2.0 * A3(U, nk, 2, 2, j) - A3(U, nk, 2, 3, j);
        A3(U, nk, 3, 1, j) = 0.0;
        A3(U, nk, 4, 1, j) = 1.0 / gamma;
        if (nk >= 5) A3(U, nk, 5, 1, j) = c->p.psib[j - 1];
    }
    for (j = 1; j <= jmax; j++) {          /* outflow, cc.f90:32-36 */
        A3(U, nk, 1, imax, j) = 2.0 * A3(U, nk, 1, imax - 1, j) - A3(U, nk, 1, imax - 2, j);
        A3(U, nk, 2, imax, j) = 2.0 * A3(U, nk, 2, imax - 1, j) - A3(U, nk, 2, imax - 2, j);
        A3(U, nk, 3, imax, j) = 2.0 * A3(U, nk, 3, imax - 1, j) - A3(U, nk, 3, imax - 2, j);
        A3(U, nk, 4, imax, j) = 1.0 / gamma;
        if (nk >= 5) A3(U, nk, 5, imax, j) = 2.0 * A3(U, nk, 5, imax - 1, j) - A3(U, nk, 5, imax - 2, j);
    }
    for (i = 1; i <= imax; i++) {          /* upper, cc.f90:39-43 */
        A3(U, nk, 1, i, jmax) = 2.0 * A3(U, nk, 1, i, jmax - 1) - A3(U, nk, 1, i, jmax - 2);
        A3(U, nk, 2, i, jmax) = 2.0 * A3(U, nk, 2, i, jmax - 1) - A3(U, nk, 2, i, jmax - 2);
        A3(U, nk, 3, i, jmax) = 2.0 * A3(U, nk, 3, i, jmax - 1) - A3(U, nk, 3, i, jmax - 2);
        A3(U, nk, 4, i, jmax) = 1.0 / gamma;
        if (nk >= 5) A3(U, nk, 5, i, jmax) = 1.0;
    }
    for (i = 1; i <= imax; i++) {          /* lower, cc.f90:55-59 */
        A3(U, nk, 1, i, 1) = 2.0 * A3(U, nk, 1, i, 1 + 1) - A3(U, nk, 1, i, 1 + 2);
        A3(U, nk, 2, i, 1) = 2.0 * A3(U, nk, 2, i, 1 + 1) - A3(U, nk, 2, i, 1 + 2);
        A3(U, nk, 3, i, 1) = 2.0 * A3(U, nk, 3, i, 1 + 1) - A3(U, nk, 3, i, 1 + 2);
        A3(U, nk, 4, i, 1) = 1.0 / gamma;
        if (nk >= 5) A3(U, nk, 5, i, 1) = 0.0;
    }
}

/* rk_euler, rk.f90:12-75 */
int ora_run(ora_ctx *c, double *U, int iter0, int nsteps)
{
    const size_t n = (size_t)c->p.nk * IMAX * JMAX;
    int step, irk;
    for (step = 0; step < nsteps; step++) {
        const int iter = iter0 + step;
        memset(c->w, 0, n * sizeof(double));            /* rk.f90:21 */
        for (irk = 0; irk < 6; irk++) {                 /* rk.f90:52 */
            if (c->p.source_mode) acousticfont(c, ctk[irk], iter);
            rhs_euler(c, c->dudt, U);
            rk_steep(c, alphat[irk], betat[irk], U);
            ora_bufferxy(c, U);
            ora_filterx(c, U, c->p.nk);
            ora_filtery(c, U, c->p.nk);
            ora_ccpml(c, U);
        }
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* Grid setup, init.f90:56-210                                              */
/* ---------------------------------------------------------------------- */

void ora_init_dados(int imax, int jmax, int D, double mmin, double mmax,
                    double nmin, double nmax, double c1b, double c2b,
                    int quirk_buffer, double *m, double *n, double *meshx,
                    double *meshy, double *sigmax, double *sigmay,
                    double *dm_out, double *dn_out)
{
    /* imaxpml/jmaxpml are never assigned (global.f90:86); quirk_buffer=1
     * takes them as 0, otherwise as D. */
    const int imaxpml = quirk_buffer ? 0 : D, jmaxpml = quirk_buffer ? 0 : D;
    const double Aa = 2.0, alpham = 2.0;
    double dm, dn, Dx, Dy, xli, xld, yli, yls, x, y, xs, xe, ys, ye;
    int i, j;
    /* real(imax-1) is a default REAL (single precision) conversion of an
     * exactly representable integer, so the quotient is the double one. */
    dm = (mmax - mmin) / (double)(float)(imax - 1);
    dn = (nmax - nmin) / (double)(float)(jmax - 1);
    Dx = dm * D;
    Dy = dn * D;
    xli = mmin + Dx;
    xld = mmax - Dx;
    yli = nmin + Dy;
    yls = nmax - Dy;
    for (i = 1; i <= imax; i++) m[i - 1] = mmin + (double)(float)(i - 1) * dm;
    for (j = 1; j <= jmax; j++) n[j - 1] = nmin + (double)(float)(j - 1) * dn;
    for (i = 1; i <= imax; i++) {
        meshx[i - 1] = 1.0;
        if ((i >= 1) && (i <= D + 1))
            meshx[i - 1] = 1.0 / (1.0 + Aa * pow(fabs((m[i - 1] - (xli)) / (Dx)), alpham));
        if ((i >= imax - D) && (i <= imax))
            meshx[i - 1] = 1.0 / (1.0 + Aa * pow(fabs((m[i - 1] - xld) / (Dx)), alpham));
    }
    for (j = 1; j <= jmax; j++) {
        meshy[j - 1] = 1.0;
        if ((j >= 1) && (j <= D + 1))
            meshy[j - 1] = 1.0 / (1.0 + Aa * pow(fabs((n[j - 1] - (yli)) / (Dy)), alpham));
        if ((j >= jmax - D + 1) && (j <= jmax))
            meshy[j - 1] = 1.0 / (1.0 + Aa * pow(fabs((n[j - 1] - (yls)) / (Dy)), alpham));
    }
    for (i = 1; i <= imax; i++) {
        sigmax[i - 1] = 0.0;
        if ((i >= 1) && (i <= imaxpml)) {
            xs = xli; xe = mmin;
            x = (m[i - 1] - xs) / (xe - xs);
            sigmax[i - 1] = (1.0 - c1b * x * x) * (1.0 - (1.0 - exp(c2b * x * x)) / (1.0 - exp(c2b)));
        }
        if ((i >= imax - D + 1) && (i <= imax)) {
            xs = xld; xe = mmax;
            x = (m[i - 1] - xs) / (xe - xs);
            sigmax[i - 1] = (1.0 - c1b * x * x) * (1.0 - (1.0 - exp(c2b * x * x)) / (1.0 - exp(c2b)));
        }
    }
    for (j = 1; j <= jmax; j++) {
        sigmay[j - 1] = 0.0;
        if ((j >= 1) && (j <= jmaxpml)) {
            ys = yli; ye = nmin;
            y = (n[j - 1] - ys) / (ye - ys);
            sigmay[j - 1] = (1.0 - c1b * y * y) * (1.0 - (1.0 - exp(c2b * y * y)) / (1.0 - exp(c2b)));
        }
        if ((j >= jmax - D + 1) && (j <= jmax)) {
            ys = yls; ye = nmax;
            y = (n[j - 1] - ys) / (ye - ys);
            sigmay[j - 1] = (1.0 - c1b * y * y) * (1.0 - (1.0 - exp(c2b * y * y)) / (1.0 - exp(c2b)));
        }
    }
    *dm_out = dm;
    *dn_out = dn;
}

/* init_variables profiles, init.f90:359-373 (gamma = 1.4 at :361,
 * deltamx = 0.4 at :358, psi1 = 1 and psi2 = 0 at :362-363). */
void ora_mixing_layer(int jmax, const double *n, double U1, double U2,
                      double T1, double T2, double *uba, double *Tb,
                      double *rhob, double *psib)
{
    const double u1b = U1, u2b = U2, deltamx = 0.4, gamma = 1.4;
    const double psi1 = 1.0, psi2 = 0.0;
    int j;
    for (j = 1; j <= jmax; j++) {
        uba[j - 1] = 0.5 * (u1b + u2b + (u1b - u2b) * tanh(2.0 * n[j - 1] / deltamx));
        Tb[j - 1] = T1 * (uba[j - 1] - u2b) / (u1b - u2b) + T2 * (u1b - uba[j - 1]) / (u1b - u2b) +
                    (gamma - 1.0) / 2.0 * (u1b - uba[j - 1]) * (uba[j - 1] - u2b);
        rhob[j - 1] = 1.0 / (Tb[j - 1]);
        psib[j - 1] = 0.5 * (psi1 + psi2 + (psi1 - psi2) * tanh(2.0 * n[j - 1] / deltamx));
    }
}

/* 1-based access into an (nn,imx,*) array with an explicit row length */
#define A3x(a, nn, imx, k, i, j) \
    (a)[((size_t)(k)-1) + (size_t)(nn) * (((size_t)(i)-1) + (size_t)(imx) * ((size_t)(j)-1))]

/* diffall.f90 derivatives of variable k at (i,j): deropm (:5-43) dispatches
 * to dudx (:45-64), dx4 (:66-106), dx5 (:108-150), dx6 (:152-193) with
 * p = -1 at the right end (coefficients mirrored, summed from z = 7 down).
 * Each term is (a*u)/h, summed left to right; no metric. */
static double dall_point(const double *u, int nn, int k, int imax, int jmax, int i, int j,
                         int along_y, double h)
{
    const int nq = along_y ? jmax : imax, q = along_y ? j : i;
    const double *c;
    int o0, z;
    double r = 0.0;
#define UQ(qq) (along_y ? A3x(u, nn, imax, k, i, (qq)) : A3x(u, nn, imax, k, (qq), j))
    if (q >= 4 && q <= nq - 3) {
        for (z = 1; z <= 3; z++) r = r + (a_dudx[z] * (UQ(q + z) - UQ(q - z))) / h;
        return r;
    }
    if (q <= 3) {
        /* dx6 (q=1, offsets 0..6), dx5 (q=2, -1..5), dx4 (q=3, -2..4) */
        c = (q == 1) ? a_dudx6 : (q == 2) ? a_dudx5 : a_dudx4;
        o0 = 1 - q;
        for (z = 1; z <= 7; z++) r = r + c[z] * UQ(q + o0 + z - 1) / h;
        return r;
    }
    /* right end: z = 7 down to 1 with the mirrored a(z) = a_dudx*b(z) */
    c = (q == nq) ? a_dudx6b : (q == nq - 1) ? a_dudx5b : a_dudx4b;
    o0 = (q == nq) ? -7 : (q == nq - 1) ? -6 : -5;
    for (z = 7; z >= 1; z--) r = r + c[z] * UQ(q + z + o0) / h;
    return r;
#undef UQ
}

void ora_vorticity(int imax, int jmax, int nk, double dm, double dn,
                   const double *U, double *omega)
{
    int j;
#pragma omp parallel for schedule(static)
    for (j = 1; j <= jmax; j++) {
        int i;
        for (i = 1; i <= imax; i++) {
            const double dvdx = dall_point(U, nk, 3, imax, jmax, i, j, 0, dm);
            const double dudy = dall_point(U, nk, 2, imax, jmax, i, j, 1, dn);
            omega[(size_t)(i - 1) + (size_t)imax * (j - 1)] = dvdx - dudy;
        }
    }
}
