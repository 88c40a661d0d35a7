/*
 * ns_oracle.h -- CPU oracle for the LDDRK time-step hot path of
 * mathe1s/NavierStokes (rk.f90 and everything it calls).
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, FP64, line-by-line
 * restatement of the Fortran reference.  The CUDA path is checked against
 * it (tests/, __graft_entry__.smoke(), bench.py's CPU baseline); it is
 * never linked into, loaded by, or called from the product library.
 *
 * Parity status: the reference ships no tests, fixtures or golden vectors
 * and cannot be compiled here (no Fortran compiler; the sources also have
 * compile errors).  The restatement is pinned by known-answer tests derived
 * from the reference's own coefficient tables (stencil moments, filter
 * response, LDDRK order conditions, fixed points) -- "parity unpinned" by
 * reference-produced vectors.
 *
 * Array layout follows the reference exactly: U(nk,imax,jmax), Fortran
 * column-major, variable index fastest (euler.f90:107, rk.f90:17).
 */
#ifndef NS_ORACLE_H
#define NS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_params {
    int imax, jmax;      /* grid points (global.f90:13) */
    int nk;              /* variables carried: 5 = (rho,u,v,p,psi) as in the
                            reference (global.f90:19); 4 drops the passive psi */
    int D;               /* buffer width in points (dados.in &grid D) */
    int inviscid;        /* 1: Euler, 1/Re = 0 (viscous/heat terms vanish) */
    int metric_mode;     /* 0: reference metricsX/metricsY bands
                               (diff.f90:276-350); 1: the 1-D metric
                               multiplies every derivative (stretched grid) */
    double dt, dm, dn, sigmaf, gamma, Re, Pr, Tref;
    const double *meshx, *meshy;    /* [imax], [jmax] (init.f90:119-153) */
    const double *sigmax, *sigmay;  /* [imax], [jmax] (init.f90:158-206) */
    const double *Ub;               /* (nk,imax,jmax) base flow (init.f90:392-404) */
    const double *rhob, *psib;      /* [jmax] inflow profiles (cc.f90:23,27) */
    /* acoustic source (rk.f90:171-193): 0 none, 1 reference formula, 2 field */
    int source_mode;
    const double *m, *n;            /* coordinates [imax], [jmax] (mode 1) */
    double amplitude, wf, m_pt, n_pt, r0;
    const double *src_field;        /* [imax*jmax], i fastest (mode 2):
                                       s = sin(wf*(iter+c)*dt) * field */
} ora_params;

typedef struct ora_ctx ora_ctx;

/* Allocate the work arrays of the reference (global.f90 module state). */
ora_ctx *ora_create(const ora_params *p);
void ora_destroy(ora_ctx *c);
/* One call of rk_euler(U,t,iter,nk) (rk.f90:12-75), repeated nsteps times
 * with iter = iter0 .. iter0+nsteps-1.  U is updated in place. */
int ora_run(ora_ctx *c, double *U, int iter0, int nsteps);
/* Single pieces, for unit tests of the restatement. */
void ora_deropm(const ora_ctx *c, double *dU, const double *U, int nk);
void ora_deropn(const ora_ctx *c, double *dU, const double *U, int nk);
void ora_filterx(const ora_ctx *c, double *U, int nk);
void ora_filtery(const ora_ctx *c, double *U, int nk);
void ora_ccpml(const ora_ctx *c, double *U);
void ora_bufferxy(const ora_ctx *c, double *U);
/* One right-hand side evaluation (rhs.f90:10-46) with s_acou for (iter,ct). */
void ora_rhs(ora_ctx *c, double *dUdt, const double *U, int iter, double ct);
/* Transport law (coefficients.f90:71-123): writes mu0, k0 for Tref. */
void ora_transport_ref(double Tref, double *mu0, double *k0);
void ora_transport(double Tref, double T, double *mu, double *k);
/* Grid setup (init.f90:56-210) for a uniform grid in [mmin,mmax]x[nmin,nmax].
 * quirk_buffer=1 reproduces the unassigned imaxpml/jmaxpml (left and bottom
 * sigma stay 0, global.f90:86, init.f90:168,192). */
void ora_init_dados(int imax, int jmax, int D, double mmin, double mmax,
                    double nmin, double nmax, double c1b, double c2b,
                    int quirk_buffer, double *m, double *n, double *meshx,
                    double *meshy, double *sigmax, double *sigmay,
                    double *dm, double *dn);
/* Base-flow profiles of init_variables (init.f90:341-373): the tanh mixing
 * layer uba, Tb, rhob = 1/Tb and psib on rows n[jmax], gamma = 1.4,
 * deltamx = 0.4, psi1 = 1, psi2 = 0. */
void ora_mixing_layer(int jmax, const double *n, double U1, double U2,
                      double T1, double T2, double *uba, double *Tb,
                      double *rhob, double *psib);
/* Vorticity of the output path (outt.f90:43-49): the metric-free DRP
 * derivatives of diffall.f90:5-380 on the whole grid, omega =
 * dv/dx - du/dy, written omega[(i-1) + imax*(j-1)]. */
void ora_vorticity(int imax, int jmax, int nk, double dm, double dn,
                   const double *U, double *omega);
/* Coefficient tables of the reference, for known-answer tests.
 * which: 0 a_dudx(3), 1 a_dudx4, 2 a_dudx5, 3 a_dudx6, 4 a_dudx4b,
 * 5 a_dudx5b, 6 a_dudx6b (7 each), 7 df(-6:6) (13), 8 dfb x (-1:5),
 * 9 dfb y (-1:5, REAL(4)-rounded), 10 alphat(6), 11 betat(6), 12 ct(6). */
int ora_coeffs(int which, double *out);
void ora_set_threads(int n);
int ora_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
