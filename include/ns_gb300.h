/*
 * ns_gb300.h -- C ABI of the GB300 (sm_103a) time-step library for the
 * mathe1s/NavierStokes aeroacoustic solver.
 *
 * The library replaces the reference's LDDRK stage loop, rk_euler
 * (rk.f90:12-75), and everything it calls: the DRP derivatives with their
 * boundary closures and 1-D metrics (diff.f90, derivs.f90), the transport
 * law (coefficients.f90), the primitive Navier-Stokes right-hand side
 * (rhs.f90, eqeuler.f90), the stage update and buffer damping (rk.f90), the
 * in-place 13-point selective filter (filtering.f90) and the boundary
 * conditions (cc.f90).  The inputs the reference reads from module `global`
 * (global.f90) are passed once in ns_params; the state U stays resident on
 * the GPU between calls.
 *
 * Conventions: plain C types only; every entry point returns an ns_status
 * (0 = NS_OK) and never aborts the process; ns_last_error() gives the text
 * of the last failure on a context.  One context per host thread; calls on
 * one context are not re-entrant.
 */
#ifndef NS_GB300_H
#define NS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NS_ABI_VERSION 1

#if defined(__GNUC__)
#define NS_API __attribute__((visibility("default")))
#else
#define NS_API
#endif

typedef enum ns_status {
    NS_OK = 0,
    NS_ERR_PARAM = 1,       /* invalid argument or unsupported size */
    NS_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    NS_ERR_OOM = 3,         /* device or host allocation failed */
    NS_ERR_NONFINITE = 4,   /* the state holds NaN/Inf (ns_check_finite) */
    NS_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    NS_ERR_STATE = 6,       /* call out of order (e.g. step before set_state) */
    NS_ERR_UNSUPPORTED = 7, /* feature not available for these parameters */
    NS_ERR_CHECK = 8        /* checked build only: a device index check failed */
} ns_status;

/* Host array layouts accepted by ns_set_state/ns_get_state. */
enum {
    NS_LAYOUT_FORTRAN = 0, /* U(nk,imax,jmax), column-major: the reference's
                              own array (euler.f90:107) */
    NS_LAYOUT_SOA = 1,     /* U[k][j][i], i fastest: one plane per variable */
    NS_LAYOUT_ROWS = 2     /* a field constant along i, given by rows:
                              nk*jmax values, k fastest, (k,j) -> U(k,:,j);
                              expanded on the device (Ub of init.f90:387-396
                              and the initial U = Ub of :376-384) */
};

/* Arithmetic of the stage loop. */
enum {
    NS_PREC_FP64 = 0,  /* plain FP64, the reference's arithmetic */
    NS_PREC_SPLIT = 1, /* FP64 mean flow + FP32 perturbation arithmetic;
                          u', v', p' stored as FP32 hi + lo pairs, rho' as
                          one FP32; Euler (inviscid = 1), nk = 4, base flow
                          Ub uniform in x with v = 0 and uniform p */
    NS_PREC_SPLIT32 = 2 /* the same with every perturbation one FP32 number
                          (fewer bytes; the FP32 storage noise of u' drives
                          p' near a strong vortex); the batched path's split
                          mode */
};

/* Acoustic source of rk.f90:171-193. */
enum {
    NS_SRC_NONE = 0,
    NS_SRC_GAUSSIAN = 1, /* s = amplitude*sin(wf*(iter+c)*dt)
                                *exp(-ln2*((m-m_pt)^2+(n-n_pt)^2)/r0^2) */
    NS_SRC_FIELD = 2     /* s = sin(wf*(iter+c)*dt) * src_field(i,j) */
};

/* Metric application of diff.f90:276-350. */
enum {
    NS_METRIC_BANDS = 0,   /* reference: meshx/meshy multiply derivatives only
                              inside the D-wide buffer bands */
    NS_METRIC_EVERYWHERE = 1 /* meshx(i)/meshy(j) multiply every derivative
                                (stretched-grid cases) */
};

/*
 * Everything rk_euler reads from module `global` (global.f90) and from the
 * setup routines init_dados/init_variables (init.f90:56-418).  The library
 * copies what it needs during ns_create; the caller may free the arrays
 * afterwards.
 */
typedef struct ns_params {
    int32_t abi_version;   /* = NS_ABI_VERSION */
    int32_t imax, jmax;    /* grid points, >= 13 each (global.f90:13) */
    int32_t nk;            /* 5 = (rho,u,v,p,psi) as the reference
                              (global.f90:19); 4 = without the passive psi */
    int32_t D;             /* buffer width, 0 <= 2*D <= min(imax,jmax) */
    int32_t inviscid;      /* 1: Euler (1/Re = 0); 0: Navier-Stokes */
    int32_t metric_mode;   /* NS_METRIC_* */
    int32_t precision;     /* NS_PREC_* */
    int32_t source_mode;   /* NS_SRC_* */
    int32_t device;        /* CUDA device ordinal */
    int32_t ub_layout;     /* layout of Ub: NS_LAYOUT_* */
    int32_t reserved0;
    double dt, dm, dn;     /* time step, grid steps (init.f90:68-70) */
    double sigmaf;         /* filter strength (dados.in &grid sigmaf) */
    double gamma;          /* ratio of specific heats (init.f90:361) */
    double Re, Pr;         /* Reynolds, Prandtl numbers (&flow) */
    double Tref;           /* reference temperature (&flow) */
    /* Transport fit exp(A*ln(x)+B/x+C/x^2+D), x = Tref*T, for mu and k
     * (coefficients.f90:27-59; N2 values in SPECIE_N, :113-123). */
    double A_mi, B_mi, C_mi, D_mi;
    double A_k, B_k, C_k, D_k;
    /* source parameters (&freq), used by NS_SRC_GAUSSIAN / NS_SRC_FIELD */
    double amplitude, wf, m_pt, n_pt, r0;
    const double *m;       /* [imax] x coordinates (init.f90:104-107) */
    const double *n;       /* [jmax] y coordinates (init.f90:113-115) */
    const double *meshx;   /* [imax] x metric (init.f90:123-137) */
    const double *meshy;   /* [jmax] y metric (init.f90:139-153) */
    const double *sigmax;  /* [imax] buffer damping (init.f90:158-181) */
    const double *sigmay;  /* [jmax] buffer damping (init.f90:183-206) */
    const double *rhob;    /* [jmax] inflow density (cc.f90:23) */
    const double *psib;    /* [jmax] inflow scalar (cc.f90:27), nk = 5 */
    const double *Ub;      /* base flow, nk*imax*jmax in ub_layout
                              (init.f90:392-404) */
    const double *src_field; /* [imax*jmax], i fastest (NS_SRC_FIELD) */
} ns_params;

typedef struct ns_ctx ns_ctx;

/* Library/ABI identification. */
NS_API int ns_abi_version(void);
NS_API const char *ns_build_info(void);

/* Fills the defaults the reference fixes in code: gamma = 1.4
 * (init.f90:361), the N2 transport fit (coefficients.f90:113-123),
 * Tref = 273.15, nk = 5, metric bands, FP64.  Sizes and arrays are zeroed. */
NS_API int ns_params_init(ns_params *p);

/* Validates p, allocates the device state and work arrays and uploads the
 * setup arrays.  Replaces the module state that init_read/init_dados/
 * init_variables leave for rk_euler (init.f90:10-418). */
NS_API int ns_create(const ns_params *p, ns_ctx **out);
NS_API void ns_destroy(ns_ctx *ctx);
NS_API const char *ns_last_error(const ns_ctx *ctx);  /* ctx may be NULL */

/* Host <-> device state transfer (synchronous).  U holds nk*imax*jmax
 * doubles in `layout`. */
NS_API int ns_set_state(ns_ctx *ctx, const double *U, int layout);
NS_API int ns_get_state(ns_ctx *ctx, double *U, int layout);

/* Advances the resident state by nsteps calls of rk_euler (rk.f90:12) with
 * iter = iter0, iter0+1, ...: six LDDRK stages each.  Asynchronous with
 * respect to the host (ordered on the context's stream); launch errors are
 * returned at once, execution errors by the next synchronising call. */
NS_API int ns_step(ns_ctx *ctx, int iter0, int nsteps);
NS_API int ns_synchronize(ns_ctx *ctx);

/* The drop-in for one call `call rk_euler(U,t,iter,nk)` (euler.f90:130,
 * rk.f90:12): host U in the reference layout U(nk,imax,jmax) is uploaded,
 * advanced one step and written back.  t is unused, as in the reference.
 * When U is page-locked host memory, FP64 contexts copy it in row bands and
 * start the step on the bands already copied; split contexts read and write
 * it in place from the GPU.  Returns when U holds the new state. */
NS_API int ns_rk_euler(ns_ctx *ctx, double *U, double t, int iter, int nk);

/* Page-locks (and releases) an existing host array, e.g. the Fortran U, so
 * that ns_rk_euler takes the page-locked path on it (cudaHostRegister on
 * the current device's context; `bytes` from the start of the array). */
NS_API int ns_pin_host(void *p, size_t bytes);
NS_API int ns_unpin_host(void *p);

/* Reads U(1..nk) at np points (1-based i, j) into out[np*nk] (point-major):
 * the probe writes of euler.f90:156-161 without a full download. */
NS_API int ns_get_probes(ns_ctx *ctx, int np, const int32_t *pi, const int32_t *pj,
                  double *out);

/* Scans the state for NaN/Inf; sets *nonfinite to the count found and
 * returns NS_ERR_NONFINITE when it is non-zero. */
NS_API int ns_check_finite(ns_ctx *ctx, int64_t *nonfinite);

/* Stream the context enqueues on (a cudaStream_t, 0 = the context's own). */
NS_API int ns_set_stream(ns_ctx *ctx, void *stream);
NS_API int ns_get_stream(ns_ctx *ctx, void **stream);

/* Device pointer of the resident SoA state: plane k of variable k+1 starts
 * at *dptr + k*jmax*pitch, row j at + j*pitch (pitch in elements).  For
 * zero-copy views from PyTorch; valid until ns_destroy. */
NS_API int ns_state_device(ns_ctx *ctx, void **dptr, int64_t *pitch);

/* Number of kernel launches one ns_step(…,1) enqueues, and the filter
 * warm-up length used for the chunked recurrences. */
NS_API int ns_step_launches(ns_ctx *ctx, int *launches);
NS_API int ns_filter_warmup(ns_ctx *ctx, int *warmup);

/* Kernel classes of the step, for ns_time_kernels. */
enum {
    NS_KC_STAGE_SIN = 0, /* per-step source phase sin(wf*(iter+c_k)*dt) */
    NS_KC_PRIM = 1,      /* T = gamma*p/rho, 1/rho                 (rhs.f90:20) */
    NS_KC_FIRST = 2,     /* first derivatives, mu, k, tau, k*grad T (diff.f90,
                            derivs.f90, coefficients.f90, eqeuler.f90:28-47) */
    NS_KC_UPDATE = 3,    /* second derivatives, RHS, LDDRK update, buffer
                            (eqeuler.f90:53-99, rk.f90:77-169) */
    NS_KC_FILTER_X = 4,  /* lddfilterx                 (filtering.f90:9-96) */
    NS_KC_FILTER_Y = 5,  /* lddfiltery                 (filtering.f90:98-190) */
    NS_KC_BC = 6,        /* ccpml                      (cc.f90:6-68) */
    NS_KC_SPLIT_STAGE = 7, /* split precision: fused FP32 derivatives, RHS,
                              FP64 LDDRK update, buffer (rk.f90:52-64) */
    NS_KC_SPLIT_FX = 8,  /* split precision: lddfilterx on the FP32 perturbation */
    NS_KC_SPLIT_FY = 9,  /* split precision: lddfiltery on the FP32 perturbation */
    NS_KC_SPLIT_BC = 10, /* split precision: ccpml on the perturbation */
    NS_KC_SPLIT_VISC = 11, /* split precision, Navier-Stokes: tau' and k grad T'
                              of the perturbation (eqeuler.f90:28-47,
                              derivs.f90:48-56) */
    NS_KC_COUNT = 12
};

/* Advances the state by `reps` steps from iter0, launching every kernel on
 * its own (no graph) between CUDA events on the context stream, and writes
 * per kernel class the mean device time of one launch in ms_per_launch[c]
 * and the launches per step in launches[c] (arrays of NS_KC_COUNT). */
NS_API int ns_time_kernels(ns_ctx *ctx, int iter0, int reps, double *ms_per_launch,
                           int *launches);
NS_API const char *ns_kernel_name(int kernel_class);

/* Library diagnostic, no counterpart in the reference: measured FP64 FMA
 * throughput of `device` in TFLOP/s (2 flops per DFMA), the bound of the
 * FP64 stage kernels on GB300. */
NS_API int ns_fp64_peak(int device, double *tflops);

/* Library diagnostic, no counterpart in the reference: the exp (fn = 0),
 * log (fn = 1) and 1/x (fn = 2) the stage kernels use for the transport law
 * mu(T), k(T) (coefficients.f90:27-59), evaluated on device `device` for
 * x[0..n) into y[0..n) (host arrays). */
NS_API int ns_math_eval(int fn, const double *x, double *y, int n, int device);

/* Library diagnostic, no counterpart in the reference: mu(T) and k(T) of the
 * transport law (coefficients.f90:27-59, divided by mu0 and k0) exactly as
 * the context's first-derivative kernel evaluates them (its piecewise
 * polynomial table, or exp and log outside the table's range), for
 * T[0..n) into mu[0..n), k[0..n) (host arrays).  NS_ERR_STATE for an
 * inviscid context. */
NS_API int ns_transport_eval(ns_ctx *ctx, const double *T, double *mu, double *k, int n);

/* Library diagnostic, no counterpart in the reference: runs one block whose
 * mbarrier expects bytes that no copy delivers, with the bounded wait of the
 * TMA tile loads limited to spin_limit polls (1 .. 2^16).  Returns
 * NS_ERR_TIMEOUT when the wait ran out and reported it, as the stage
 * kernels do (their limit is 2^24 polls). */
NS_API int ns_tma_wait_test(int device, long long spin_limit);

/* Library diagnostics of the checked build, no counterpart in the reference.
 * The checked build (libns_gb300_checked.so, compiled with -DNS_CHECKED)
 * range-checks every tile, halo, segment and work-list index its kernels
 * derive; a failed check is recorded instead of the access and the next
 * synchronising call returns NS_ERR_CHECK with the file and line in
 * ns_last_error.  ns_checked_build() is 1 in that build and 0 otherwise;
 * ns_check_selftest runs one warp in which half the lanes fail a check that
 * guards no access: NS_ERR_CHECK in the checked build, NS_OK otherwise. */
NS_API int ns_checked_build(void);
NS_API int ns_check_selftest(int device);

/* Library diagnostic, host only: the piecewise-polynomial table of mu(T),
 * k(T) that ns_create builds for a viscous context (Tref, fits {A,B,C,D} of
 * mu and k).  Writes NS_TRANSPORT_TABLE_DOUBLES doubles: piece (e, j) for
 * T = 2^e (1 + (j + f)/256), e = -2 .. 2, at (e + 2)*256 + j, holding six
 * coefficients of mu then six of k in powers of u = T - 2^e (1 + j/256). */
#define NS_TRANSPORT_TABLE_DOUBLES (5 * 256 * 12)

/* Library diagnostic, host only: the launch shape of an FP64 filter sweep
 * over nlines lines (per variable, nk variables) of n points with a warm-up
 * of `warm` points on a device of nsm multiprocessors: every warp takes
 * *seg consecutive pass-2 positions of the warp-lines (32 lines of one
 * variable) laid end to end; *blocks blocks of 128 threads. */
NS_API int ns_filter_plan(int nlines, int n, int nk, int warm, int nsm, int64_t *seg,
                          int *blocks);
NS_API int ns_transport_table(double Tref, const double *fit_mu, const double *fit_k,
                              double *out);

/* Library diagnostic, host only: the coefficient tables every setup path of
 * the library uses, numbered as the oracle numbers them: 0 the interior DRP
 * weights a(1..3), 1..3 the left closures at points 3, 2, 1 (a_dudx4, 5, 6),
 * 4..6 the right closures (a_dudx4b, 5b, 6b) (init.f90:288-338); 7 the
 * 13-point filter df(-6..6) (filtering.f90:54-66); 8 and 9 the boundary
 * filter dfb(-1..5) in x (REAL(8), filtering.f90:25-31) and y (REAL(4),
 * filtering.f90:114-120); 10..12 LDDRK alpha, beta and c_k (rk.f90:27-46).
 * Writes the table to out (room for 16 doubles) and returns its length,
 * or 0 for an unknown number. */
NS_API int ns_coef_table(int which, double *out);

/*
 * Batched sweeps: many independent Euler instances (inviscid = 1, nk = 4,
 * base flow uniform in x with v = 0 and uniform p; each with its own size,
 * metric, buffer, time step and source) advanced together, one cooperative
 * persistent kernel per step (captured in a CUDA graph) whose phases run over
 * a work list spanning every instance.  Each instance follows rk_euler
 * (rk.f90:12-75) exactly as ns_step does; precision NS_PREC_FP64 or
 * NS_PREC_SPLIT.  All instances share one sigmaf and one device.
 */
typedef struct ns_batch ns_batch;
NS_API int ns_batch_create(const ns_params *const *params, int n, int precision, ns_batch **out);
NS_API void ns_batch_destroy(ns_batch *b);
NS_API int ns_batch_set_state(ns_batch *b, int instance, const double *U, int layout);
NS_API int ns_batch_get_state(ns_batch *b, int instance, double *U, int layout);
NS_API int ns_batch_step(ns_batch *b, int iter0, int nsteps);
/* Waits for the batch's work; NS_ERR_TIMEOUT if a phase barrier gave up. */
NS_API int ns_batch_synchronize(ns_batch *b);
NS_API int ns_batch_set_stream(ns_batch *b, void *stream);
/* Tile autotuner: times every tile height (8, 16 rows) and residency for
 * `reps` steps on the current state (advancing it), keeps the fastest. */
NS_API int ns_batch_autotune(ns_batch *b, int iter0, int reps, int *tile_rows,
                             int *blocks_per_sm, double *ms_per_step);
/* Current launch shape: grid blocks, tile rows, blocks per SM, and the work
 * items per phase items[4] = {tiles, x lines, y lines, instances}. */
NS_API int ns_batch_info(ns_batch *b, int *grid, int *tile_rows, int *blocks_per_sm,
                         int *items);
/* Failure-detection hook: one step whose barriers wait for `extra` blocks
 * that do not exist, each wait bounded by spin_limit spins; returns
 * NS_ERR_TIMEOUT and leaves the batch and its state usable. */
NS_API int ns_batch_barrier_test(ns_batch *b, int extra, long long spin_limit);
/* Library diagnostic: runs one step (advancing the state, without the graph)
 * in which block 0 reads the global timer after every phase barrier;
 * ms[0..3] = the time of phases A (tiles), B (x lines), C (y lines) and
 * D (edges), each summed over the six stages, barrier waits included. */
NS_API int ns_batch_phase_times(ns_batch *b, int iter0, double *ms);

/*
 * Discrete adjoint of the FP64 Euler step (inviscid = 1, nk = 4, source
 * NS_SRC_FIELD, uniform p_b): the gradient of
 *   L = sum over steps n = 1..N of sum over observers m of p'(x_m, y_m, t_n)^2,
 * p' = p - p_b interpolated bilinearly, with respect to the source field
 * S(i,j) of rk.f90:188-189 (s = sin(wf*(iter+c_k)*dt) * S).  The reverse pass
 * transposes ccpml, both filter sweeps, bufferxy, rk_steep, the pointwise
 * Jacobians of EULERNONLINEAR and the DRP stencils with their closures.
 * checkpoint_every >= 1: the forward state is checkpointed every
 * checkpoint_every steps and the reverse pass recomputes each segment.
 * checkpoint_every = 0: every stage's input state is kept (nsteps x 6 x 4
 * planes) when that fits in three quarters of the free device memory, and
 * the reverse pass recomputes only each stage's first derivatives;
 * otherwise checkpoints every 100 steps.
 */
typedef struct ns_adjoint ns_adjoint;
NS_API int ns_adjoint_create(const ns_params *p, int nobs, const double *obs_x,
                             const double *obs_y, int checkpoint_every, ns_adjoint **out);
NS_API void ns_adjoint_destroy(ns_adjoint *a);
/* Replaces S (imax*jmax doubles, i fastest). */
NS_API int ns_adjoint_set_source(ns_adjoint *a, const double *field);
/* Forward pass from host U0 (layout NS_LAYOUT_*), nsteps steps from iter0;
 * writes the loss. */
NS_API int ns_adjoint_forward(ns_adjoint *a, const double *U0, int layout, int iter0,
                              int nsteps, double *loss);
/* Reverse pass of the last forward pass: grad_field = dL/dS (imax*jmax). */
NS_API int ns_adjoint_backward(ns_adjoint *a, double *grad_field);
/* The forward context (for its state and diagnostics). */
NS_API int ns_adjoint_context(ns_adjoint *a, ns_ctx **ctx);
/* Bytes of stage inputs the last forward pass kept (0: it checkpointed). */
NS_API int ns_adjoint_stored_bytes(const ns_adjoint *a, int64_t *bytes);

/*
 * The program around the step: euler.f90's time loop with its probes and
 * field dumps, the dados.in reader and the grid/base-flow setup of init.f90.
 * None of these is on the reference's rk.f90 boundary; they replace
 * euler.f90:36-206, init.f90:10-52 (init_read), :56-210 (init_dados) and
 * :341-404 (init_variables), and outt.f90:17-55 (output).
 */

/* The dados.in namelists (dados.in:1-85) as init_read reads them
 * (init.f90:18-23): &grid (imax..ctd), &freq, &freeadm, &flow, a second
 * &grid (D, c1b, c2b, c3b: the namelist statement at init.f90:22 extends
 * group grid), &mpi.  Names the file does not set stay 0. */
typedef struct ns_dados {
    int32_t imax, jmax, maxit, cgd, cfd, ctd;  /* &grid */
    int32_t D;                                 /* &grid (second group) */
    int32_t iterw;                             /* &freq */
    int32_t num_procs_x, num_procs_y;          /* &mpi */
    double dt, sigmaf;                         /* &grid */
    double r0_acous, amplitude, m_pt_acous, n_pt_acous, wfi, wff, wf;  /* &freq */
    double pxfft[5];                           /* &freq pxfft1..pxfft5 */
    double mmin, mmax, nmin, nmax;             /* &freeadm */
    double pxr[3], pyr[3];                     /* &freeadm pxr1..3, pyr1..3 */
    double U1, U2, Re, Pr, T1, T2, Tref;       /* &flow */
    double c1b, c2b, c3b;                      /* &grid (second group) */
} ns_dados;

/* init_read (init.f90:10-52): reads the six groups in order, each found by
 * scanning forward from the end of the previous one.  Accepts '!' comments,
 * ',' or blanks between items, REAL(8) constants with d/D/e/E exponents and
 * the terminators '/', '&end' and '$end' (dados.in:85).  A name outside the
 * group, a malformed value, a missing group or a missing terminator is
 * NS_ERR_PARAM with the line in ns_last_error(NULL).  ns_parse_dados takes
 * the file's text. */
NS_API int ns_read_dados(const char *path, ns_dados *out);
NS_API int ns_parse_dados(const char *text, ns_dados *out);

/* init_dados (init.f90:56-210): coordinates m[imax], n[jmax], buffer
 * metrics meshx, meshy, damping sigmax, sigmay (quirk_buffer = 1: the left
 * and bottom sigma stay 0 as in the reference, whose imaxpml/jmaxpml are
 * never set), dm_dn[2] = {dm, dn} and the 1-based probe points
 * probe_ij[6] = {px1, py1, px2, py2, px3, py3} (init.f90:80-85). */
NS_API int ns_dados_grid(const ns_dados *d, int quirk_buffer, double *m, double *n,
                         double *meshx, double *meshy, double *sigmax, double *sigmay,
                         double *dm_dn, int32_t *probe_ij);

/* Base-flow rows of init_variables (init.f90:359-373): the tanh mixing
 * layer uba, Tb, rhob = 1/Tb and psib on the rows n[jmax]. */
NS_API int ns_dados_profiles(const ns_dados *d, const double *n, double *uba, double *Tb,
                             double *rhob, double *psib);

/* A context for the dados.in case: Navier-Stokes with Re, Pr, Tref, nk = 4
 * or 5 variables, the Gaussian source of rk.f90:171-193, band metrics; Ub
 * is built on the device from its rows and the state starts at U = Ub
 * (init.f90:376-404), so no full-size host array is made. */
NS_API int ns_create_dados(const ns_dados *d, int nk, int device, int quirk_buffer,
                           ns_ctx **out);

/* Vorticity of the output path (outt.f90:43-49): diffall.f90's DRP
 * derivatives, which apply no metric, on the device: omega = dv/dx - du/dy
 * at every point, copied to omega[imax*jmax] (host, i fastest). */
NS_API int ns_vorticity(ns_ctx *ctx, double *omega);

/* One contorno_<icount>.dat file (outt.f90:40-55): per point the
 * list-directed record m(i), n(j), rho, u, v, p, omega, psi (psi only when
 * nk = 5), j fastest, an empty record after each i.  m, n: host coordinate
 * arrays [imax], [jmax]. */
NS_API int ns_write_contorno(ns_ctx *ctx, const char *path, const double *m, const double *n);

/* One REAL(8) item as list-directed output writes it (G25.17 with a three-
 * digit exponent: F20.(16-e) and five blanks for 0.1 <= |x| < 1e17, else
 * E25.17E3 with one digit before the point); buf gets the 25 characters
 * and a NUL.  Returns the field width, or -1 if len < 26. */
NS_API int ns_format_real(double x, char *buf, int len);

/* Probe recorder for the time loop: ns_probes_arm sets npts points
 * (1-based pi, pj) and room for `capacity` records; each ns_probes_capture
 * enqueues a copy of U(1..nk) at every point as the next record (no host
 * synchronisation); ns_probes_drain copies the records taken so far,
 * out[rec][point][k], sets *nrec and empties the recorder.  Capturing into
 * a full recorder is NS_ERR_STATE. */
NS_API int ns_probes_arm(ns_ctx *ctx, int npts, const int32_t *pi, const int32_t *pj,
                         int capacity);
NS_API int ns_probes_capture(ns_ctx *ctx);
NS_API int ns_probes_drain(ns_ctx *ctx, double *out, int *nrec);

/* The euler.f90 program (euler.f90:36-206) on the GPU: reads dados_path,
 * sets up the case (init.f90), runs iter = 0..maxit (maxit < 0: the
 * file's), and writes, in outdir, temp1_D60.dat .. temp3_D60.dat (t and
 * U(1..4) at the three probe points every ctd steps) and contorno_<n>.dat
 * every cgd steps, with the reference's screen lines on stdout.
 * flags: NS_RUN_NO_CONTORNO skips the field files, NS_RUN_QUIET the screen
 * lines. */
enum { NS_RUN_NO_CONTORNO = 1, NS_RUN_QUIET = 2 };
NS_API int ns_run_euler(const char *dados_path, const char *outdir, int nk, int device,
                        int maxit, int flags);

/*
 * ns_step_noalloc -- the time step for callers that cannot allocate device
 * memory.  No counterpart in the reference: it is an addition for hosts
 * whose device memory belongs to something else (a framework or pool that
 * hands out fixed buffers, a process under a hard memory cap where a
 * cudaMalloc failure in the middle of a run is not acceptable, a caller that
 * must not let an allocation synchronise the device between its own kernels).
 *
 * Advances the state U by nsteps calls of rk_euler without calling
 * cudaMalloc, cudaFree or any allocating library routine: every work array,
 * the transport-law table of a viscous case included, lives in one
 * file-scope __device__ array of NS_NOALLOC_MAX_BYTES, which every GPU that
 * loads the library keeps until the process exits.  The kernels are those of
 * ns_step, with the halo tiles read from global memory instead of by TMA
 * (the same arithmetic in the same order).  The caller passes the inputs and
 * the output: p as for ns_create (host arrays, read on every call), and U,
 * the device state: nk planes of jmax rows of `pitch` doubles (pitch >= imax,
 * a multiple of 32), updated in place.  stream: a cudaStream_t, NULL for the
 * default stream; the call returns once the work is enqueued.  The calling
 * thread's current device is the same after the call as before it.
 *
 * Limits: imax, jmax <= NS_NOALLOC_MAX_LINE, pitch <= NS_NOALLOC_MAX_BYTES/8,
 * and about (5*nk+9)*pitch*jmax doubles of work area (a 96x72 nk = 5 case
 * uses 1.9 MB; 512x480 with nk = 4 fits); larger cases are rejected with
 * NS_ERR_PARAM and a message giving the bytes needed.
 *
 * The first call on a device finds the work area's device address
 * (cudaGetSymbolAddress, with that device current, which may also load the
 * module).  Each call copies its setup tables from host memory that the next
 * call reuses; a call made on a stream that is capturing returns
 * NS_ERR_UNSUPPORTED without enqueueing anything.  Every call shares the
 * one work area and leaves its contents behind; each call writes every part
 * it reads, so results never depend on an earlier call, but calls that
 * overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.
 */
#define NS_NOALLOC_MAX_BYTES (64u << 20)
#define NS_NOALLOC_MAX_LINE 8192
NS_API int ns_step_noalloc(const ns_params *p, double *U, int64_t pitch, int iter0, int nsteps,
                           void *stream);

#ifdef __cplusplus
}
#endif
#endif /* NS_GB300_H */
