"""Problem setup: every input the time step reads, built on the host.

`init_dados` and `mixing_layer` restate the reference's setup routines
(init.f90:56-210 and :341-404); the other builders are the initial-condition
hooks the reference lacks (it hard-codes a tanh mixing layer and zero
perturbation, init.f90:368-390): a quiescent or uniform mean flow with a
Gaussian acoustic pulse and a Gaussian isentropic vortex, and a stretched y
grid.  They are new, not reference behaviour.

State arrays are NumPy float64 arrays of shape (jmax, imax, nk), C order:
the memory of the reference's Fortran array U(nk,imax,jmax).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

from . import _lib as L

GAMMA = 1.4          # init.f90:361
# Svehla N2 fit, coefficients.f90:113-123 (SPECIE_N)
N2_FIT = dict(A_mi=0.62526577, B_mi=-31.779652, C_mi=-1640.7913, D_mi=1.7454992,
              A_k=0.85372829, B_k=105.18665, C_k=-12229.753, D_k=0.48299104)


@dataclasses.dataclass
class Case:
    name: str
    imax: int
    jmax: int
    nk: int
    D: int
    dt: float
    dm: float
    dn: float
    sigmaf: float
    m: np.ndarray
    n: np.ndarray
    meshx: np.ndarray
    meshy: np.ndarray
    sigmax: np.ndarray
    sigmay: np.ndarray
    Ub: np.ndarray          # (jmax, imax, nk)
    rhob: np.ndarray
    psib: np.ndarray
    U0: np.ndarray          # (jmax, imax, nk)
    inviscid: bool = False
    metric_mode: int = L.NS_METRIC_BANDS
    gamma: float = GAMMA
    Re: float = 10000.0
    Pr: float = 0.71
    Tref: float = 273.15
    source_mode: int = L.NS_SRC_NONE
    amplitude: float = 0.0
    wf: float = 0.0
    m_pt: float = 0.0
    n_pt: float = 0.0
    r0: float = 1.0
    src_field: Optional[np.ndarray] = None   # (jmax, imax)
    steps: int = 1
    notes: str = ""

    @property
    def points(self) -> int:
        return self.imax * self.jmax

    def state_bytes(self) -> int:
        return self.imax * self.jmax * self.nk * 8


# --------------------------------------------------------------------------
# Reference setup routines
# --------------------------------------------------------------------------

def init_dados(imax, jmax, D, mmin, mmax, nmin, nmax, c1b, c2b, quirk_buffer=True):
    """Grid, buffer metrics and damping profiles, init.f90:56-210.

    quirk_buffer=True reproduces the reference as compiled: imaxpml/jmaxpml
    are never assigned (global.f90:86), so the left and bottom sigma stay 0
    (init.f90:168, :192) and those buffers clamp the state to Ub.
    """
    imaxpml = 0 if quirk_buffer else D
    jmaxpml = 0 if quirk_buffer else D
    Aa, alpham = 2.0, 2.0
    dm = (mmax - mmin) / float(imax - 1)
    dn = (nmax - nmin) / float(jmax - 1)
    Dx, Dy = dm * D, dn * D
    xli, xld, yli, yls = mmin + Dx, mmax - Dx, nmin + Dy, nmax - Dy
    i = np.arange(1, imax + 1)
    j = np.arange(1, jmax + 1)
    m = mmin + (i - 1).astype(np.float64) * dm
    n = nmin + (j - 1).astype(np.float64) * dn
    meshx = np.ones(imax)
    meshy = np.ones(jmax)
    for q in range(imax):
        ii = q + 1
        if 1 <= ii <= D + 1:
            meshx[q] = 1.0 / (1.0 + Aa * math.pow(abs((m[q] - xli) / Dx), alpham))
        if imax - D <= ii <= imax:
            meshx[q] = 1.0 / (1.0 + Aa * math.pow(abs((m[q] - xld) / Dx), alpham))
    for q in range(jmax):
        jj = q + 1
        if 1 <= jj <= D + 1:
            meshy[q] = 1.0 / (1.0 + Aa * math.pow(abs((n[q] - yli) / Dy), alpham))
        if jmax - D + 1 <= jj <= jmax:
            meshy[q] = 1.0 / (1.0 + Aa * math.pow(abs((n[q] - yls) / Dy), alpham))

    def prof(z, zs, ze):
        x = (z - zs) / (ze - zs)
        return (1.0 - c1b * x * x) * (1.0 - (1.0 - math.exp(c2b * x * x)) / (1.0 - math.exp(c2b)))

    sigmax = np.zeros(imax)
    sigmay = np.zeros(jmax)
    for q in range(imax):
        ii = q + 1
        if 1 <= ii <= imaxpml:
            sigmax[q] = prof(m[q], xli, mmin)
        if imax - D + 1 <= ii <= imax:
            sigmax[q] = prof(m[q], xld, mmax)
    for q in range(jmax):
        jj = q + 1
        if 1 <= jj <= jmaxpml:
            sigmay[q] = prof(n[q], yli, nmin)
        if jmax - D + 1 <= jj <= jmax:
            sigmay[q] = prof(n[q], yls, nmax)
    return dict(m=m, n=n, meshx=meshx, meshy=meshy, sigmax=sigmax, sigmay=sigmay, dm=dm, dn=dn)


def psi_profile(n, deltamx=0.4, psi1=1.0, psi2=0.0):
    """psib(j), init.f90:372."""
    return 0.5 * (psi1 + psi2 + (psi1 - psi2) * np.tanh(2.0 * n / deltamx))


def mixing_layer(n, U1, U2, T1, T2, gamma=GAMMA, deltamx=0.4):
    """Base mixing-layer profiles uba, Tb, rhob, psib, init.f90:368-373."""
    uba = 0.5 * (U1 + U2 + (U1 - U2) * np.tanh(2.0 * n / deltamx))
    Tb = T1 * (uba - U2) / (U1 - U2) + T2 * (U1 - uba) / (U1 - U2) + \
        (gamma - 1.0) / 2.0 * (U1 - uba) * (uba - U2)
    rhob = 1.0 / Tb
    return uba, Tb, rhob, psi_profile(n, deltamx)


def base_field(imax, nk, rho_j, u_j, v_j, p_j, psi_j):
    """Ub(k,i,j) from 1-D profiles (init.f90:392-404), shape (jmax, imax, nk)."""
    jmax = len(rho_j)
    Ub = np.empty((jmax, imax, nk))
    Ub[:, :, 0] = np.asarray(rho_j)[:, None]
    Ub[:, :, 1] = np.asarray(u_j)[:, None]
    Ub[:, :, 2] = np.asarray(v_j)[:, None]
    Ub[:, :, 3] = np.asarray(p_j)[:, None]
    if nk >= 5:
        Ub[:, :, 4] = np.asarray(psi_j)[:, None]
    return Ub


# --------------------------------------------------------------------------
# Cases
# --------------------------------------------------------------------------

def mixing_layer_case(imax=521, jmax=481, nk=5, maxit=8000, dt=0.01, sigmaf=0.1,
                      mmin=-6.5, mmax=19.5, nmin=-2.4, nmax=2.4, U1=0.9, U2=0.1, Re=10000.0,
                      Pr=0.71, T1=1.0, T2=0.5, Tref=273.15, D=90, c1b=0.01, c2b=20.0,
                      r0=0.03, amplitude=0.8, m_pt=0.0, n_pt=0.0, wf=1.0, quirk_buffer=True):
    """The reference's own case: dados.in (dados.in:1-85) through init_dados and
    init_variables (init.f90:56-418): a tanh mixing layer excited by the
    time-harmonic acoustic source of rk.f90:171-193."""
    g = init_dados(imax, jmax, D, mmin, mmax, nmin, nmax, c1b, c2b, quirk_buffer)
    uba, Tb, rhob, psib = mixing_layer(g["n"], U1, U2, T1, T2)
    p = np.full(jmax, 1.0 / GAMMA)
    Ub = base_field(imax, nk, rhob, uba, np.zeros(jmax), p, psib)
    return Case(name=f"mixing_layer_{imax}x{jmax}", imax=imax, jmax=jmax, nk=nk, D=D, dt=dt,
                dm=g["dm"], dn=g["dn"], sigmaf=sigmaf, m=g["m"], n=g["n"], meshx=g["meshx"],
                meshy=g["meshy"], sigmax=g["sigmax"], sigmay=g["sigmay"], Ub=Ub, rhob=rhob,
                psib=psib, U0=Ub.copy(), inviscid=False, Re=Re, Pr=Pr, Tref=Tref,
                source_mode=L.NS_SRC_GAUSSIAN, amplitude=amplitude, wf=wf, m_pt=m_pt,
                n_pt=n_pt, r0=r0, steps=maxit + 1,
                notes="reference dados.in mixing layer (init.f90:341-404)")


def _pulse(X, Y, xc, yc, amp, halfwidth):
    return amp * np.exp(-math.log(2.0) * ((X - xc) ** 2 + (Y - yc) ** 2) / halfwidth ** 2)


def _isentropic_vortex(X, Y, xc, yc, eps, R, gamma=GAMMA):
    """Gaussian isentropic vortex on T = gamma*p/rho = 1, rho = 1:
    u_theta = eps*(r/R)*exp((1-r^2/R^2)/2), T = 1 - (gamma-1)/2*eps^2*exp(1-r^2/R^2),
    rho = T^(1/(gamma-1)), p = T^(gamma/(gamma-1))/gamma."""
    r2 = ((X - xc) ** 2 + (Y - yc) ** 2) / R ** 2
    e = np.exp(0.5 * (1.0 - r2))
    du = -eps * (Y - yc) / R * e
    dv = eps * (X - xc) / R * e
    T = 1.0 - (gamma - 1.0) / 2.0 * eps ** 2 * np.exp(1.0 - r2)
    rho = T ** (1.0 / (gamma - 1.0))
    p = T ** (gamma / (gamma - 1.0)) / gamma
    return rho, du, dv, p


def acoustic_pulse_case(imax=201, jmax=201, nk=5, D=30, sigmaf=0.2, amp=0.01, halfwidth=3.0,
                        mach=0.0, cfl=0.5, steps=500, c1b=0.01, c2b=20.0, quirk_buffer=True,
                        inviscid=True, Re=1000.0, Pr=0.72):
    """Gaussian acoustic pulse p' = rho'*c^2 = amp*exp(-ln2*r^2/b^2) at the grid
    centre in a quiescent (mach = 0) or uniform (mean u = mach) medium on a
    uniform grid with dx = dy = 1 centred on the origin.  rho = 1,
    p = 1/gamma, so c = 1 and dt = cfl*dx/(|u|+c)."""
    hx, hy = (imax - 1) / 2.0, (jmax - 1) / 2.0
    g = init_dados(imax, jmax, D, -hx, hx, -hy, hy, c1b, c2b, quirk_buffer)
    X, Y = np.meshgrid(g["m"], g["n"])      # (jmax, imax)
    rho0 = np.ones(jmax)
    psib = psi_profile(g["n"])
    Ub = base_field(imax, nk, rho0, np.full(jmax, mach), np.zeros(jmax),
                    np.full(jmax, 1.0 / GAMMA), psib)
    U0 = Ub.copy()
    pp = _pulse(X, Y, 0.0, 0.0, amp, halfwidth)
    U0[:, :, 3] += pp
    U0[:, :, 0] += pp          # rho' = p'/c^2, c = 1
    dt = cfl * min(g["dm"], g["dn"]) / (abs(mach) + 1.0)
    return Case(name=f"acoustic_pulse_{imax}x{jmax}", imax=imax, jmax=jmax, nk=nk, D=D, dt=dt,
                dm=g["dm"], dn=g["dn"], sigmaf=sigmaf, m=g["m"], n=g["n"], meshx=g["meshx"],
                meshy=g["meshy"], sigmax=g["sigmax"], sigmay=g["sigmay"], Ub=Ub, rhob=rho0,
                psib=psib, U0=U0, inviscid=inviscid, Re=Re, Pr=Pr, steps=steps,
                notes="Gaussian pulse, uniform grid (new initial-condition hook)")


# Stability of the explicit step for the viscous terms: the LDDRK
# amplification polynomial (rk.f90:27-46) stays within |G| <= 1 on the
# negative real axis up to z = -4.071, and a diffusion operator built from two
# DRP first derivatives (diff.f90:40-47) has eigenvalues down to
# -2.703*nu/h^2 per direction.
LDDRK_REAL_LIMIT = 4.071
DRP_K2_MAX = 2.7034


def viscous_dt(Re, Pr, inv_h2_sum, gamma=GAMMA, safety=0.5):
    """Largest stable dt of the diffusion terms: the stress term diffuses
    momentum with nu = (4/3)/Re and the heat-flux term of eqeuler.f90:90-91
    diffuses pressure with gamma/(Re*Pr) (rho = T = 1)."""
    nu = max(4.0 / 3.0 / Re, gamma / (Re * Pr))
    return safety * LDDRK_REAL_LIMIT / (nu * DRP_K2_MAX * inv_h2_sum)


def uniform_flow_case(imax=4096, jmax=4096, nk=4, D=30, sigmaf=0.2, mach=0.5, pulse_amp=1e-4,
                      pulse_halfwidth=3.0, vortex_eps=1e-3, vortex_radius=6.0,
                      vortex_upstream=200, cfl=0.5, steps=1000, c1b=0.01, c2b=20.0,
                      quirk_buffer=True, inviscid=True, Re=1000.0, Pr=0.72):
    """Euler on a uniform grid (dx = dy = 1, centred on the origin) with a
    uniform mean flow u = mach, rho = 1, p = 1/gamma, a Gaussian pulse
    p' = rho' = pulse_amp*exp(-ln2*r^2/b^2) at the centre and a Gaussian
    isentropic vortex of strength vortex_eps and radius vortex_radius cells
    vortex_upstream cells upstream; dt = cfl*dx/(|u|+c).  With the default
    sizes this is the split-precision workload: the acoustic-pulse case
    scaled to 4096x4096 at M = 0.5 with small perturbations."""
    hx, hy = (imax - 1) / 2.0, (jmax - 1) / 2.0
    g = init_dados(imax, jmax, D, -hx, hx, -hy, hy, c1b, c2b, quirk_buffer)
    X, Y = np.meshgrid(g["m"], g["n"])
    rho0 = np.ones(jmax)
    psib = psi_profile(g["n"])
    Ub = base_field(imax, nk, rho0, np.full(jmax, mach), np.zeros(jmax),
                    np.full(jmax, 1.0 / GAMMA), psib)
    U0 = Ub.copy()
    pp = _pulse(X, Y, 0.0, 0.0, pulse_amp, pulse_halfwidth)
    vr, vu, vv, vp = _isentropic_vortex(X, Y, -float(vortex_upstream), 0.0, vortex_eps,
                                        vortex_radius)
    U0[:, :, 0] = vr + pp
    U0[:, :, 1] = mach + vu
    U0[:, :, 2] = vv
    U0[:, :, 3] = vp + pp
    dt = cfl * min(g["dm"], g["dn"]) / (abs(mach) + 1.0)
    return Case(name=f"uniform_flow_{imax}x{jmax}", imax=imax, jmax=jmax, nk=nk, D=D, dt=dt,
                dm=g["dm"], dn=g["dn"], sigmaf=sigmaf, m=g["m"], n=g["n"], meshx=g["meshx"],
                meshy=g["meshy"], sigmax=g["sigmax"], sigmay=g["sigmay"], Ub=Ub, rhob=rho0,
                psib=psib, U0=U0, inviscid=inviscid, Re=Re, Pr=Pr, steps=steps,
                notes="uniform mean flow, pulse + isentropic vortex (new hook)")


def stretched_ns_case(imax=4096, jmax=2048, nk=4, D=40, sigmaf=0.2, mach=0.5, Re=1000.0,
                      Pr=0.72, pulse_amp=1e-3, pulse_cells=4.0, vortex_eps=0.1,
                      vortex_cells=6.0, vortex_upstream=200, cfl=0.5, steps=200, c1b=0.01,
                      c2b=20.0, beta=2.5, quirk_buffer=True):
    """Navier-Stokes on a y-grid stretched toward the centreline: the
    computational coordinate eta = n(j), uniform in [-1, 1], is
    eta = tanh(beta*y)/tanh(beta), i.e. y = atanh(eta*tanh(beta))/beta, so the
    rows are finest at y = 0 (dy = deta*tanh(beta)/beta) and coarsest at
    y = +-1.  meshy(j) = d(eta)/dy times the buffer factor of
    init.f90:139-153, applied to every y-derivative (NS_METRIC_EVERYWHERE).
    x is uniform with dx equal to the centreline dy.  Uniform mean flow
    u = mach, rho = 1, p = 1/gamma; a pulse of half-width pulse_cells*dx at
    the centre and an isentropic vortex of radius vortex_cells*dx,
    vortex_upstream cells upstream.  dt is the smaller of the convective
    CFL step and half the viscous stability limit (which binds at Re = 1000
    on this grid)."""
    dn = 2.0 / (jmax - 1)
    tb = math.tanh(beta)
    dx = dn * tb / beta
    g = init_dados(imax, jmax, D, 0.0, dx * (imax - 1), -1.0, 1.0, c1b, c2b, quirk_buffer)
    eta = g["n"]
    yphys = np.arctanh(np.clip(eta * tb, -1.0, 1.0)) / beta
    detady = beta * (1.0 - (eta * tb) ** 2) / tb
    meshy = g["meshy"] * detady
    X, Y = np.meshgrid(g["m"], yphys)
    xc = g["m"][imax // 2]
    psib = psi_profile(eta)
    rho0 = np.ones(jmax)
    Ub = base_field(imax, nk, rho0, np.full(jmax, mach), np.zeros(jmax),
                    np.full(jmax, 1.0 / GAMMA), psib)
    U0 = Ub.copy()
    pp = _pulse(X, Y, xc, 0.0, pulse_amp, pulse_cells * dx)
    vr, vu, vv, vp = _isentropic_vortex(X, Y, xc - vortex_upstream * dx, 0.0, vortex_eps,
                                        vortex_cells * dx)
    U0[:, :, 0] = vr + pp
    U0[:, :, 1] = mach + vu
    U0[:, :, 2] = vv
    U0[:, :, 3] = vp + pp
    dy_min = float(np.min(np.diff(yphys)))
    dt_conv = cfl * min(dx / (abs(mach) + 1.0), dy_min / 1.0)
    inv_h2 = 1.0 / dx ** 2 + float(np.max(meshy / dn)) ** 2
    dt = min(dt_conv, viscous_dt(Re, Pr, inv_h2))
    return Case(name=f"stretched_ns_{imax}x{jmax}", imax=imax, jmax=jmax, nk=nk, D=D, dt=dt,
                dm=g["dm"], dn=g["dn"], sigmaf=sigmaf, m=g["m"], n=eta, meshx=g["meshx"],
                meshy=meshy, sigmax=g["sigmax"], sigmay=g["sigmay"], Ub=Ub, rhob=rho0,
                psib=psib, U0=U0, inviscid=False, metric_mode=L.NS_METRIC_EVERYWHERE, Re=Re,
                Pr=Pr, steps=steps,
                notes="eta = tanh(2.5 y)/tanh(2.5) (finest at y = 0), pulse + isentropic "
                      "vortex, dt = min(CFL 0.5, viscous limit) (new hook)")


def sweep_cases(n=64, seed=0, nmin=128, nmax=1024, D=30, sigmaf=0.2, cfl=0.5, steps=300,
                quirk_buffer=True):
    """The parameter sweep of many independent Euler instances: sizes
    Nx, Ny = 32*round(exp(U[ln nmin, ln nmax])/32), a time-harmonic monopole
    S = A*sin(omega*t)*exp(-ln2*r^2/3^2) at the centre (the form of
    rk.f90:188-189, with stage time) with A ~ U[1e-4, 1e-2] and
    omega ~ U[0.2, 1.0], and a uniform mean flow M ~ U[0, 0.6] along x.
    Uniform grids with dx = dy = 1, quiescent start, dt = cfl/(M+1).
    Draws come from numpy.random.default_rng(seed) in this order: Nx, Ny, A,
    omega, M (each an array of n)."""
    rng = np.random.default_rng(seed)
    lo, hi = math.log(nmin), math.log(nmax)
    nx = (32 * np.round(np.exp(rng.uniform(lo, hi, n)) / 32)).astype(int)
    ny = (32 * np.round(np.exp(rng.uniform(lo, hi, n)) / 32)).astype(int)
    amp = rng.uniform(1e-4, 1e-2, n)
    omega = rng.uniform(0.2, 1.0, n)
    mach = rng.uniform(0.0, 0.6, n)
    out = []
    for q in range(n):
        c = uniform_flow_case(imax=int(nx[q]), jmax=int(ny[q]), mach=float(mach[q]), D=D,
                              sigmaf=sigmaf, pulse_amp=0.0, vortex_eps=0.0, cfl=cfl,
                              steps=steps, quirk_buffer=quirk_buffer)
        c.name = f"sweep{q}_{c.imax}x{c.jmax}"
        c.source_mode = L.NS_SRC_GAUSSIAN
        c.amplitude, c.wf, c.m_pt, c.n_pt, c.r0 = float(amp[q]), float(omega[q]), 0.0, 0.0, 3.0
        c.notes = f"sweep instance {q} (seed {seed}): A={amp[q]:.3g} omega={omega[q]:.3g} M={mach[q]:.3g}"
        out.append(c)
    return out


def params_from_case(case: Case, device: int = 0, precision: int = L.NS_PREC_FP64):
    """Fills an ns_params for `case`; returns (params, keep-alive arrays)."""
    lib = L.load()
    p = L.NsParams()
    lib.ns_params_init(C_ref(p))
    keep = []

    def arr(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return a.ctypes.data

    p.imax, p.jmax, p.nk, p.D = case.imax, case.jmax, case.nk, case.D
    p.inviscid = int(case.inviscid)
    p.metric_mode = int(case.metric_mode)
    p.precision = int(precision)
    p.source_mode = int(case.source_mode)
    p.device = int(device)
    p.ub_layout = L.NS_LAYOUT_FORTRAN
    p.dt, p.dm, p.dn, p.sigmaf = case.dt, case.dm, case.dn, case.sigmaf
    p.gamma, p.Re, p.Pr, p.Tref = case.gamma, case.Re, case.Pr, case.Tref
    for k, v in N2_FIT.items():
        setattr(p, k, v)
    p.amplitude, p.wf, p.m_pt, p.n_pt, p.r0 = case.amplitude, case.wf, case.m_pt, case.n_pt, case.r0
    p.m, p.n = arr(case.m), arr(case.n)
    p.meshx, p.meshy = arr(case.meshx), arr(case.meshy)
    p.sigmax, p.sigmay = arr(case.sigmax), arr(case.sigmay)
    p.rhob, p.psib = arr(case.rhob), arr(case.psib)
    p.Ub = arr(case.Ub)
    p.src_field = arr(case.src_field)
    return p, keep


def C_ref(p):
    import ctypes
    return ctypes.byref(p)
