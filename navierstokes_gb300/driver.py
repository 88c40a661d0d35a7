"""The program around the step: dados.in, the init.f90 setup, the output
path and the euler.f90 time loop, over the C ABI (include/ns_gb300.h).

    d = read_dados("dados.in")            # init_read, init.f90:10-52
    g = dados_grid(d)                     # init_dados, init.f90:56-210
    s = solver_from_dados(d)              # U = Ub built on the device
    s.step(0, 100); omega = vorticity(s)  # outt.f90:43-49
    run_euler("dados.in", "out/")         # euler.f90:36-206

The same program is the `ns_euler` executable built next to the library.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import _lib as L
from .cases import Case, mixing_layer_case

DRIVER_PATH = Path(__file__).resolve().parent / "ns_euler"


def parse_dados(text: str) -> L.NsDados:
    d = L.NsDados()
    L.check(L.load().ns_parse_dados(text.encode(), C.byref(d)))
    return d


def read_dados(path) -> L.NsDados:
    d = L.NsDados()
    L.check(L.load().ns_read_dados(str(path).encode(), C.byref(d)))
    return d


def dados_grid(d: L.NsDados, quirk_buffer: bool = True) -> dict:
    """m, n, meshx, meshy, sigmax, sigmay, dm, dn and the 1-based probe
    points [(px1, py1), (px2, py2), (px3, py3)]."""
    imax, jmax = d.imax, d.jmax
    out = {k: np.zeros(imax if k in ("m", "meshx", "sigmax") else jmax)
           for k in ("m", "n", "meshx", "meshy", "sigmax", "sigmay")}
    hh = np.zeros(2)
    pij = np.zeros(6, dtype=np.int32)
    L.check(L.load().ns_dados_grid(C.byref(d), int(quirk_buffer), out["m"].ctypes.data,
                                   out["n"].ctypes.data, out["meshx"].ctypes.data,
                                   out["meshy"].ctypes.data, out["sigmax"].ctypes.data,
                                   out["sigmay"].ctypes.data, hh.ctypes.data, pij.ctypes.data))
    out["dm"], out["dn"] = float(hh[0]), float(hh[1])
    out["probes"] = [(int(pij[2 * q]), int(pij[2 * q + 1])) for q in range(3)]
    return out


def dados_profiles(d: L.NsDados, n: np.ndarray):
    """uba, Tb, rhob, psib of init_variables (init.f90:359-373)."""
    n = np.ascontiguousarray(n, dtype=np.float64)
    out = [np.zeros(d.jmax) for _ in range(4)]
    L.check(L.load().ns_dados_profiles(C.byref(d), n.ctypes.data, *[o.ctypes.data for o in out]))
    return tuple(out)


def dados_case(d: L.NsDados, nk: int = 5, quirk_buffer: bool = True) -> Case:
    """The dados.in case as a Case (for the oracle): the grid and the rows
    from the library's own setup, so both sides start from the same bits."""
    c = mixing_layer_case(imax=d.imax, jmax=d.jmax, nk=nk, maxit=d.maxit, dt=d.dt,
                          sigmaf=d.sigmaf, mmin=d.mmin, mmax=d.mmax, nmin=d.nmin, nmax=d.nmax,
                          U1=d.U1, U2=d.U2, Re=d.Re, Pr=d.Pr, T1=d.T1, T2=d.T2, Tref=d.Tref,
                          D=d.D, c1b=d.c1b, c2b=d.c2b, r0=d.r0_acous, amplitude=d.amplitude,
                          m_pt=d.m_pt_acous, n_pt=d.n_pt_acous, wf=d.wf,
                          quirk_buffer=quirk_buffer)
    g = dados_grid(d, quirk_buffer)
    for k in ("m", "n", "meshx", "meshy", "sigmax", "sigmay", "dm", "dn"):
        setattr(c, k, g[k])
    uba, _, rhob, psib = dados_profiles(d, g["n"])
    Ub = np.empty((d.jmax, d.imax, nk))
    Ub[:, :, 0] = rhob[:, None]
    Ub[:, :, 1] = uba[:, None]
    Ub[:, :, 2] = 0.0
    Ub[:, :, 3] = 1.0 / 1.4
    if nk == 5:
        Ub[:, :, 4] = psib[:, None]
    c.Ub, c.U0, c.rhob, c.psib = Ub, Ub.copy(), rhob, psib
    return c


def solver_from_dados(d: L.NsDados, nk: int = 5, device: int = 0, quirk_buffer: bool = True):
    """A Solver on ns_create_dados: state U = Ub, built on the device."""
    from .solver import Solver
    lib = L.load()
    ctx = C.c_void_p()
    L.check(lib.ns_create_dados(C.byref(d), nk, device, int(quirk_buffer), C.byref(ctx)))
    s = Solver.__new__(Solver)
    s.lib = lib
    s.case = dados_case(d, nk, quirk_buffer)
    s.shape = (d.jmax, d.imax, nk)
    s._ctx = ctx
    return s


def vorticity(solver) -> np.ndarray:
    """omega = dv/dx - du/dy with diffall.f90's metric-free DRP, (jmax, imax)."""
    c = solver.case
    om = np.empty((c.jmax, c.imax))
    L.check(solver.lib.ns_vorticity(solver._ctx, om.ctypes.data), solver._ctx)
    return om


def write_contorno(solver, path) -> None:
    c = solver.case
    m = np.ascontiguousarray(c.m, dtype=np.float64)
    n = np.ascontiguousarray(c.n, dtype=np.float64)
    L.check(solver.lib.ns_write_contorno(solver._ctx, str(path).encode(), m.ctypes.data,
                                         n.ctypes.data), solver._ctx)


def format_real(x: float) -> str:
    buf = C.create_string_buffer(32)
    if L.load().ns_format_real(float(x), buf, 32) != 25:
        raise ValueError("ns_format_real failed")
    return buf.value.decode()


class ProbeRecorder:
    """ns_probes_*: U(1..nk) at fixed points, captured on the device."""

    def __init__(self, solver, points, capacity=1024):
        self.s = solver
        self.npts = len(points)
        pi = np.array([p[0] for p in points], dtype=np.int32)
        pj = np.array([p[1] for p in points], dtype=np.int32)
        L.check(solver.lib.ns_probes_arm(solver._ctx, self.npts, pi.ctypes.data, pj.ctypes.data,
                                         int(capacity)), solver._ctx)
        self.capacity = capacity

    def capture(self) -> None:
        L.check(self.s.lib.ns_probes_capture(self.s._ctx), self.s._ctx)

    def drain(self) -> np.ndarray:
        nk = self.s.case.nk
        out = np.empty((self.capacity, self.npts, nk))
        nrec = C.c_int()
        L.check(self.s.lib.ns_probes_drain(self.s._ctx, out.ctypes.data, C.byref(nrec)),
                self.s._ctx)
        return out[:nrec.value].copy()


def run_euler(dados_path, outdir=".", nk: int = 5, device: int = 0, maxit: int = -1,
              contorno: bool = True, quiet: bool = True) -> None:
    flags = (0 if contorno else L.NS_RUN_NO_CONTORNO) | (L.NS_RUN_QUIET if quiet else 0)
    os.makedirs(outdir, exist_ok=True)
    L.check(L.load().ns_run_euler(str(dados_path).encode(), str(outdir).encode(), nk, device,
                                  int(maxit), flags))
