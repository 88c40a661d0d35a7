"""CPU oracle for the LDDRK time-step hot path -- TEST INFRASTRUCTURE ONLY.

Wraps ns_oracle.c, the plain-C FP64 restatement of the reference's rk.f90
stage loop and everything it calls (see the header of ns_oracle.c).  Only
tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it; the
product library never loads it.

Parity status: unpinned by reference-produced vectors -- the Fortran
reference ships no tests or fixtures and cannot be compiled here.  The
restatement is pinned by known-answer tests derived from the reference's
coefficient tables (tests/test_oracle_kat.py) and cross-checked against an
independent NumPy restatement (oracle/numpy_ref.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "ns_oracle.c"
HDR = HERE / "ns_oracle.h"
LIB = HERE / "_build" / "libns_oracle.so"
# The same source built with AddressSanitizer and UndefinedBehaviorSanitizer
# (abort on the first report); loaded instead of LIB when NS_ORACLE_SANITIZE
# is set, in a process that preloads the ASan runtime.
LIB_SANITIZED = HERE / "_build" / "libns_oracle_san.so"
# -ffp-contract=off: no fused multiply-add, so the oracle rounds every
# operation as the reference's statements do, on x86 and on Arm alike.
CFLAGS = ["-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
          "-std=c11", "-Wall"]
SANITIZE_FLAGS = ["-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
                  "-fno-sanitize-recover=all"]


def build(force: bool = False, sanitize: bool = False) -> Path:
    lib = LIB_SANITIZED if sanitize else LIB
    lib.parent.mkdir(exist_ok=True)
    if not force and lib.exists() and lib.stat().st_mtime >= max(SRC.stat().st_mtime,
                                                                  HDR.stat().st_mtime):
        return lib
    tmp = lib.with_suffix(".tmp.so")
    flags = [f for f in CFLAGS if f != "-O3"] + SANITIZE_FLAGS if sanitize else CFLAGS
    cmd = ["gcc", *flags, str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


class OraParams(C.Structure):
    _fields_ = [
        ("imax", C.c_int), ("jmax", C.c_int), ("nk", C.c_int), ("D", C.c_int),
        ("inviscid", C.c_int), ("metric_mode", C.c_int),
        ("dt", C.c_double), ("dm", C.c_double), ("dn", C.c_double), ("sigmaf", C.c_double),
        ("gamma", C.c_double), ("Re", C.c_double), ("Pr", C.c_double), ("Tref", C.c_double),
        ("meshx", C.c_void_p), ("meshy", C.c_void_p), ("sigmax", C.c_void_p),
        ("sigmay", C.c_void_p), ("Ub", C.c_void_p), ("rhob", C.c_void_p), ("psib", C.c_void_p),
        ("source_mode", C.c_int),
        ("m", C.c_void_p), ("n", C.c_void_p),
        ("amplitude", C.c_double), ("wf", C.c_double), ("m_pt", C.c_double),
        ("n_pt", C.c_double), ("r0", C.c_double),
        ("src_field", C.c_void_p),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build(sanitize=bool(os.environ.get("NS_ORACLE_SANITIZE")))
        L = C.CDLL(str(path))
        L.ora_create.restype = C.c_void_p
        L.ora_create.argtypes = [C.POINTER(OraParams)]
        L.ora_destroy.argtypes = [C.c_void_p]
        L.ora_run.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        for name in ("ora_deropm", "ora_deropn"):
            getattr(L, name).argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        for name in ("ora_filterx", "ora_filtery"):
            getattr(L, name).argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.ora_ccpml.argtypes = [C.c_void_p, C.c_void_p]
        L.ora_bufferxy.argtypes = [C.c_void_p, C.c_void_p]
        L.ora_rhs.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double]
        L.ora_transport_ref.argtypes = [C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.ora_transport.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_double),
                                    C.POINTER(C.c_double)]
        L.ora_init_dados.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_double] * 6 + [C.c_int] + \
            [C.c_void_p] * 6 + [C.POINTER(C.c_double)] * 2
        L.ora_mixing_layer.argtypes = [C.c_int, C.c_void_p] + [C.c_double] * 4 + \
            [C.c_void_p] * 4
        L.ora_vorticity.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                    C.c_void_p, C.c_void_p]
        L.ora_coeffs.argtypes = [C.c_int, C.c_void_p]
        L.ora_coeffs.restype = C.c_int
        L.ora_set_threads.argtypes = [C.c_int]
        L.ora_get_threads.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def coeffs(which: int) -> np.ndarray:
    out = np.zeros(16)
    n = lib().ora_coeffs(which, out.ctypes.data)
    return out[:n].copy()


def set_threads(n: int) -> None:
    lib().ora_set_threads(int(n))


def get_threads() -> int:
    return int(lib().ora_get_threads())


def transport(Tref: float, T: float):
    mu, k = C.c_double(), C.c_double()
    lib().ora_transport(Tref, T, C.byref(mu), C.byref(k))
    return mu.value, k.value


def transport_ref(Tref: float):
    mu0, k0 = C.c_double(), C.c_double()
    lib().ora_transport_ref(Tref, C.byref(mu0), C.byref(k0))
    return mu0.value, k0.value


def init_dados(imax, jmax, D, mmin, mmax, nmin, nmax, c1b, c2b, quirk_buffer=True):
    """init.f90:56-210 -> dict of m, n, meshx, meshy, sigmax, sigmay, dm, dn."""
    out = {k: np.zeros(imax if k in ("m", "meshx", "sigmax") else jmax)
           for k in ("m", "n", "meshx", "meshy", "sigmax", "sigmay")}
    dm, dn = C.c_double(), C.c_double()
    lib().ora_init_dados(imax, jmax, D, mmin, mmax, nmin, nmax, c1b, c2b, int(quirk_buffer),
                         out["m"].ctypes.data, out["n"].ctypes.data, out["meshx"].ctypes.data,
                         out["meshy"].ctypes.data, out["sigmax"].ctypes.data,
                         out["sigmay"].ctypes.data, C.byref(dm), C.byref(dn))
    out["dm"], out["dn"] = dm.value, dn.value
    return out


def mixing_layer(n, U1, U2, T1, T2):
    """init.f90:359-373 -> uba, Tb, rhob, psib on the rows n."""
    n = np.ascontiguousarray(n, dtype=np.float64)
    out = [np.zeros(len(n)) for _ in range(4)]
    lib().ora_mixing_layer(len(n), n.ctypes.data, U1, U2, T1, T2, *[o.ctypes.data for o in out])
    return tuple(out)


def vorticity(U, dm, dn):
    """outt.f90:43-49 with diffall.f90's metric-free DRP: U is the memory of
    U(nk,imax,jmax) shaped (jmax, imax, nk); returns omega (jmax, imax)."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    jmax, imax, nk = U.shape
    om = np.zeros((jmax, imax))
    lib().ora_vorticity(imax, jmax, nk, dm, dn, U.ctypes.data, om.ctypes.data)
    return om


class Oracle:
    """The reference stage loop on the CPU, on the reference's U(nk,imax,jmax).

    `case` is any object with the attributes of navierstokes_gb300.cases.Case
    (sizes, scalars, 1-D setup arrays, Ub).  State arrays are NumPy arrays of
    shape (jmax, imax, nk), C order -- the memory of the Fortran array
    U(nk,imax,jmax).
    """

    def __init__(self, case):
        self.case = case
        self._keep = []

        def arr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            self._keep.append(a)
            return a.ctypes.data

        p = OraParams()
        p.imax, p.jmax, p.nk, p.D = case.imax, case.jmax, case.nk, case.D
        p.inviscid = int(case.inviscid)
        p.metric_mode = int(case.metric_mode)
        p.dt, p.dm, p.dn, p.sigmaf = case.dt, case.dm, case.dn, case.sigmaf
        p.gamma, p.Re, p.Pr, p.Tref = case.gamma, case.Re, case.Pr, case.Tref
        p.meshx, p.meshy = arr(case.meshx), arr(case.meshy)
        p.sigmax, p.sigmay = arr(case.sigmax), arr(case.sigmay)
        p.Ub, p.rhob, p.psib = arr(case.Ub), arr(case.rhob), arr(case.psib)
        p.source_mode = int(case.source_mode)
        p.m, p.n = arr(case.m), arr(case.n)
        p.amplitude, p.wf = case.amplitude, case.wf
        p.m_pt, p.n_pt, p.r0 = case.m_pt, case.n_pt, case.r0
        p.src_field = arr(case.src_field)
        self._p = p
        self._ctx = lib().ora_create(C.byref(p))
        if not self._ctx:
            raise ValueError("ora_create rejected the case")

    def close(self):
        if self._ctx:
            lib().ora_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, U):
        c = self.case
        assert U.dtype == np.float64 and U.flags.c_contiguous
        assert U.shape == (c.jmax, c.imax, c.nk), U.shape

    def run(self, U: np.ndarray, iter0: int, nsteps: int) -> np.ndarray:
        """Advances U in place by nsteps calls of rk_euler; returns U."""
        self._check(U)
        lib().ora_run(self._ctx, U.ctypes.data, int(iter0), int(nsteps))
        return U

    def rhs(self, U, iter_=0, ct=0.0):
        self._check(U)
        out = np.zeros_like(U)
        lib().ora_rhs(self._ctx, out.ctypes.data, U.ctypes.data, int(iter_), float(ct))
        return out

    def deropm(self, F):
        F = np.ascontiguousarray(F, dtype=np.float64)
        out = np.zeros_like(F)
        lib().ora_deropm(self._ctx, out.ctypes.data, F.ctypes.data, F.shape[2])
        return out

    def deropn(self, F):
        F = np.ascontiguousarray(F, dtype=np.float64)
        out = np.zeros_like(F)
        lib().ora_deropn(self._ctx, out.ctypes.data, F.ctypes.data, F.shape[2])
        return out

    def filterx(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64).copy()
        lib().ora_filterx(self._ctx, U.ctypes.data, U.shape[2])
        return U

    def filtery(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64).copy()
        lib().ora_filtery(self._ctx, U.ctypes.data, U.shape[2])
        return U

    def ccpml(self, U):
        self._check(U)
        U = U.copy()
        lib().ora_ccpml(self._ctx, U.ctypes.data)
        return U

    def bufferxy(self, U):
        self._check(U)
        U = U.copy()
        lib().ora_bufferxy(self._ctx, U.ctypes.data)
        return U
