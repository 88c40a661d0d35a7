"""Host-side mirror of the reference's time-step interface over the C ABI.

`Solver.rk_euler(U, t, iter)` is the drop-in for `call rk_euler(U,t,iter,nk)`
(euler.f90:130, rk.f90:12): the host array U (memory of U(nk,imax,jmax)) is
advanced one LDDRK step in place.  The resident-state calls (set_state, step,
get_state, probes) are what a time loop uses to keep U on the GPU between
steps, reading back only probes and dumps (euler.f90:133-161).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .cases import Case, params_from_case


class Solver:
    def __init__(self, case: Case, device: int = 0, precision: int = L.NS_PREC_FP64):
        self.lib = L.load()
        self.case = case
        self.shape = (case.jmax, case.imax, case.nk)
        params, keep = params_from_case(case, device=device, precision=precision)
        ctx = C.c_void_p()
        rc = self.lib.ns_create(C.byref(params), C.byref(ctx))
        L.check(rc)
        self._ctx = ctx
        del keep

    # -- lifecycle -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self.lib.ns_destroy(self._ctx)
            self._ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _rc(self, rc):
        L.check(rc, self._ctx)

    # -- state ---------------------------------------------------------------
    def _host(self, U, writable=False):
        if not isinstance(U, np.ndarray) or U.dtype != np.float64 or not U.flags.c_contiguous:
            raise TypeError("U must be a C-contiguous float64 ndarray")
        if U.shape != self.shape:
            raise ValueError(f"U has shape {U.shape}, expected {self.shape} (jmax, imax, nk)")
        if writable and not U.flags.writeable:
            raise ValueError("U must be writable")
        return U.ctypes.data

    def set_state(self, U: np.ndarray) -> None:
        self._rc(self.lib.ns_set_state(self._ctx, self._host(U), L.NS_LAYOUT_FORTRAN))

    def get_state(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.shape)
        self._rc(self.lib.ns_get_state(self._ctx, self._host(out, True), L.NS_LAYOUT_FORTRAN))
        return out

    def step(self, iter0: int, nsteps: int = 1) -> None:
        """Enqueues nsteps calls of rk_euler with iter = iter0, iter0+1, ..."""
        self._rc(self.lib.ns_step(self._ctx, int(iter0), int(nsteps)))

    def synchronize(self) -> None:
        self._rc(self.lib.ns_synchronize(self._ctx))

    def rk_euler(self, U: np.ndarray, t: float, iter_: int) -> np.ndarray:
        """rk_euler(U,t,iter,nk) on a host array, in place (rk.f90:12)."""
        self._rc(self.lib.ns_rk_euler(self._ctx, self._host(U, True), float(t), int(iter_),
                                      self.case.nk))
        return U

    def run(self, U0: np.ndarray, iter0: int, nsteps: int) -> np.ndarray:
        self.set_state(np.ascontiguousarray(U0, dtype=np.float64))
        self.step(iter0, nsteps)
        return self.get_state()

    def probes(self, pi, pj) -> np.ndarray:
        """U(1..nk) at 1-based points (pi[q], pj[q]); shape (len(pi), nk)."""
        pi = np.ascontiguousarray(pi, dtype=np.int32)
        pj = np.ascontiguousarray(pj, dtype=np.int32)
        out = np.empty((len(pi), self.case.nk))
        self._rc(self.lib.ns_get_probes(self._ctx, len(pi), pi.ctypes.data, pj.ctypes.data,
                                        out.ctypes.data))
        return out

    def check_finite(self) -> int:
        n = C.c_int64(0)
        rc = self.lib.ns_check_finite(self._ctx, C.byref(n))
        if rc not in (L.NS_OK, L.NS_ERR_NONFINITE):
            self._rc(rc)
        return int(n.value)

    # -- introspection -------------------------------------------------------
    def launches_per_step(self) -> int:
        n = C.c_int()
        self._rc(self.lib.ns_step_launches(self._ctx, C.byref(n)))
        return n.value

    def filter_warmup(self) -> int:
        n = C.c_int()
        self._rc(self.lib.ns_filter_warmup(self._ctx, C.byref(n)))
        return n.value

    def state_device(self):
        ptr, pitch = C.c_void_p(), C.c_int64()
        self._rc(self.lib.ns_state_device(self._ctx, C.byref(ptr), C.byref(pitch)))
        return ptr.value, pitch.value

    def set_stream(self, stream_handle: int) -> None:
        self._rc(self.lib.ns_set_stream(self._ctx, C.c_void_p(stream_handle)))


class Batch:
    """Many independent Euler instances advanced together (ns_batch_*)."""

    def __init__(self, case_list, device: int = 0, precision: int = L.NS_PREC_FP64):
        self.lib = L.load()
        self.cases = list(case_list)
        self._keep = []
        ps = []
        for c in self.cases:
            p, keep = params_from_case(c, device=device, precision=precision)
            self._keep.append((p, keep))
            ps.append(p)
        arr = (C.c_void_p * len(ps))(*[C.addressof(p) for p in ps])
        h = C.c_void_p()
        L.check(self.lib.ns_batch_create(arr, len(ps), int(precision), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self.lib.ns_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _rc(self, rc):
        L.check(rc)

    def set_state(self, q: int, U: np.ndarray) -> None:
        c = self.cases[q]
        U = np.ascontiguousarray(U, dtype=np.float64)
        assert U.shape == (c.jmax, c.imax, 4)
        self._rc(self.lib.ns_batch_set_state(self._h, q, U.ctypes.data, L.NS_LAYOUT_FORTRAN))

    def get_state(self, q: int) -> np.ndarray:
        c = self.cases[q]
        out = np.empty((c.jmax, c.imax, 4))
        self._rc(self.lib.ns_batch_get_state(self._h, q, out.ctypes.data, L.NS_LAYOUT_FORTRAN))
        return out

    def set_initial(self) -> None:
        for q, c in enumerate(self.cases):
            self.set_state(q, c.U0)

    def step(self, iter0: int, nsteps: int = 1) -> None:
        self._rc(self.lib.ns_batch_step(self._h, int(iter0), int(nsteps)))

    def synchronize(self) -> None:
        self._rc(self.lib.ns_batch_synchronize(self._h))

    def set_stream(self, handle: int) -> None:
        self._rc(self.lib.ns_batch_set_stream(self._h, C.c_void_p(handle)))

    def autotune(self, iter0: int = 0, reps: int = 2):
        ty, bps, ms = C.c_int(), C.c_int(), C.c_double()
        self._rc(self.lib.ns_batch_autotune(self._h, iter0, reps, C.byref(ty), C.byref(bps),
                                            C.byref(ms)))
        return ty.value, bps.value, ms.value

    def phase_times(self, iter0: int = 0):
        """Advances one step with the phase stamps on: ms of phases A..D
        (tiles, x lines, y lines, edges) summed over the six stages."""
        ms = (C.c_double * 4)()
        self._rc(self.lib.ns_batch_phase_times(self._h, iter0, ms))
        return dict(zip(("tiles", "x_lines", "y_lines", "edges"), list(ms)))

    def info(self):
        g, ty, bps = C.c_int(), C.c_int(), C.c_int()
        items = (C.c_int * 4)()
        self._rc(self.lib.ns_batch_info(self._h, C.byref(g), C.byref(ty), C.byref(bps), items))
        return {"grid": g.value, "tile_rows": ty.value, "blocks_per_sm": bps.value,
                "items": list(items)}

    def barrier_test(self, extra: int = 1, spin_limit: int = 20000) -> int:
        return self.lib.ns_batch_barrier_test(self._h, extra, spin_limit)
