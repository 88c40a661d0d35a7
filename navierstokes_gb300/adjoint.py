"""Gradient of an acoustic observer loss with respect to a source field,
through the hand-written discrete adjoint of the FP64 Euler step
(ns_adjoint_*, include/ns_gb300.h), exposed as a torch.autograd.Function.

The workload: 2-D Euler on a uniform grid with a mean flow along x; the
source of rk.f90:188-189 is s = sin(wf*(iter+c_k)*dt) * S(i,j), where the
field S is a Gaussian monopole envelope exp(-ln2*r^2/b^2) (b = 32 cells,
at the grid centre) times an amplitude A(i,j) interpolated bicubically
(Keys cubic convolution, a = -0.5) from a 16x16 grid of control values.
Loss: the sum over steps of p'^2 at observers equally spaced on a circle,
p' interpolated bilinearly from the four surrounding grid points.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from .cases import Case, params_from_case, uniform_flow_case


def keys_weights(t: np.ndarray):
    """Keys cubic convolution (a = -0.5) weights for offsets -1, 0, 1, 2."""
    a = -0.5

    def k(x):
        x = np.abs(x)
        return np.where(x <= 1, (a + 2) * x ** 3 - (a + 3) * x ** 2 + 1,
                        np.where(x < 2, a * x ** 3 - 5 * a * x ** 2 + 8 * a * x - 4 * a, 0.0))
    return np.stack([k(t + 1), k(t), k(t - 1), k(t - 2)], axis=-1)


def cubic_basis(n: int, nc: int) -> np.ndarray:
    """B (n x nc): value at grid index i of the cubic interpolant of control
    node c; nodes at i = c*(n-1)/(nc-1), indices clamped at the ends."""
    B = np.zeros((n, nc))
    pos = np.arange(n) * (nc - 1) / (n - 1)
    base = np.floor(pos).astype(int)
    t = pos - base
    w = keys_weights(t)
    for off in range(4):
        idx = np.clip(base - 1 + off, 0, nc - 1)
        np.add.at(B, (np.arange(n), idx), w[:, off])
    return B


class SourceProblem:
    """The source problem: the case, the control basis and the observers."""

    def __init__(self, n=512, nc=16, mach=0.3, omega=0.5, steps=2000, radius=150.0, nobs=32,
                 envelope_cells=32.0, D=30, sigmaf=0.2, seed=0, control_std=1e-3):
        c = uniform_flow_case(imax=n, jmax=n, mach=mach, D=D, sigmaf=sigmaf, pulse_amp=0.0,
                              vortex_eps=0.0, steps=steps)
        c.name = f"adjoint_{n}x{n}"
        c.source_mode = L.NS_SRC_FIELD
        c.wf = omega
        self.case: Case = c
        self.steps = steps
        X, Y = np.meshgrid(c.m, c.n)
        self.env = np.exp(-math.log(2.0) * (X ** 2 + Y ** 2) / envelope_cells ** 2)
        self.Bx = cubic_basis(c.imax, nc)
        self.By = cubic_basis(c.jmax, nc)
        rng = np.random.default_rng(seed)
        self.controls = rng.normal(0.0, control_std, (nc, nc))
        th = 2 * np.pi * np.arange(nobs) / nobs
        self.obs_x = radius * np.cos(th)
        self.obs_y = radius * np.sin(th)
        c.src_field = self.field(self.controls)

    def field(self, controls: np.ndarray) -> np.ndarray:
        """S = envelope * (By @ controls @ Bx^T), shape (jmax, imax)."""
        return self.env * (self.By @ np.asarray(controls) @ self.Bx.T)

    def controls_grad(self, grad_field: np.ndarray) -> np.ndarray:
        return self.By.T @ (self.env * grad_field) @ self.Bx


class Adjoint:
    """ns_adjoint_* wrapper.  checkpoint_every = 0 keeps every stage's input
    state when device memory allows (the reverse pass then recomputes only
    first derivatives), else checkpoints every 100 steps."""

    def __init__(self, problem: SourceProblem, checkpoint_every=100, device=0):
        self.lib = L.load()
        self.problem = problem
        c = problem.case
        p, self._keep = params_from_case(c, device=device)
        h = C.c_void_p()
        ox = np.ascontiguousarray(problem.obs_x)
        oy = np.ascontiguousarray(problem.obs_y)
        L.check(self.lib.ns_adjoint_create(C.byref(p), len(ox), ox.ctypes.data, oy.ctypes.data,
                                           int(checkpoint_every), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self.lib.ns_adjoint_destroy(self._h)
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

    def set_field(self, field: np.ndarray):
        f = np.ascontiguousarray(field, dtype=np.float64)
        L.check(self.lib.ns_adjoint_set_source(self._h, f.ctypes.data))

    def forward(self, nsteps=None, iter0=0) -> float:
        c = self.problem.case
        U0 = np.ascontiguousarray(c.U0)
        loss = C.c_double()
        L.check(self.lib.ns_adjoint_forward(self._h, U0.ctypes.data, L.NS_LAYOUT_FORTRAN,
                                            int(iter0), int(nsteps or self.problem.steps),
                                            C.byref(loss)))
        return loss.value

    def stored_bytes(self) -> int:
        """Bytes of stage inputs the last forward pass kept (0: checkpoints)."""
        b = C.c_int64()
        L.check(self.lib.ns_adjoint_stored_bytes(self._h, C.byref(b)))
        return b.value

    def backward(self) -> np.ndarray:
        c = self.problem.case
        g = np.empty((c.jmax, c.imax))
        L.check(self.lib.ns_adjoint_backward(self._h, g.ctypes.data))
        return g

    def loss_and_grad(self, controls, nsteps=None):
        self.set_field(self.problem.field(controls))
        loss = self.forward(nsteps)
        return loss, self.problem.controls_grad(self.backward())


def source_loss_function():
    """torch.autograd.Function: controls (16x16, FP64) -> loss, whose
    backward runs the discrete adjoint."""
    import torch

    class SourceLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, controls, adj: Adjoint, nsteps: int):
            c = controls.detach().cpu().numpy()
            adj.set_field(adj.problem.field(c))
            loss = adj.forward(nsteps)
            ctx.adj = adj
            ctx.device = controls.device
            return torch.tensor(loss, dtype=torch.float64, device=controls.device)

        @staticmethod
        def backward(ctx, grad_out):
            g = ctx.adj.problem.controls_grad(ctx.adj.backward())
            gt = torch.from_numpy(g).to(ctx.device) * grad_out
            return gt, None, None

    return SourceLoss
