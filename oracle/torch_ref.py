"""Pure-PyTorch FP64 restatement of the Euler step -- TEST INFRASTRUCTURE ONLY.

A second, independent restatement of rk_euler (rk.f90:12-75) for the
inviscid case with nk = 4 (rho, u, v, p), written with differentiable torch
operations so that autograd gives the reference gradient the hand-written
discrete adjoint (navierstokes_gb300/csrc/ns_adjoint.cu) is checked
against.  It follows the same statements as ns_oracle.c: the DRP stencils
and closures of diff.f90:40-238 with the band metrics of diff.f90:276-350,
EULERNONLINEAR (eqeuler.f90:63-92, 1/Re = 0), rk_steep on the interior
(rk.f90:153-169), bufferxy (rk.f90:77-151), the in-place filter sweeps of
filtering.f90 (pass by pass, point by point), ccpml (cc.f90:6-68) and the
source s = sin(wf*(iter+c_k)*dt) * S (rk.f90:188-189).  Fields are
(4, jmax, imax) tensors.  Small grids only: the filter sweeps run as Python
loops over positions.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import coeffs

A = coeffs(0)
A4, A5, A6, A4B, A5B, A6B = (coeffs(k) for k in (1, 2, 3, 4, 5, 6))
DF = coeffs(7)          # df(-6..6)
DFBX, DFBY = coeffs(8), coeffs(9)
ALPHA, BETA, CT = coeffs(10), coeffs(11), coeffs(12)


def _deriv_last(F, h, mult):
    """d/d(last axis) with closures, times the per-position multiplier."""
    n = F.shape[-1]
    closure = lambda c, q, o0: (sum(c[z] * F[..., q + o0 + z] for z in range(7)) / h)[..., None]
    inner = sum(A[s - 1] * (F[..., 3 + s:n - 3 + s] - F[..., 3 - s:n - 3 - s])
                for s in (1, 2, 3)) / h
    out = torch.cat([closure(A6, 0, 0), closure(A5, 1, -1), closure(A4, 2, -2), inner,
                     closure(A4B, n - 3, -4), closure(A5B, n - 2, -5), closure(A6B, n - 1, -6)],
                    dim=-1)
    return out * mult


def deriv_x(F, P):
    return _deriv_last(F, P["dm"], P["mx"])


def deriv_y(F, P):
    return _deriv_last(F.transpose(-1, -2), P["dn"], P["my"]).transpose(-1, -2)


def _filter_last(F, sigmaf, dfb):
    """The three in-place sweeps of lddfilterx along the last axis."""
    n = F.shape[-1]
    u = list(F.unbind(-1))
    for q in range(1, 7):
        Du = sum(dfb[s + 1] * u[q + s] for s in range(-1, 6))
        u[q] = u[q] - sigmaf * Du
    for q in range(6, n - 6):
        Du = sum(DF[s + 6] * u[q + s] for s in range(-6, 7))
        u[q] = u[q] - sigmaf * Du
    for q in range(n - 2, n - 8, -1):
        Du = sum(dfb[s + 1] * u[q - s] for s in range(-1, 6))
        u[q] = u[q] - sigmaf * Du
    return torch.stack(u, dim=-1)


def filter_x(F, P):
    return _filter_last(F, P["sigmaf"], DFBX)


def filter_y(F, P):
    return _filter_last(F.transpose(-1, -2), P["sigmaf"], DFBY).transpose(-1, -2)


def rhs(U, S, sin_k, P):
    rho, u, v, p = U[0], U[1], U[2], U[3]
    Ux, Uy = deriv_x(U, P), deriv_y(U, P)
    g = P["gamma"]
    r0 = -(u * Ux[0] + rho * Ux[1] + v * Uy[0] + rho * Uy[2])
    r1 = -(u * Ux[1] + 1.0 / rho * Ux[3] + v * Uy[1])
    r2 = -(u * Ux[2] + v * Uy[2] + 1.0 / rho * Uy[3])
    r3 = -(g * p * Ux[1] + u * Ux[3] + g * p * Uy[2] + v * Uy[3] - sin_k * S)
    return torch.stack([r0, r1, r2, r3])


def bc(U, P):
    g = P["gamma"]
    rho, u, v, p = (x.clone() for x in U.unbind(0))
    ni, nj = rho.shape[1], rho.shape[0]
    # left (cc.f90:23-27), right (:32-36), top (:39-43), bottom (:55-59)
    rho = torch.cat([P["rhob"][:, None], rho[:, 1:]], dim=1)
    u = torch.cat([(2 * u[:, 1] - u[:, 2])[:, None], u[:, 1:]], dim=1)
    v = torch.cat([torch.zeros_like(v[:, :1]), v[:, 1:]], dim=1)
    p = torch.cat([torch.full_like(p[:, :1], 1.0 / g), p[:, 1:]], dim=1)
    ext = lambda f: torch.cat([f[:, :-1], (2 * f[:, -2] - f[:, -3])[:, None]], dim=1)
    rho, u, v = ext(rho), ext(u), ext(v)
    p = torch.cat([p[:, :-1], torch.full_like(p[:, :1], 1.0 / g)], dim=1)
    top = lambda f: torch.cat([f[:-1], (2 * f[-2] - f[-3])[None]], dim=0)
    rho, u, v = top(rho), top(u), top(v)
    p = torch.cat([p[:-1], torch.full_like(p[:1], 1.0 / g)], dim=0)
    bot = lambda f: torch.cat([(2 * f[1] - f[2])[None], f[1:]], dim=0)
    rho, u, v = bot(rho), bot(u), bot(v)
    p = torch.cat([torch.full_like(p[:1], 1.0 / g), p[1:]], dim=0)
    return torch.stack([rho, u, v, p])


def buffer(U, P):
    return P["Ub"] + P["sxy"] * (U - P["Ub"])


def step(U, S, it, P):
    w = torch.zeros_like(U)
    mask = P["interior"]
    for k in range(6):
        sin_k = math.sin(P["wf"] * ((it + CT[k]) * P["dt"]))
        R = rhs(U, S, sin_k, P)
        w = torch.where(mask, ALPHA[k] * w + P["dt"] * R, w)
        U = torch.where(mask, U + BETA[k] * w, U)
        U = buffer(U, P)
        U = filter_x(U, P)
        U = filter_y(U, P)
        U = bc(U, P)
    return U


def params(case, device="cpu"):
    """Tensors of a Case (nk = 4, inviscid, band metrics) for step()."""
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=device)
    D, imax, jmax = case.D, case.imax, case.jmax
    mx = np.where((np.arange(imax) < D) | (np.arange(imax) >= imax - D), case.meshx, 1.0)
    my = np.where((np.arange(jmax) < D) | (np.arange(jmax) >= jmax - D), case.meshy, 1.0)
    sx = np.where((np.arange(imax) < D) | (np.arange(imax) >= imax - D), case.sigmax, 1.0)
    sy = np.where((np.arange(jmax) < D) | (np.arange(jmax) >= jmax - D), case.sigmay, 1.0)
    interior = np.zeros((jmax, imax), dtype=bool)
    interior[1:-1, 1:-1] = True
    return {"dm": case.dm, "dn": case.dn, "mx": t(mx), "my": t(my), "gamma": case.gamma,
            "sigmaf": case.sigmaf, "dt": case.dt, "wf": case.wf,
            "Ub": t(np.moveaxis(case.Ub, 2, 0)), "sxy": t(sy[:, None] * sx[None, :]),
            "rhob": t(case.rhob), "interior": torch.as_tensor(interior, device=device)}


def observer_loss(U, obs_x, obs_y, case, pb):
    """sum_m p'(x_m, y_m)^2, bilinear."""
    tot = 0.0
    for x, y in zip(obs_x, obs_y):
        fx, fy = (x - case.m[0]) / case.dm, (y - case.n[0]) / case.dn
        i0, j0 = int(math.floor(fx)), int(math.floor(fy))
        wx, wy = fx - i0, fy - j0
        p = U[3] - pb
        v = ((1 - wx) * (1 - wy) * p[j0, i0] + wx * (1 - wy) * p[j0, i0 + 1] +
             (1 - wx) * wy * p[j0 + 1, i0] + wx * wy * p[j0 + 1, i0 + 1])
        tot = tot + v * v
    return tot


def loss_and_grad(case, S, obs_x, obs_y, nsteps, iter0=0):
    """Loss and dLoss/dS by autograd through nsteps reference steps."""
    P = params(case)
    St = torch.tensor(np.ascontiguousarray(S), dtype=torch.float64, requires_grad=True)
    U = torch.as_tensor(np.moveaxis(case.U0, 2, 0).copy(), dtype=torch.float64)
    pb = float(case.Ub[0, 0, 3])
    L = 0.0
    for n in range(nsteps):
        U = step(U, St, iter0 + n, P)
        L = L + observer_loss(U, obs_x, obs_y, case, pb)
    L.backward()
    return float(L.detach()), St.grad.numpy().copy(), np.moveaxis(U.detach().numpy(), 0, 2)
