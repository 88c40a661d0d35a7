"""Parity metrics shared by the GPU tests, smoke() and bench.py.

The bar for the plain FP64 path: for every variable k,
    max|q_gpu - q_oracle| / S_k <= 1e-12
after N steps, where S_k = max|q_k| for rho, p and psi, and for the velocity
components u, v the characteristic speed of the state, S = max(|u|,|v|) + c,
c = sqrt(gamma*p/rho).  Velocities need a velocity scale: v is a pure
perturbation in every case of the reference (its base flow is 0,
init.f90:386), and its rounding floor is set by p and rho (one ulp of an
O(1) value), not by its own amplitude.  The stricter figure relative to the
perturbation of each variable,
    max|q_gpu - q_oracle| / max|q_oracle - q_base|,
is reported beside it.
"""
from __future__ import annotations

import numpy as np

TOL_FP64 = 1e-12
GAMMA = 1.4


def scales(ref: np.ndarray, gamma: float = GAMMA):
    nk = ref.shape[-1]
    s = [float(np.max(np.abs(ref[..., k]))) for k in range(nk)]
    c = np.sqrt(gamma * np.abs(ref[..., 3]) / np.abs(ref[..., 0]))
    speed = float(np.max(np.maximum(np.abs(ref[..., 1]), np.abs(ref[..., 2])) + c))
    s[1] = s[2] = speed
    return s


def rel_errors(got: np.ndarray, ref: np.ndarray, base: np.ndarray | None = None):
    """Per variable (relative to its scale, relative to its perturbation)."""
    nk = ref.shape[-1]
    sc = scales(ref)
    out = []
    for k in range(nk):
        d = float(np.max(np.abs(got[..., k] - ref[..., k])))
        rel = d / sc[k] if sc[k] > 0 else d
        if base is not None:
            pert = float(np.max(np.abs(ref[..., k] - base[..., k])))
            relp = d / pert if pert > 0 else (0.0 if d == 0 else float("inf"))
        else:
            relp = float("nan")
        out.append((rel, relp))
    return out


def assert_parity(got, ref, base=None, tol=TOL_FP64, label=""):
    assert np.all(np.isfinite(got)), f"{label}: non-finite values in the GPU state"
    errs = rel_errors(got, ref, base)
    worst = max(e[0] for e in errs)
    assert worst <= tol, f"{label}: max relative error {worst:.3e} > {tol:.1e}; per variable {errs}"
    return errs
