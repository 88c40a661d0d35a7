"""Parity metrics shared by the GPU tests, smoke() and bench.py.

The bar for the plain FP64 path: for every variable k,
    max|q_gpu - q_oracle| / max|q_oracle| <= 1e-12
after N steps.  The stricter figure relative to the perturbation,
    max|q_gpu - q_oracle| / max|q_oracle - q_base|,
is reported beside it.
"""
from __future__ import annotations

import numpy as np

TOL_FP64 = 1e-12


def rel_errors(got: np.ndarray, ref: np.ndarray, base: np.ndarray | None = None):
    """Per-variable (rel_to_max, rel_to_perturbation) of arrays (jmax, imax, nk)."""
    nk = ref.shape[-1]
    out = []
    for k in range(nk):
        d = float(np.max(np.abs(got[..., k] - ref[..., k])))
        scale = float(np.max(np.abs(ref[..., k])))
        rel = d / scale if scale > 0 else d
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
