"""The transport law's exp, log and 1/x (ns_fastmath.cuh), written from
Tang's table-driven method, against correctly rounded values (200-bit
mpmath, tests/golden/make_fastmath_ref.py) and the library's special-value
behaviour (GPU)."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ev(lib, fn, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    assert lib.ns_math_eval(fn, x.ctypes.data, y.ctypes.data, len(x), 0) == 0
    return y


def ulps(got, ref):
    return np.abs(got - ref) / np.spacing(np.abs(ref))


REF = Path(__file__).parent / "golden" / "fastmath_ref.npz"   # make_fastmath_ref.py


def test_exp(nslib):
    r = np.load(REF)
    assert ulps(ev(nslib, 0, r["xe"]), r["exp"]).max() <= 2.0


def test_log_and_reciprocal(nslib):
    r = np.load(REF)
    x, ref = r["xl"], r["log"]
    lg, rc = ev(nslib, 1, x), ev(nslib, 2, x)
    big = np.abs(ref) >= 1.0
    assert ulps(lg[big], ref[big]).max() <= 2.0
    assert np.abs(lg[~big] - ref[~big]).max() <= 4e-16      # absolute near log x = 0
    assert ulps(rc, r["rcp"]).max() <= 2.0


def test_special_values_follow_the_library(nslib):
    x = np.array([np.nan, np.inf, -np.inf, 1000.0, -1000.0, 710.0, -720.0])
    with np.errstate(over="ignore", under="ignore"):
        want = np.exp(x)
    got = ev(nslib, 0, x)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    assert np.allclose(got[ok], want[ok], rtol=1e-15, atol=0.0)
    x = np.array([0.0, -0.0, -1.0, np.inf, np.nan, 5e-324, 1e-310, 1e308])
    with np.errstate(divide="ignore", invalid="ignore"):
        wl, wr = np.log(x), 1.0 / x
    gl, gr = ev(nslib, 1, x), ev(nslib, 2, x)
    for g, w in ((gl, wl), (gr, wr)):
        assert np.array_equal(np.isnan(g), np.isnan(w))
        ok = ~np.isnan(w)
        assert np.allclose(g[ok], w[ok], rtol=1e-15, atol=0.0)
