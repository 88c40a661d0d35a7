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


def test_transport_table(nslib):
    """mu(T), k(T) as the first-derivative kernel evaluates them: the
    piecewise-polynomial table over T in [1/4, 8), exp and log outside it,
    against the law evaluated in extended precision."""
    from navierstokes_gb300.cases import N2_FIT, acoustic_pulse_case
    from navierstokes_gb300.solver import Solver

    if np.finfo(np.longdouble).eps > 1e-18:
        pytest.skip("numpy long double is not wider than double here")
    case = acoustic_pulse_case(imax=32, jmax=32, nk=4, D=8, inviscid=False)
    rng = np.random.default_rng(5)
    inside = np.concatenate([rng.uniform(0.25, 8.0, 20000), 2.0 ** rng.uniform(-2, 3, 20000),
                             [0.25, 0.5, 1.0, 2.0, 4.0, np.nextafter(8.0, 0.0),
                              np.nextafter(0.25, 1.0), 1.0 + 2.0 ** -44]])
    outside = np.array([0.1, 0.2, np.nextafter(0.25, 0.0), 8.0, 20.0, 0.05, 300.0])
    T = np.ascontiguousarray(np.concatenate([inside, outside]))
    mu, k = np.empty_like(T), np.empty_like(T)
    with Solver(case) as s:
        assert nslib.ns_transport_eval(s._ctx, T.ctypes.data, mu.ctypes.data, k.ctypes.data,
                                       len(T)) == 0
    ld = np.longdouble

    def law(A, B, C_, D):
        """exp(arg) and arg = g(Tref T) - g(Tref)"""
        def g(x):
            return ld(A) * np.log(x) + ld(B) / x + ld(C_) / (x * x) + ld(D)
        arg = g(ld(case.Tref) * T.astype(ld)) - g(ld(case.Tref))
        return np.exp(arg), np.abs(arg).astype(np.float64)

    f = N2_FIT
    n = len(inside)
    for got, (ref, arg) in ((mu, law(f["A_mi"], f["B_mi"], f["C_mi"], f["D_mi"])),
                            (k, law(f["A_k"], f["B_k"], f["C_k"], f["D_k"]))):
        rel = np.abs((got.astype(ld) - ref) / ref).astype(np.float64)
        assert rel[:n].max() <= 3e-16          # table: about 2 ulp
        # exp/log path: the rounding of the exponent argument (about
        # 1.1e-16 |arg| absolute) becomes relative error of exp, plus a few ulp
        assert np.all(rel[n:] <= 2.2e-16 * (4.0 + arg[n:]))
