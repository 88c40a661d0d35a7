"""The piecewise-polynomial table of the transport law mu(T), k(T)
(coefficients.f90:27-59, divided by mu0 and k0) that viscous contexts use,
built on the host (no GPU) and evaluated here in extended precision against
the law itself."""
import numpy as np
import pytest

from navierstokes_gb300 import _lib as L
from navierstokes_gb300.cases import N2_FIT

TREF = 273.15


def table(nslib):
    out = np.empty(L.NS_TRANSPORT_TABLE_DOUBLES)
    mu = np.array([N2_FIT[k] for k in ("A_mi", "B_mi", "C_mi", "D_mi")])
    kk = np.array([N2_FIT[k] for k in ("A_k", "B_k", "C_k", "D_k")])
    assert nslib.ns_transport_table(TREF, mu.ctypes.data, kk.ctypes.data, out.ctypes.data) == 0
    return out.reshape(5 * 256, 2, 6), mu, kk


def law(fit, T):
    ld = np.longdouble

    def g(x):
        return ld(fit[0]) * np.log(x) + ld(fit[1]) / x + ld(fit[2]) / (x * x) + ld(fit[3])
    return np.exp(g(ld(TREF) * T.astype(ld)) - g(ld(TREF)))


def pieces(T):
    e = np.floor(np.log2(T)).astype(int)
    m = T / np.exp2(e)
    j = np.floor((m - 1.0) * 256).astype(int)
    t0 = np.exp2(e) * (1.0 + j / 256.0)
    return (e + 2) * 256 + j, T - t0


def test_table_interpolates_the_law(nslib):
    if np.finfo(np.longdouble).eps > 1e-18:
        pytest.skip("numpy long double is not wider than double here")
    tab, mu, kk = table(nslib)
    rng = np.random.default_rng(3)
    T = np.concatenate([2.0 ** rng.uniform(-2, 3, 50000), [0.25, 1.0, 7.999]])
    p, u = pieces(T)
    ul = u.astype(np.longdouble)
    for f, fit in ((0, mu), (1, kk)):
        c = tab[p, f].astype(np.longdouble)
        val = c[:, 5]
        for q in range(4, -1, -1):
            val = val * ul + c[:, q]
        rel = np.abs((val - law(fit, T)) / law(fit, T)).astype(np.float64)
        # coefficients rounded to double; interpolation error far below
        assert rel.max() <= 1.5e-16, (f, rel.max())


def test_table_rejects_bad_arguments(nslib):
    out = np.empty(L.NS_TRANSPORT_TABLE_DOUBLES)
    fit = np.zeros(4)
    assert nslib.ns_transport_table(0.0, fit.ctypes.data, fit.ctypes.data,
                                    out.ctypes.data) == L.NS_ERR_PARAM
    assert nslib.ns_transport_table(TREF, None, fit.ctypes.data, out.ctypes.data) == L.NS_ERR_PARAM
