"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no tests, fixtures or golden vectors and cannot be
compiled here, so the oracle is pinned by facts derived from the reference's
own coefficient tables (init.f90:288-338, filtering.f90:25-66, :114-120,
rk.f90:27-46) and by exact invariants of its statements.
"""
import math

import numpy as np
import pytest

from navierstokes_gb300 import cases


def test_interior_drp_exact_to_degree_4(oracle_mod):
    a = oracle_mod.coeffs(0)
    s = np.arange(1, 4)
    # antisymmetric stencil sum_s a_s (f(x+s)-f(x-s)): moments of odd degree
    m1 = np.sum(a * 2 * s)
    m3 = np.sum(a * 2 * s ** 3)
    assert abs(m1 - 1.0) < 1e-11
    assert abs(m3) < 1e-10


@pytest.mark.parametrize("which,off0", [(1, -2), (2, -1), (3, 0), (4, -4), (5, -5), (6, -6)])
def test_closures_exact_to_degree_4(oracle_mod, which, off0):
    c = oracle_mod.coeffs(which)
    offs = off0 + np.arange(7)
    moments = [np.sum(c * offs.astype(float) ** p) for p in range(5)]
    assert abs(moments[0]) < 1e-8
    assert abs(moments[1] - 1.0) < 1e-7
    for p in (2, 3, 4):
        assert abs(moments[p]) < 5e-7


def test_selective_filter_response(oracle_mod):
    d = oracle_mod.coeffs(7)
    s = np.arange(-6, 7)
    assert abs(np.sum(d)) < 1e-15
    assert abs(np.sum(d * np.cos(np.pi * s)) - 1.0) < 1e-11
    np.testing.assert_array_equal(d, d[::-1])


@pytest.mark.parametrize("which", [8, 9])
def test_boundary_filter_moments(oracle_mod, which):
    b = oracle_mod.coeffs(which)
    s = np.arange(-1, 6)
    tol = 1e-11 if which == 8 else 5e-8
    assert abs(np.sum(b)) < tol
    assert abs(np.sum(b * s)) < tol * 10
    assert abs(np.sum(b * np.cos(np.pi * s)) - 1.0) < tol * 10


def test_y_boundary_filter_is_single_precision(oracle_mod):
    bx, by = oracle_mod.coeffs(8), oracle_mod.coeffs(9)
    np.testing.assert_array_equal(by, bx.astype(np.float32).astype(np.float64))
    assert np.max(np.abs(by - bx)) > 1e-10


def test_lddrk_amplification_polynomial(oracle_mod):
    alpha, beta, ct = oracle_mod.coeffs(10), oracle_mod.coeffs(11), oracle_mod.coeffs(12)
    # 2N-storage on y' = z*y: coefficients of the amplification polynomial
    P = np.polynomial.Polynomial
    y, w = P([1.0]), P([0.0])
    z = P([0.0, 1.0])
    for k in range(6):
        w = alpha[k] * w + z * y
        y = y + beta[k] * w
    c = y.coef
    for kk, fact in enumerate([1, 1, 2, 6, 24]):
        assert abs(c[kk] - 1.0 / fact) < 1e-11, (kk, c[kk])
    assert abs(c[5] - 0.0078568) < 1e-6
    assert abs(c[6] - 0.00096) < 1e-5
    # stage times c_k are the partial sums of the update weights
    cs = [0.0]
    yy, ww = 0.0, 0.0
    for k in range(5):
        ww = alpha[k] * ww + 1.0
        yy = yy + beta[k] * ww
        cs.append(yy)
    np.testing.assert_allclose(cs, ct, atol=1e-11)


def test_transport_reference_values(oracle_mod):
    mu0, k0 = oracle_mod.transport_ref(273.15)
    # mu(T=1) = k(T=1) = 1 by construction (nondimensionalised at Tref)
    mu, k = oracle_mod.transport(273.15, 1.0)
    assert abs(mu - 1.0) < 1e-14 and abs(k - 1.0) < 1e-14
    # Svehla N2 at 273.15 K: mu ~ 1.66e-4 poise*?, k ~ 2.4e-4 in the fit's units
    assert 1e-5 < mu0 < 1e3 and 1e-5 < k0 < 1e3
    mu2, k2 = oracle_mod.transport(273.15, 2.0)
    assert mu2 > 1.0 and k2 > 1.0      # gas viscosity and conductivity grow with T


def test_init_dados_matches_product_setup(oracle_mod):
    args = (131, 97, 20, -6.5, 19.5, -2.4, 2.4, 0.01, 20.0)
    for quirk in (True, False):
        a = oracle_mod.init_dados(*args, quirk_buffer=quirk)
        b = cases.init_dados(*args, quirk_buffer=quirk)
        for key in ("m", "n", "meshx", "meshy", "sigmax", "sigmay"):
            np.testing.assert_array_equal(a[key], b[key], err_msg=key)
        assert a["dm"] == b["dm"] and a["dn"] == b["dn"]
    q = oracle_mod.init_dados(*args, quirk_buffer=True)
    assert np.all(q["sigmax"][:20] == 0.0) and np.all(q["sigmay"][:20] == 0.0)
    # the damping profile falls to 0 at the outer edge (x = 1 in init.f90:179)
    assert np.all(q["sigmax"][-20:-1] > 0.0) and q["sigmax"][-1] == 0.0


def test_uniform_state_fixed_point_oracle(oracle_mod):
    """A uniform state is a fixed point except for the y boundary filter,
    whose REAL(4)-rounded coefficients (filtering.f90:114-120) sum to
    -8.4e-9 instead of 0: each stage moves a constant by at most
    6*sigma_f*|sum dfb_y|*max|U| near the top and bottom rows."""
    c = cases.acoustic_pulse_case(imax=40, jmax=33, nk=5, D=6, amp=0.0)
    c.Ub[:, :, 4] = 0.0
    c.psib[:] = 0.0
    U = c.Ub.copy()
    o = oracle_mod.Oracle(c)
    nsteps = 3
    o.run(U, 0, nsteps)
    eps = abs(np.sum(oracle_mod.coeffs(9)))
    assert 1e-9 < eps < 1e-8
    bound = nsteps * 6 * 6 * c.sigmaf * eps * np.abs(c.Ub[..., :4]).max()
    dev = np.abs(U[..., :4] - c.Ub[..., :4]).max()
    assert dev <= bound
    # the x boundary filter (REAL(8) coefficients) alone keeps it to rounding
    U2 = c.Ub.copy()
    F = o.filterx(U2)
    np.testing.assert_allclose(F[..., :4], c.Ub[..., :4], atol=1e-15, rtol=0)


def test_derivative_of_polynomial(oracle_mod):
    """deropm/deropn reproduce d/dx of a quartic (metric 1 away from bands)."""
    c = cases.acoustic_pulse_case(imax=30, jmax=26, nk=4, D=0)
    o = oracle_mod.Oracle(c)
    X, Y = np.meshgrid(c.m, c.n)
    F = np.zeros((c.jmax, c.imax, 4))
    F[..., 0] = 0.01 * X ** 4 + X ** 2 * Y
    F[..., 1] = Y ** 3
    dx, dy = o.deropm(F), o.deropn(F)
    np.testing.assert_allclose(dx[..., 0], 0.04 * X ** 3 + 2 * X * Y, atol=1e-4 * np.abs(F).max())
    np.testing.assert_allclose(dy[..., 1], 3 * Y ** 2, atol=1e-4 * np.abs(F).max())


def test_filter_annihilates_constants_and_damps_nyquist(oracle_mod):
    c = cases.acoustic_pulse_case(imax=40, jmax=30, nk=4, D=0, sigmaf=0.2)
    o = oracle_mod.Oracle(c)
    U = np.ones((c.jmax, c.imax, 4)) * 3.0
    np.testing.assert_allclose(o.filterx(U), U, atol=1e-14)
    np.testing.assert_allclose(o.filtery(U), U, atol=1e-14)
    i = np.arange(c.imax)
    U2 = np.zeros_like(U)
    U2[..., 0] = ((-1.0) ** i)[None, :]
    F = o.filterx(U2)
    # interior points of the odd-even mode are damped by (1 - sigma_f) per
    # application in the Jacobi limit; the in-place sweep damps no less
    assert np.max(np.abs(F[:, 20, 0])) < 1.0


def test_filter_sweep_is_sequential(oracle_mod):
    """The in-place sweep differs from a Jacobi application of the same
    stencil (filtering.f90:69-79 updates u(i) with already-filtered u(i-s))."""
    c = cases.acoustic_pulse_case(imax=40, jmax=20, nk=4, D=0, sigmaf=0.2)
    o = oracle_mod.Oracle(c)
    rng = np.random.default_rng(0)
    U = rng.standard_normal((c.jmax, c.imax, 4))
    F = o.filterx(U)
    d = oracle_mod.coeffs(7)
    j, i = 5, 20
    jac = U[j, i, 0] - 0.2 * np.dot(d, U[j, i - 6:i + 7, 0])
    seq = U[j, i, 0] - 0.2 * (np.dot(d[:6], F[j, i - 6:i, 0]) + np.dot(d[6:], U[j, i:i + 7, 0]))
    assert abs(F[j, i, 0] - seq) < 1e-13
    assert abs(F[j, i, 0] - jac) > 1e-6


@pytest.mark.parametrize("which", range(13))
def test_library_tables_equal_the_oracle(oracle_mod, nslib, which):
    """Every setup path of the library (single grid, batch, no-alloc) takes
    its DRP, filter and LDDRK tables from one header; those tables equal the
    oracle's restatement of init.f90, filtering.f90 and rk.f90 bit for bit."""
    out = np.zeros(16)
    n = nslib.ns_coef_table(which, out.ctypes.data)
    ref = oracle_mod.coeffs(which)
    assert n == len(ref)
    np.testing.assert_array_equal(out[:n], ref)
