"""Split precision (FP64 base flow + FP32 perturbation, the velocity
perturbation as hi + lo FP32 pairs) against the plain FP64 path on the GPU,
measured on the pressure perturbation p' = p - p_b: relative L2 and max
error <= 1e-5 against the FP64 run, for acoustic cases and for the 1e-3
vortex beside the 1e-4 pulse (whose FP32-only velocity had left p' about
ten ulps of the vortex off)."""
import numpy as np
import pytest

from navierstokes_gb300 import _lib as L
from navierstokes_gb300 import cases

pytestmark = pytest.mark.gpu
TOL_PPRIME = 1e-5


def p_errors(split, ref, base):
    dp = split[..., 3] - ref[..., 3]
    pr = ref[..., 3] - base[..., 3]
    l2 = float(np.linalg.norm(dp) / np.linalg.norm(pr))
    mx = float(np.max(np.abs(dp)) / np.max(np.abs(pr)))
    return l2, mx


def run(case, nsteps, precision, iter0=0):
    from navierstokes_gb300 import Solver
    with Solver(case, precision=precision) as s:
        return s.run(case.U0, iter0, nsteps)


@pytest.mark.parametrize("mach", [0.0, 0.5])
def test_split_matches_fp64_pulse(nslib, mach):
    c = cases.uniform_flow_case(imax=600, jmax=480, mach=mach, vortex_eps=0.0, steps=300)
    ref = run(c, 300, L.NS_PREC_FP64)
    got = run(c, 300, L.NS_PREC_SPLIT)
    l2, mx = p_errors(got, ref, c.Ub)
    print(f"pulse, mach {mach}: p' rel L2 {l2:.2e} max {mx:.2e}")
    assert l2 <= TOL_PPRIME and mx <= TOL_PPRIME


@pytest.mark.parametrize("mach", [0.0, 0.5])
def test_split_pulse_and_vortex(nslib, mach):
    c = cases.uniform_flow_case(imax=600, jmax=480, mach=mach, vortex_upstream=100, steps=300)
    ref = run(c, 300, L.NS_PREC_FP64)
    got = run(c, 300, L.NS_PREC_SPLIT)
    l2, mx = p_errors(got, ref, c.Ub)
    qmax = max(np.max(np.abs(c.U0[..., k] - c.Ub[..., k])) for k in range(4))
    ulp = 2.0 ** -24 * qmax
    du = [float(np.max(np.abs(got[..., k] - ref[..., k])) / ulp) for k in range(4)]
    print(f"pulse+vortex, mach {mach}: p' rel L2 {l2:.2e} max {mx:.2e}; "
          f"max error in FP32 ulps of the largest perturbation {du}")
    assert l2 <= TOL_PPRIME and mx <= TOL_PPRIME
    for k in range(4):
        assert du[k] <= 50.0


@pytest.mark.parametrize("vortex", [0.0, 1e-3])
def test_split32_every_perturbation_fp32(nslib, vortex):
    """NS_PREC_SPLIT32 stores every perturbation as one FP32 number: within
    1e-5 for the acoustic pulse; next to the 1e-3 vortex the FP32 storage
    noise of u' drives p' to about 1e-4 (the reason NS_PREC_SPLIT pairs u',
    v', p')."""
    c = cases.uniform_flow_case(imax=600, jmax=480, mach=0.5, vortex_eps=vortex,
                                vortex_upstream=100, steps=300)
    ref = run(c, 300, L.NS_PREC_FP64)
    got = run(c, 300, L.NS_PREC_SPLIT32)
    l2, mx = p_errors(got, ref, c.Ub)
    print(f"split32, vortex {vortex}: p' rel L2 {l2:.2e} max {mx:.2e}")
    if vortex == 0.0:
        assert l2 <= TOL_PPRIME and mx <= TOL_PPRIME
    else:
        assert l2 <= 2e-4 and mx <= 5e-4


@pytest.mark.slow
def test_split_4096_squared_1000_steps(nslib):
    """The split-precision workload at full size: 4096x4096 Euler at M = 0.5,
    pulse 1e-4 and vortex 1e-3, NS_PREC_SPLIT against the FP64 path on the
    same GPU; p' relative L2 and max error <= 1e-5 at steps 100, 500 and
    1000, and within half of that: the margin that the FP64 product
    beta*dt in the accumulator update and the float-float base-flow
    advection give (3.9e-6 at step 1000; an FP32 dt*R and FP32 advection
    left 9.0e-6)."""
    from navierstokes_gb300 import Solver
    c = cases.uniform_flow_case()
    assert (c.imax, c.jmax, c.steps) == (4096, 4096, 1000)
    marks = (100, 500, 1000)
    snaps = {}
    for prec in (L.NS_PREC_FP64, L.NS_PREC_SPLIT):
        with Solver(c, precision=prec) as s:
            s.set_state(c.U0)
            done = 0
            for n in marks:
                s.step(done, n - done)
                done = n
                snaps[prec, n] = s.get_state()
    for n in marks:
        l2, mx = p_errors(snaps[L.NS_PREC_SPLIT, n], snaps[L.NS_PREC_FP64, n], c.Ub)
        print(f"4096^2 split, step {n}: p' rel L2 {l2:.2e} max {mx:.2e}")
        assert l2 <= TOL_PPRIME / 2 and mx <= TOL_PPRIME / 2, (n, l2, mx)


def test_split_with_source_and_chunked_filters(nslib):
    c = cases.uniform_flow_case(imax=1500, jmax=1100, mach=0.3, pulse_amp=0.0, vortex_eps=0.0,
                                steps=80)
    c.source_mode = L.NS_SRC_GAUSSIAN
    c.amplitude, c.wf, c.m_pt, c.n_pt, c.r0 = 1e-3, 0.6, 0.0, 0.0, 3.0
    ref = run(c, 80, L.NS_PREC_FP64, iter0=5)
    got = run(c, 80, L.NS_PREC_SPLIT, iter0=5)
    l2, mx = p_errors(got, ref, c.Ub)
    print(f"source: p' rel L2 {l2:.2e} max {mx:.2e}")
    assert l2 <= TOL_PPRIME and mx <= TOL_PPRIME


def test_split_uniform_state_drift_matches_fp64(nslib):
    """The REAL(4) y boundary filter moves a uniform state (its coefficients
    sum to -8.4e-9); the split path adds that FP64 action on the base flow
    back, so its drift matches the FP64 path's."""
    c = cases.uniform_flow_case(imax=300, jmax=260, pulse_amp=0.0, vortex_eps=0.0)
    c.U0 = c.Ub.copy()
    ref = run(c, 20, L.NS_PREC_FP64)
    got = run(c, 20, L.NS_PREC_SPLIT)
    drift = np.max(np.abs(ref - c.Ub))
    assert drift > 1e-9
    assert np.max(np.abs(got - ref)) <= 1e-3 * drift


def test_split_rk_euler_and_probes(nslib):
    from navierstokes_gb300 import Solver
    c = cases.uniform_flow_case(imax=128, jmax=96, vortex_upstream=30, steps=5)
    U = c.U0.copy()
    with Solver(c, precision=L.NS_PREC_SPLIT) as s:
        for it in range(3):
            s.rk_euler(U, 0.0, it)
        res = s.run(c.U0, 0, 3)
        pr = s.probes([64], [48])
    # the host round trip U = Ub + q' -> q' = f32(U - Ub) loses the low bits
    # of tiny q' (below 2^-52 |Ub|) at every call; the two paths agree to
    # well below the FP32 resolution of the perturbation
    print("rk_euler vs resident max diff", np.max(np.abs(U - res)))
    np.testing.assert_allclose(U, res, rtol=0, atol=1e-11)
    np.testing.assert_array_equal(pr[0], res[47, 63])


def test_split_sheared_mean_flow(nslib):
    """A base flow that varies in y (the reference's mixing layer, Euler,
    with its acoustic source): the y-derivatives of the base flow enter the
    perturbation equations as FP64-computed per-row terms."""
    c = cases.mixing_layer_case(imax=200, jmax=160, nk=4, D=24)
    c.inviscid = True
    ref = run(c, 40, L.NS_PREC_FP64)
    got = run(c, 40, L.NS_PREC_SPLIT)
    l2, mx = p_errors(got, ref, c.Ub)
    print(f"mixing layer: p' rel L2 {l2:.2e} max {mx:.2e}")
    assert l2 <= TOL_PPRIME and mx <= TOL_PPRIME


def test_split_navier_stokes_stretched(nslib):
    """Navier-Stokes on the y-stretched grid (the 4096x2048 workload's flow,
    pulse and 0.1 vortex, at 512x256): the viscous stresses and heat flux of
    the perturbation in FP32 (k_split_visc, T' formed without cancellation),
    their divergence in the stage kernel, the metric in every y derivative;
    p' within 1e-5 of the FP64 path after 100 steps."""
    c = cases.stretched_ns_case(imax=512, jmax=256, D=20, vortex_upstream=60)
    assert not c.inviscid
    ref = run(c, 100, L.NS_PREC_FP64)
    got = run(c, 100, L.NS_PREC_SPLIT)
    l2, mx = p_errors(got, ref, c.Ub)
    # the viscous terms matter: the Euler split path lands far from the
    # Navier-Stokes FP64 run
    e = cases.stretched_ns_case(imax=512, jmax=256, D=20, vortex_upstream=60)
    e.inviscid = True
    euler = run(e, 100, L.NS_PREC_SPLIT)
    l2e, mxe = p_errors(euler, ref, c.Ub)
    print(f"split Navier-Stokes: p' rel L2 {l2:.2e} max {mx:.2e}; "
          f"inviscid split against it: {l2e:.2e} / {mxe:.2e}")
    assert l2 <= TOL_PPRIME and mx <= TOL_PPRIME
    assert mxe > 100 * mx


def test_split_rejects_unsupported(nslib):
    from navierstokes_gb300 import Solver
    m = cases.mixing_layer_case(imax=64, jmax=48, nk=4, D=8)   # viscous, sheared base flow
    with pytest.raises(L.NsError) as e:
        Solver(m, precision=L.NS_PREC_SPLIT)
    assert e.value.code == L.NS_ERR_UNSUPPORTED
    m5 = cases.mixing_layer_case(imax=64, jmax=48, nk=5, D=8)  # the passive scalar
    with pytest.raises(L.NsError) as e:
        Solver(m5, precision=L.NS_PREC_SPLIT)
    assert e.value.code == L.NS_ERR_UNSUPPORTED
    u = cases.uniform_flow_case(imax=64, jmax=48, D=8, vortex_upstream=10)
    u.Ub[:, :, 2] = 1e-3                              # base flow with v != 0
    with pytest.raises(L.NsError) as e:
        Solver(u, precision=L.NS_PREC_SPLIT)
    assert e.value.code == L.NS_ERR_UNSUPPORTED
