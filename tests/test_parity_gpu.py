"""GPU parity of the FP64 stage loop against the CPU oracle (through the C ABI).

Cases cover every branch the reference has: Euler and Navier-Stokes, nk = 4
and 5 (the passive scalar), the acoustic source (Gaussian and field), the
band and stretched metrics, the buffer quirk on and off, tiny grids where
the derivative closures and the three filter passes overlap, and grids long
enough for the filters to run as chunked recurrences.
"""
import numpy as np
import pytest

from parity import TOL_FP64, assert_parity
from navierstokes_gb300 import _lib as L
from navierstokes_gb300 import cases

pytestmark = pytest.mark.gpu


def _run_both(oracle_mod, case, nsteps, iter0=0):
    from navierstokes_gb300 import Solver
    ref = case.U0.copy()
    ora = oracle_mod.Oracle(case)
    ora.run(ref, iter0, nsteps)
    ora.close()
    with Solver(case) as s:
        got = s.run(case.U0, iter0, nsteps)
    return got, ref


@pytest.mark.parametrize("imax,jmax,nk", [(13, 13, 5), (20, 17, 5), (32, 32, 4), (14, 29, 5)])
def test_tiny_grids_ns_source(oracle_mod, nslib, imax, jmax, nk):
    c = cases.mixing_layer_case(imax=imax, jmax=jmax, nk=nk, D=min(imax, jmax) // 4, dt=0.005,
                                mmin=-2.0, mmax=4.0, nmin=-1.5, nmax=1.5, r0=0.3)
    got, ref = _run_both(oracle_mod, c, 10, iter0=3)
    assert_parity(got, ref, c.Ub, label=f"tiny {imax}x{jmax} nk={nk}")


@pytest.mark.parametrize("nk", [4, 5])
def test_acoustic_pulse_short(oracle_mod, nslib, nk):
    c = cases.acoustic_pulse_case(imax=101, jmax=91, nk=nk, D=20)
    got, ref = _run_both(oracle_mod, c, 40)
    assert_parity(got, ref, c.Ub, label=f"pulse nk={nk}")


def test_acoustic_pulse_201x201_500_steps(oracle_mod, nslib):
    """201x201 Euler pulse, sigma_f = 0.2, D = 30, CFL 0.5, 500 steps."""
    c = cases.acoustic_pulse_case()
    got, ref = _run_both(oracle_mod, c, 500)
    errs = assert_parity(got, ref, c.Ub, label="pulse 201x201, 500 steps")
    print("pulse 201x201 per variable (rel max, rel perturbation):", errs)


def test_mixing_layer_reference_case(oracle_mod, nslib):
    """The reference's dados.in physics (mixing layer, source, Re = 1e4) on a
    reduced grid, with the buffer quirk as compiled."""
    c = cases.mixing_layer_case(imax=130, jmax=121, D=22, maxit=0)
    got, ref = _run_both(oracle_mod, c, 25)
    assert_parity(got, ref, c.Ub, label="mixing layer")


def test_mixing_layer_no_quirk_field_source(oracle_mod, nslib):
    c = cases.mixing_layer_case(imax=96, jmax=80, nk=4, D=16, quirk_buffer=False)
    rng = np.random.default_rng(7)
    c.source_mode = L.NS_SRC_FIELD
    c.src_field = 1e-3 * rng.standard_normal((c.jmax, c.imax))
    c.wf = 0.7
    got, ref = _run_both(oracle_mod, c, 15, iter0=11)
    assert_parity(got, ref, c.Ub, label="field source, no quirk")


def test_stretched_ns_reduced(oracle_mod, nslib):
    """The stretched-grid Navier-Stokes case (metric everywhere) at 512x256."""
    c = cases.stretched_ns_case(imax=512, jmax=256, D=20, vortex_upstream=60)
    got, ref = _run_both(oracle_mod, c, 12)
    assert_parity(got, ref, c.Ub, label="stretched NS 512x256")


def test_chunked_filters(oracle_mod, nslib):
    """Lines long enough that both filters run as several chunks with warm-up."""
    from navierstokes_gb300 import Solver
    c = cases.stretched_ns_case(imax=1600, jmax=900, nk=5, D=30, vortex_upstream=150)
    with Solver(c) as s:
        assert s.filter_warmup() >= 36
    got, ref = _run_both(oracle_mod, c, 4)
    assert_parity(got, ref, c.Ub, label="chunked filters 1600x900")


def test_uniform_state_is_fixed_point(oracle_mod, nslib):
    """A uniform state equal to the base flow at the full 4096x2048 size:
    it moves only where the REAL(4) y boundary filter acts (its coefficients
    sum to -8.4e-9, filtering.f90:114-120) -- rows far from the top and
    bottom stay exact -- and that drift equals the oracle's."""
    from navierstokes_gb300 import Solver
    c = cases.stretched_ns_case(pulse_amp=0.0, vortex_eps=0.0)
    nsteps = 2
    with Solver(c) as s:
        s.set_state(c.Ub)
        s.step(0, nsteps)
        U = s.get_state()
        assert s.check_finite() == 0
    assert np.max(np.abs(U[200:-200] - c.Ub[200:-200])) < 1e-13
    assert np.max(np.abs(U - c.Ub)) < 1e-6
    ref = c.Ub.copy()
    oracle_mod.Oracle(c).run(ref, 0, nsteps)
    assert_parity(U, ref, c.Ub, label="uniform state 4096x2048")


def test_navier_stokes_4096x2048_ten_steps(oracle_mod, nslib):
    """4096x2048 Navier-Stokes (the benchmark workload), ten steps, GPU vs
    oracle at full size: TMA tiles, the transport-law table and the
    segmented filters over the whole grid."""
    c = cases.stretched_ns_case()
    got, ref = _run_both(oracle_mod, c, 10)
    errs = assert_parity(got, ref, c.Ub, label="Navier-Stokes 4096x2048, 10 steps")
    print("4096x2048 NS, 10 steps, per variable (rel max, rel perturbation):", errs)


@pytest.mark.slow
def test_navier_stokes_4096x2048_200_steps(oracle_mod, nslib):
    """The benchmark workload over its whole stated run: 4096x2048
    Navier-Stokes on the stretched grid, 200 steps on the GPU against 200
    oracle steps on every host core (about two minutes), per variable
    <= 1e-12 of its scale; the error relative to each perturbation is
    printed beside it."""
    c = cases.stretched_ns_case()
    assert c.steps == 200
    got, ref = _run_both(oracle_mod, c, c.steps)
    errs = assert_parity(got, ref, c.Ub, label="Navier-Stokes 4096x2048, 200 steps")
    print("4096x2048 NS, 200 steps, per variable (rel max, rel perturbation):", errs)


def test_rk_euler_dropin_matches_resident(oracle_mod, nslib):
    """ns_rk_euler (host U in, host U out, one step per call) equals the
    resident-state path and the oracle."""
    from navierstokes_gb300 import Solver
    c = cases.mixing_layer_case(imax=64, jmax=48, D=10)
    U = c.U0.copy()
    with Solver(c) as s:
        for it in range(5):
            s.rk_euler(U, (it + 1) * c.dt, it)
        res = s.run(c.U0, 0, 5)
    ref = c.U0.copy()
    oracle_mod.Oracle(c).run(ref, 0, 5)
    assert np.array_equal(U, res)
    assert_parity(U, ref, c.Ub, label="rk_euler drop-in")


@pytest.mark.parametrize("precision", ["fp64", "fp64_bands", "euler_bands", "fp64_2048",
                                       "split"])
def test_rk_euler_pinned_host_reads_directly(nslib, precision):
    """ns_rk_euler on page-locked host memory: FP64 copies the host array in
    row bands and starts stage 0 on the bands that have landed; on grids large
    enough (2048 x 2048: 4 bands) it also runs the last stage's y sweep and
    ccpml in row bands and sends each band home while the next is filtered;
    split precision reads and writes the array in place.  Results equal the
    pageable path's bit for bit, or to rounding where the last stage is
    banded."""
    import torch
    from navierstokes_gb300 import Solver
    from navierstokes_gb300 import _lib as L
    if precision == "fp64":
        c, prec = cases.mixing_layer_case(imax=64, jmax=48, D=10), L.NS_PREC_FP64
    elif precision == "fp64_bands":
        # 3 bands of 72, 72 and 56 rows; Navier-Stokes with psi (nk = 5)
        c, prec = cases.mixing_layer_case(imax=96, jmax=200, D=10), L.NS_PREC_FP64
    elif precision == "fp64_2048":
        c = cases.uniform_flow_case(imax=2048, jmax=2048, D=30, vortex_upstream=300)
        prec = L.NS_PREC_FP64
    elif precision == "euler_bands":
        # 8 bands; Euler (nk = 4) with a source
        c = cases.acoustic_pulse_case(imax=72, jmax=520, nk=4, D=12)
        c.source_mode, c.amplitude, c.wf, c.r0 = L.NS_SRC_GAUSSIAN, 1e-3, 0.3, 3.0
        prec = L.NS_PREC_FP64
    else:
        c, prec = cases.uniform_flow_case(imax=96, jmax=80, D=10, vortex_upstream=20), \
            L.NS_PREC_SPLIT
    pinned = torch.empty(c.U0.shape, dtype=torch.float64, pin_memory=True).numpy()
    pinned[...] = c.U0
    paged = c.U0.copy()
    with Solver(c, precision=prec) as s:
        for it in range(4):
            s.rk_euler(pinned, (it + 1) * c.dt, it)
    with Solver(c, precision=prec) as s:
        for it in range(4):
            s.rk_euler(paged, (it + 1) * c.dt, it)
    assert not np.array_equal(pinned, c.U0)
    if precision != "fp64_2048":
        assert np.array_equal(pinned, paged)
    else:
        # 2048 x 2048 runs the last stage's y sweep in row bands on the pinned
        # path: its pieces warm up from other points than the whole sweep's,
        # so the two agree to rounding
        assert_parity(pinned, paged, c.Ub, tol=1e-14, label="banded last stage")


def test_rk_euler_on_registered_host_array(nslib):
    """An existing host array (as a Fortran U would be) page-locked with
    ns_pin_host takes the banded path of ns_rk_euler; results equal the
    pageable path's bit for bit, and ns_unpin_host releases it."""
    from navierstokes_gb300 import Solver
    c = cases.mixing_layer_case(imax=96, jmax=200, D=10)
    U = np.ascontiguousarray(c.U0.copy())
    paged = c.U0.copy()
    assert nslib.ns_pin_host(U.ctypes.data, U.nbytes) == 0
    try:
        with Solver(c) as s:
            for it in range(3):
                s.rk_euler(U, (it + 1) * c.dt, it)
    finally:
        assert nslib.ns_unpin_host(U.ctypes.data) == 0
    with Solver(c) as s:
        for it in range(3):
            s.rk_euler(paged, (it + 1) * c.dt, it)
    assert np.array_equal(U, paged)


def test_probes_and_layouts(nslib):
    from navierstokes_gb300 import Solver
    c = cases.acoustic_pulse_case(imax=50, jmax=40, D=8)
    with Solver(c) as s:
        s.set_state(c.U0)
        pr = s.probes([1, 25, 50], [1, 20, 40])
        np.testing.assert_array_equal(pr[0], c.U0[0, 0])
        np.testing.assert_array_equal(pr[1], c.U0[19, 24])
        np.testing.assert_array_equal(pr[2], c.U0[39, 49])
        back = s.get_state()
        np.testing.assert_array_equal(back, c.U0)
        with pytest.raises(L.NsError):
            s.probes([0], [1])


def test_nonfinite_detected(nslib):
    from navierstokes_gb300 import Solver
    c = cases.acoustic_pulse_case(imax=30, jmax=30, D=5)
    U = c.U0.copy()
    U[10, 11, 2] = np.nan
    U[3, 4, 0] = np.inf
    with Solver(c) as s:
        s.set_state(U)
        assert s.check_finite() == 2
