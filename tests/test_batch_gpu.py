"""Batched instances in one persistent launch per step, against the
single-grid paths (GPU)."""
import numpy as np
import pytest

from parity import assert_parity
from navierstokes_gb300 import _lib as L
from navierstokes_gb300 import cases

pytestmark = pytest.mark.gpu


def small_sweep(n=5, seed=3):
    return cases.sweep_cases(n=n, seed=seed, nmin=64, nmax=256)


def single(case, nsteps, precision, iter0=0):
    from navierstokes_gb300 import Solver
    with Solver(case, precision=precision) as s:
        return s.run(case.U0, iter0, nsteps)


def test_batch_fp64_matches_single_grid(oracle_mod, nslib):
    from navierstokes_gb300 import Batch
    cs = small_sweep()
    nsteps = 30
    with Batch(cs, precision=L.NS_PREC_FP64) as b:
        b.set_initial()
        b.step(2, nsteps)
        b.synchronize()
        got = [b.get_state(q) for q in range(len(cs))]
    for q, c in enumerate(cs):
        ref = c.U0.copy()
        oracle_mod.Oracle(c).run(ref, 2, nsteps)
        assert_parity(got[q], ref, c.Ub, label=f"batch fp64 instance {q} {c.imax}x{c.jmax}")


def test_single_instance_pulse_201x201_500_steps(oracle_mod, nslib):
    """The 201x201 Euler pulse (nk = 4) as a batch of one: every step one
    persistent launch, 500 steps against the oracle."""
    from navierstokes_gb300 import Batch
    c = cases.acoustic_pulse_case(nk=4)
    with Batch([c], precision=L.NS_PREC_FP64) as b:
        b.set_initial()
        b.step(0, 500)
        b.synchronize()
        got = b.get_state(0)
    ref = c.U0.copy()
    oracle_mod.Oracle(c).run(ref, 0, 500)
    errs = assert_parity(got, ref, c.Ub, label="pulse 201x201 as one persistent instance")
    print("201x201 batch of one, 500 steps (rel max, rel perturbation):", errs)


def test_batch_split_matches_single_split(nslib):
    from navierstokes_gb300 import Batch
    cs = small_sweep(n=4, seed=5)
    nsteps = 40
    with Batch(cs, precision=L.NS_PREC_SPLIT32) as b:
        b.set_initial()
        b.step(0, nsteps)
        b.synchronize()
        got = [b.get_state(q) for q in range(len(cs))]
    for q, c in enumerate(cs):
        ref = single(c, nsteps, L.NS_PREC_FP64)
        dp = got[q][..., 3] - ref[..., 3]
        pr = ref[..., 3] - c.Ub[..., 3]
        assert np.linalg.norm(dp) / np.linalg.norm(pr) <= 1e-5, q


def test_batch_autotune_and_info(nslib):
    from navierstokes_gb300 import Batch
    cs = small_sweep(n=6, seed=7)
    with Batch(cs, precision=L.NS_PREC_SPLIT32) as b:
        b.set_initial()
        ty, bps, ms = b.autotune(0, 1)
        assert ty in (8, 16) and bps >= 1 and ms > 0
        info = b.info()
        assert info["tile_rows"] == ty and info["items"][3] == len(cs)
        b.synchronize()


def test_batch_phase_times(nslib):
    """The phase stamps of one step: every phase takes time, and together
    they make up about one step."""
    import time
    from navierstokes_gb300 import Batch
    cs = small_sweep(n=4, seed=11)
    with Batch(cs, precision=L.NS_PREC_FP64) as b:
        b.set_initial()
        b.step(0, 2)
        b.synchronize()
        ph = b.phase_times(2)
        t0 = time.perf_counter()
        b.step(3, 10)
        b.synchronize()
        step_ms = (time.perf_counter() - t0) * 100.0
    assert all(v > 0 for v in ph.values()), ph
    assert 0.3 * step_ms < sum(ph.values()) < 3.0 * step_ms, (ph, step_ms)


def test_batch_barrier_timeout_is_reported_and_recoverable(nslib):
    """A barrier that waits for blocks that do not exist gives up after its
    spin limit: NS_ERR_TIMEOUT, and the batch keeps working afterwards."""
    from navierstokes_gb300 import Batch
    cs = small_sweep(n=3, seed=9)
    with Batch(cs, precision=L.NS_PREC_FP64) as b:
        b.set_initial()
        rc = b.barrier_test(extra=1, spin_limit=20000)
        assert rc == L.NS_ERR_TIMEOUT
        b.step(0, 3)
        b.synchronize()
        after = b.get_state(1)
    ref = single(cs[1], 3, L.NS_PREC_FP64)
    assert_parity(after, ref, cs[1].Ub, label="after timeout")


def test_batch_split_mode_is_fp32(nslib):
    from navierstokes_gb300 import Batch
    with pytest.raises(L.NsError) as e:
        Batch(small_sweep(n=2), precision=L.NS_PREC_SPLIT)
    assert e.value.code == L.NS_ERR_UNSUPPORTED
