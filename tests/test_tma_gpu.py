"""The bounded mbarrier wait of the TMA tile loads (GPU): a barrier whose
bytes never arrive makes the wait run out; the error is reported as
NS_ERR_TIMEOUT and the device stays usable."""
import numpy as np
import pytest

from navierstokes_gb300 import cases

pytestmark = pytest.mark.gpu


def test_tma_wait_runs_out_and_reports(nslib):
    from navierstokes_gb300 import Solver
    from navierstokes_gb300 import _lib as L
    assert nslib.ns_tma_wait_test(0, 1000) == L.NS_ERR_TIMEOUT
    assert nslib.ns_tma_wait_test(0, 0) == L.NS_ERR_PARAM
    # the device keeps working: a TMA-tiled step afterwards
    c = cases.acoustic_pulse_case(imax=64, jmax=48, D=8, inviscid=False, nk=4)
    with Solver(c) as s:
        out = s.run(c.U0, 0, 2)
    assert np.all(np.isfinite(out)) and not np.array_equal(out, c.U0)
