"""ns_step_noalloc: the time step for callers that cannot allocate device memory.

Some hosts cannot call cudaMalloc: their device memory belongs to a
framework or pool that hands out fixed buffers, or they run under a hard
memory cap where an allocation failing halfway through a run is not
acceptable.  ns_step_noalloc serves them: the caller passes the state on the
device and the setup arrays on the host, and every work array comes from a
fixed 64 MiB area inside the library.  These tests check, through the C ABI,
that two calls in a row give the same state as the allocating entry point
(ns_create/ns_set_state/ns_step), and that a case too large for the area is
refused with a clear message.  This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from parity import assert_parity
from navierstokes_gb300 import _lib as L
from navierstokes_gb300 import cases


def _to_fortran(dev, case):
    """Device planes (nk, jmax, pitch) -> host array (jmax, imax, nk)."""
    a = dev[:, :, :case.imax].cpu().numpy()
    return np.ascontiguousarray(np.moveaxis(a, 0, 2))


@pytest.mark.gpu
def test_noalloc_matches_allocating_step_two_calls(nslib):
    import torch
    from navierstokes_gb300 import Solver

    # Navier-Stokes with the passive scalar and the Gaussian acoustic source,
    # so every kernel of the step runs.
    c = cases.mixing_layer_case(imax=96, jmax=72, D=12, dt=0.01)
    n1, n2 = 3, 4
    with Solver(c) as s:
        ref1 = s.run(c.U0, 0, n1)
        s.step(n1, n2)
        ref2 = s.get_state()

    p, keep = cases.params_from_case(c)
    pitch = (c.imax + 31) // 32 * 32
    dev = torch.zeros((c.nk, c.jmax, pitch), dtype=torch.float64, device="cuda:0")
    dev[:, :, :c.imax] = torch.from_numpy(np.ascontiguousarray(np.moveaxis(c.U0, 2, 0))).cuda()
    torch.cuda.synchronize()

    rc = nslib.ns_step_noalloc(C.byref(p), C.c_void_p(dev.data_ptr()), pitch, 0, n1, None)
    assert rc == L.NS_OK, L.last_error()
    torch.cuda.synchronize()
    assert_parity(_to_fortran(dev, c), ref1, c.Ub, label="no-alloc step, first call")

    rc = nslib.ns_step_noalloc(C.byref(p), C.c_void_p(dev.data_ptr()), pitch, n1, n2, None)
    assert rc == L.NS_OK, L.last_error()
    torch.cuda.synchronize()
    assert_parity(_to_fortran(dev, c), ref2, c.Ub, label="no-alloc step, second call")
    del keep


def test_noalloc_rejects_cases_beyond_the_work_area(nslib):
    c = cases.acoustic_pulse_case(imax=1024, jmax=1024, nk=5, D=10)
    p, keep = cases.params_from_case(c)
    rc = nslib.ns_step_noalloc(C.byref(p), C.c_void_p(1), 1024, 0, 1, None)
    assert rc == L.NS_ERR_PARAM
    msg = L.last_error()
    assert "work area" in msg and "NS_NOALLOC_MAX_BYTES" in msg
    del keep
