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


@pytest.mark.gpu
def test_noalloc_soa_base_flow_on_a_stream_after_a_larger_case(nslib):
    """An inviscid case whose base flow arrives as planes (NS_LAYOUT_SOA), on
    a stream of the caller's, run straight after a larger viscous case: the
    work area still holds that case's arrays, and none of it reaches the
    result."""
    import torch
    from navierstokes_gb300 import Solver

    big = cases.mixing_layer_case(imax=160, jmax=120, D=16, dt=0.01)
    pb, keep_b = cases.params_from_case(big)
    pitch_b = (big.imax + 31) // 32 * 32
    dev_b = torch.zeros((big.nk, big.jmax, pitch_b), dtype=torch.float64, device="cuda:0")
    dev_b[:, :, :big.imax] = torch.from_numpy(
        np.ascontiguousarray(np.moveaxis(big.U0, 2, 0))).cuda()
    torch.cuda.synchronize()
    assert nslib.ns_step_noalloc(C.byref(pb), C.c_void_p(dev_b.data_ptr()), pitch_b, 0, 2,
                                 None) == L.NS_OK, L.last_error()

    c = cases.acoustic_pulse_case(imax=80, jmax=70, nk=4, D=10)
    c.source_mode, c.amplitude, c.wf, c.r0 = L.NS_SRC_GAUSSIAN, 1e-3, 0.4, 3.0
    nsteps = 5
    with Solver(c) as s:
        ref = s.run(c.U0, 2, nsteps)
    p, keep = cases.params_from_case(c)
    ub_planes = np.ascontiguousarray(np.moveaxis(c.Ub, 2, 0))   # (nk, jmax, imax)
    p.Ub = ub_planes.ctypes.data
    p.ub_layout = L.NS_LAYOUT_SOA
    pitch = (c.imax + 31) // 32 * 32
    stream = torch.cuda.Stream()
    dev = torch.zeros((c.nk, c.jmax, pitch), dtype=torch.float64, device="cuda:0")
    dev[:, :, :c.imax] = torch.from_numpy(np.ascontiguousarray(np.moveaxis(c.U0, 2, 0))).cuda()
    torch.cuda.synchronize()
    rc = nslib.ns_step_noalloc(C.byref(p), C.c_void_p(dev.data_ptr()), pitch, 2, nsteps,
                               C.c_void_p(stream.cuda_stream))
    assert rc == L.NS_OK, L.last_error()
    stream.synchronize()
    assert_parity(_to_fortran(dev, c), ref, c.Ub, label="no-alloc step, planes, own stream")
    del keep, keep_b


def test_noalloc_rejects_cases_beyond_the_work_area(nslib):
    c = cases.acoustic_pulse_case(imax=1024, jmax=1024, nk=5, D=10)
    p, keep = cases.params_from_case(c)
    rc = nslib.ns_step_noalloc(C.byref(p), C.c_void_p(1), 1024, 0, 1, None)
    assert rc == L.NS_ERR_PARAM
    msg = L.last_error()
    assert "work area" in msg and "NS_NOALLOC_MAX_BYTES" in msg
    # a pitch whose plane size would wrap is refused before any arithmetic on it
    c = cases.acoustic_pulse_case(imax=64, jmax=64, nk=4, D=8)
    p, keep = cases.params_from_case(c)
    rc = nslib.ns_step_noalloc(C.byref(p), C.c_void_p(1), 1 << 60, 0, 1, None)
    assert rc == L.NS_ERR_PARAM and "pitch" in L.last_error()
    del keep
