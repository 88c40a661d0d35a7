"""The checked build in place of a device sanitizer.

libns_gb300_checked.so is the library compiled with -DNS_CHECKED: every
kernel range-checks the shared-tile, halo, closure, filter-segment and
work-list indices it derives, and a failed check is recorded (file and line)
instead of the access, so the host gets NS_ERR_CHECK and the device keeps
working.  These tests build it to its own path, show that a failed check is
reported, and run the parity cases with the most index arithmetic -- tiny
grids where every closure and filter pass overlaps, segmented filter sweeps,
the split-precision sweeps and the batched work lists -- against it in a
child process that loads it through NS_GB300_LIB.
"""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def checked_lib(nslib):
    from navierstokes_gb300 import _build
    return _build.build(checked=True)


def _child(checked_lib, args, timeout=1500):
    env = dict(os.environ, NS_GB300_LIB=str(checked_lib))
    return subprocess.run([sys.executable, *args], cwd=ROOT, env=env, capture_output=True,
                          text=True, timeout=timeout)


def test_a_failed_check_is_reported(checked_lib):
    code = ("from navierstokes_gb300 import _lib as L; lib = L.load(); "
            "print(lib.ns_checked_build(), lib.ns_check_selftest(0), L.last_error())")
    r = _child(checked_lib, ["-c", code], timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    built, rc, msg = r.stdout.split(maxsplit=2)
    from navierstokes_gb300 import _lib as L
    assert int(built) == 1 and int(rc) == L.NS_ERR_CHECK, r.stdout
    assert "index check failed" in msg and "ns_kernels.cu" in msg
    # the ordinary build has no checks
    assert L.load().ns_checked_build() == 0
    assert L.load().ns_check_selftest(0) == L.NS_OK


def test_parity_cases_pass_under_the_checked_build(checked_lib):
    sel = ["tests/test_parity_gpu.py::test_tiny_grids_ns_source",
           "tests/test_parity_gpu.py::test_acoustic_pulse_short",
           "tests/test_parity_gpu.py::test_mixing_layer_no_quirk_field_source",
           "tests/test_parity_gpu.py::test_stretched_ns_reduced",
           "tests/test_parity_gpu.py::test_chunked_filters",
           "tests/test_parity_gpu.py::test_rk_euler_pinned_host_reads_directly",
           "tests/test_split_gpu.py::test_split_matches_fp64_pulse",
           "tests/test_split_gpu.py::test_split_with_source_and_chunked_filters",
           "tests/test_split_gpu.py::test_split_sheared_mean_flow",
           "tests/test_split_gpu.py::test_split_navier_stokes_stretched",
           "tests/test_batch_gpu.py",
           "tests/test_adjoint_gpu.py::test_adjoint_matches_torch_autograd",
           "tests/test_zz_no_alloc.py"]
    r = _child(checked_lib, ["-m", "pytest", "-q", "-x", "-p", "no:cacheprovider", *sel])
    tail = r.stdout[-4000:] + r.stderr[-2000:]
    print(tail)
    assert r.returncode == 0, tail
    assert " passed" in r.stdout
