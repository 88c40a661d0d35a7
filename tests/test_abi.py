"""The C-ABI library loads and exports every entry point include/ns_gb300.h
declares; host-side validation rejects bad parameters before any CUDA call.
No compute runs here (no GPU needed)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "ns_gb300.h").read_text()
    return sorted(set(re.findall(r"NS_API\s+[\w\s\*]*?\b(ns_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("ns_create", "ns_destroy", "ns_step", "ns_rk_euler", "ns_set_state",
              "ns_get_state", "ns_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(nslib):
    from navierstokes_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s+(ns_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, f"declared but not exported: {missing}"
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert bound == set(declared_symbols())


def test_abi_version_and_defaults(nslib):
    from navierstokes_gb300 import _lib as L
    assert nslib.ns_abi_version() == L.ABI_VERSION
    p = L.NsParams()
    assert nslib.ns_params_init(C.byref(p)) == 0
    assert p.abi_version == L.ABI_VERSION and p.nk == 5 and p.gamma == 1.4
    assert p.A_mi == 0.62526577 and p.D_k == 0.48299104
    assert C.sizeof(L.NsParams) == 12 * 4 + 21 * 8 + 10 * 8


@pytest.mark.parametrize("field,value,msg", [
    ("imax", 12, "imax"),
    ("nk", 3, "nk"),
    ("D", 40, "D="),
    ("abi_version", 99, "abi_version"),
    ("dt", 0.0, "dt"),
    ("precision", 9, "precision"),
])
def test_create_rejects_bad_params(nslib, field, value, msg):
    from navierstokes_gb300 import _lib as L
    from navierstokes_gb300 import cases
    c = cases.acoustic_pulse_case(imax=60, jmax=60, D=10)
    p, keep = cases.params_from_case(c)
    setattr(p, field, value)
    ctx = C.c_void_p()
    rc = nslib.ns_create(C.byref(p), C.byref(ctx))
    assert rc in (L.NS_ERR_PARAM, L.NS_ERR_UNSUPPORTED)
    assert not ctx.value
    assert msg in L.last_error()


def test_null_arguments_are_errors(nslib):
    from navierstokes_gb300 import _lib as L
    assert nslib.ns_create(None, None) == L.NS_ERR_PARAM
    assert nslib.ns_step(None, 0, 1) == L.NS_ERR_PARAM
    assert nslib.ns_synchronize(None) == L.NS_ERR_PARAM
    nslib.ns_destroy(None)


def test_product_fails_loudly_without_library(monkeypatch, tmp_path):
    from navierstokes_gb300 import _lib as L
    monkeypatch.setattr(L, "LIB_PATH", tmp_path / "missing.so")
    monkeypatch.setattr(L, "_lib", None)
    with pytest.raises(ImportError, match="no CPU fallback"):
        L.load()
