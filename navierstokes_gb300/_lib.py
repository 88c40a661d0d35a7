"""ctypes binding of libns_gb300.so (include/ns_gb300.h).

The library must exist and load: there is no CPU or PyTorch fallback.  A
missing or unloadable library raises ImportError naming the build step.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

# NS_GB300_LIB names another build of the same library to load instead (the
# checked build, libns_gb300_checked.so); it must exist like the default.
LIB_PATH = Path(os.environ.get("NS_GB300_LIB") or
                Path(__file__).resolve().parent / "libns_gb300.so").resolve()

NS_OK = 0
NS_ERR_PARAM = 1
NS_ERR_CUDA = 2
NS_ERR_OOM = 3
NS_ERR_NONFINITE = 4
NS_ERR_TIMEOUT = 5
NS_ERR_STATE = 6
NS_ERR_UNSUPPORTED = 7
NS_ERR_CHECK = 8

NS_LAYOUT_FORTRAN = 0
NS_LAYOUT_SOA = 1
NS_LAYOUT_ROWS = 2
NS_PREC_FP64 = 0
NS_PREC_SPLIT = 1
NS_PREC_SPLIT32 = 2
NS_TRANSPORT_TABLE_DOUBLES = 5 * 256 * 12
NS_SRC_NONE = 0
NS_SRC_GAUSSIAN = 1
NS_SRC_FIELD = 2
NS_METRIC_BANDS = 0
NS_METRIC_EVERYWHERE = 1

ABI_VERSION = 1

# Every entry point declared in include/ns_gb300.h: (name, restype, argtypes).
_VP = C.c_void_p
SIGNATURES = [
    ("ns_abi_version", C.c_int, []),
    ("ns_build_info", C.c_char_p, []),
    ("ns_params_init", C.c_int, [_VP]),
    ("ns_create", C.c_int, [_VP, C.POINTER(_VP)]),
    ("ns_destroy", None, [_VP]),
    ("ns_last_error", C.c_char_p, [_VP]),
    ("ns_set_state", C.c_int, [_VP, _VP, C.c_int]),
    ("ns_get_state", C.c_int, [_VP, _VP, C.c_int]),
    ("ns_step", C.c_int, [_VP, C.c_int, C.c_int]),
    ("ns_synchronize", C.c_int, [_VP]),
    ("ns_rk_euler", C.c_int, [_VP, _VP, C.c_double, C.c_int, C.c_int]),
    ("ns_get_probes", C.c_int, [_VP, C.c_int, _VP, _VP, _VP]),
    ("ns_check_finite", C.c_int, [_VP, C.POINTER(C.c_int64)]),
    ("ns_set_stream", C.c_int, [_VP, _VP]),
    ("ns_get_stream", C.c_int, [_VP, C.POINTER(_VP)]),
    ("ns_state_device", C.c_int, [_VP, C.POINTER(_VP), C.POINTER(C.c_int64)]),
    ("ns_step_launches", C.c_int, [_VP, C.POINTER(C.c_int)]),
    ("ns_filter_warmup", C.c_int, [_VP, C.POINTER(C.c_int)]),
    ("ns_time_kernels", C.c_int, [_VP, C.c_int, C.c_int, _VP, _VP]),
    ("ns_kernel_name", C.c_char_p, [C.c_int]),
    ("ns_fp64_peak", C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    ("ns_math_eval", C.c_int, [C.c_int, _VP, _VP, C.c_int, C.c_int]),
    ("ns_transport_eval", C.c_int, [_VP, _VP, _VP, _VP, C.c_int]),
    ("ns_adjoint_stored_bytes", C.c_int, [_VP, C.POINTER(C.c_int64)]),
    ("ns_tma_wait_test", C.c_int, [C.c_int, C.c_longlong]),
    ("ns_checked_build", C.c_int, []),
    ("ns_check_selftest", C.c_int, [C.c_int]),
    ("ns_transport_table", C.c_int, [C.c_double, _VP, _VP, _VP]),
    ("ns_coef_table", C.c_int, [C.c_int, _VP]),
    ("ns_pin_host", C.c_int, [_VP, C.c_size_t]),
    ("ns_unpin_host", C.c_int, [_VP]),
    ("ns_filter_plan", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                 C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
    ("ns_step_noalloc", C.c_int, [_VP, _VP, C.c_int64, C.c_int, C.c_int, _VP]),
    ("ns_batch_create", C.c_int, [_VP, C.c_int, C.c_int, C.POINTER(_VP)]),
    ("ns_batch_destroy", None, [_VP]),
    ("ns_batch_set_state", C.c_int, [_VP, C.c_int, _VP, C.c_int]),
    ("ns_batch_get_state", C.c_int, [_VP, C.c_int, _VP, C.c_int]),
    ("ns_batch_step", C.c_int, [_VP, C.c_int, C.c_int]),
    ("ns_batch_synchronize", C.c_int, [_VP]),
    ("ns_batch_set_stream", C.c_int, [_VP, _VP]),
    ("ns_batch_autotune", C.c_int, [_VP, C.c_int, C.c_int, C.POINTER(C.c_int),
                                    C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    ("ns_batch_phase_times", C.c_int, [_VP, C.c_int, _VP]),
    ("ns_batch_info", C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                C.POINTER(C.c_int), _VP]),
    ("ns_batch_barrier_test", C.c_int, [_VP, C.c_int, C.c_longlong]),
    ("ns_adjoint_create", C.c_int, [_VP, C.c_int, _VP, _VP, C.c_int, C.POINTER(_VP)]),
    ("ns_adjoint_destroy", None, [_VP]),
    ("ns_adjoint_set_source", C.c_int, [_VP, _VP]),
    ("ns_adjoint_forward", C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int,
                                     C.POINTER(C.c_double)]),
    ("ns_adjoint_backward", C.c_int, [_VP, _VP]),
    ("ns_adjoint_context", C.c_int, [_VP, C.POINTER(_VP)]),
    ("ns_read_dados", C.c_int, [C.c_char_p, _VP]),
    ("ns_parse_dados", C.c_int, [C.c_char_p, _VP]),
    ("ns_dados_grid", C.c_int, [_VP, C.c_int] + [_VP] * 8),
    ("ns_dados_profiles", C.c_int, [_VP] * 6),
    ("ns_create_dados", C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.POINTER(_VP)]),
    ("ns_vorticity", C.c_int, [_VP, _VP]),
    ("ns_write_contorno", C.c_int, [_VP, C.c_char_p, _VP, _VP]),
    ("ns_format_real", C.c_int, [C.c_double, C.c_char_p, C.c_int]),
    ("ns_probes_arm", C.c_int, [_VP, C.c_int, _VP, _VP, C.c_int]),
    ("ns_probes_capture", C.c_int, [_VP]),
    ("ns_probes_drain", C.c_int, [_VP, _VP, C.POINTER(C.c_int)]),
    ("ns_run_euler", C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int]),
]

NS_RUN_NO_CONTORNO = 1
NS_RUN_QUIET = 2

NS_KC_COUNT = 12


class NsParams(C.Structure):
    """Mirror of `ns_params` (include/ns_gb300.h)."""

    _fields_ = [
        ("abi_version", C.c_int32), ("imax", C.c_int32), ("jmax", C.c_int32),
        ("nk", C.c_int32), ("D", C.c_int32), ("inviscid", C.c_int32),
        ("metric_mode", C.c_int32), ("precision", C.c_int32), ("source_mode", C.c_int32),
        ("device", C.c_int32), ("ub_layout", C.c_int32), ("reserved0", C.c_int32),
        ("dt", C.c_double), ("dm", C.c_double), ("dn", C.c_double), ("sigmaf", C.c_double),
        ("gamma", C.c_double), ("Re", C.c_double), ("Pr", C.c_double), ("Tref", C.c_double),
        ("A_mi", C.c_double), ("B_mi", C.c_double), ("C_mi", C.c_double), ("D_mi", C.c_double),
        ("A_k", C.c_double), ("B_k", C.c_double), ("C_k", C.c_double), ("D_k", C.c_double),
        ("amplitude", C.c_double), ("wf", C.c_double), ("m_pt", C.c_double),
        ("n_pt", C.c_double), ("r0", C.c_double),
        ("m", _VP), ("n", _VP), ("meshx", _VP), ("meshy", _VP), ("sigmax", _VP),
        ("sigmay", _VP), ("rhob", _VP), ("psib", _VP), ("Ub", _VP), ("src_field", _VP),
    ]


class NsDados(C.Structure):
    """Mirror of `ns_dados` (include/ns_gb300.h): the dados.in namelists."""

    _fields_ = [
        ("imax", C.c_int32), ("jmax", C.c_int32), ("maxit", C.c_int32), ("cgd", C.c_int32),
        ("cfd", C.c_int32), ("ctd", C.c_int32), ("D", C.c_int32), ("iterw", C.c_int32),
        ("num_procs_x", C.c_int32), ("num_procs_y", C.c_int32),
        ("dt", C.c_double), ("sigmaf", C.c_double),
        ("r0_acous", C.c_double), ("amplitude", C.c_double), ("m_pt_acous", C.c_double),
        ("n_pt_acous", C.c_double), ("wfi", C.c_double), ("wff", C.c_double), ("wf", C.c_double),
        ("pxfft", C.c_double * 5),
        ("mmin", C.c_double), ("mmax", C.c_double), ("nmin", C.c_double), ("nmax", C.c_double),
        ("pxr", C.c_double * 3), ("pyr", C.c_double * 3),
        ("U1", C.c_double), ("U2", C.c_double), ("Re", C.c_double), ("Pr", C.c_double),
        ("T1", C.c_double), ("T2", C.c_double), ("Tref", C.c_double),
        ("c1b", C.c_double), ("c2b", C.c_double), ("c3b", C.c_double),
    ]


class NsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[ns status {code}] {msg}")
        self.code = code


_lib = None


def load():
    """Loads libns_gb300.so; raises ImportError if it is missing or broken."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH.name} is not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
            "(needs nvcc); there is no CPU fallback")
    try:
        L = C.CDLL(str(LIB_PATH))
    except OSError as e:  # pragma: no cover - depends on the machine
        raise ImportError(f"cannot load {LIB_PATH}: {e}") from e
    for name, res, args in SIGNATURES:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if L.ns_abi_version() != ABI_VERSION:
        raise ImportError(f"{LIB_PATH.name} has ABI {L.ns_abi_version()}, binding expects {ABI_VERSION}")
    _lib = L
    return L


def last_error(ctx=None) -> str:
    msg = load().ns_last_error(ctx)
    return msg.decode() if msg else ""


def check(rc: int, ctx=None) -> None:
    if rc != NS_OK:
        raise NsError(rc, last_error(ctx))
