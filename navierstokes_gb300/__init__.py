"""GB300-native (sm_103a) LDDRK time step for the mathe1s/NavierStokes solver.

The hot path -- rk_euler (rk.f90:12-75) and everything it calls -- runs as
hand-written CUDA behind the C ABI of include/ns_gb300.h.  This package is
the Python host side: problem setup (`cases`), the ctypes binding (`_lib`)
and the reference-shaped solver interface (`Solver`).
"""
from . import _lib
from .cases import (Case, acoustic_pulse_case, init_dados, mixing_layer_case,
                    stretched_ns_case, uniform_flow_case)
from .solver import Batch, Solver

__all__ = ["Batch", "Case", "Solver", "acoustic_pulse_case", "init_dados", "mixing_layer_case",
           "stretched_ns_case", "uniform_flow_case", "_lib"]
