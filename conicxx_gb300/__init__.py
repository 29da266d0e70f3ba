"""GB300-native ConicXX interior-point path.

The hot path -- the homogeneous self-dual embedding IPM of ConicXX (src/conicxx/solver_impl.cpp)
with its cones and KKT factorisation -- runs as hand-written sm_103a CUDA kernels behind the
C-ABI in include/conicxx_gb300.h. This package holds the ctypes binding, the host-side mirror of
conicxx::Solver, the batched solver, problem containers and the synthetic workload generators.
"""
from . import _abi
from ._abi import (PRECISION_FP64, PRECISION_MIXED, STATUS_DUAL_INFEASIBLE, STATUS_MAX_ITERATIONS,
                   STATUS_NAMES, STATUS_NUMERICAL_ERROR, STATUS_PRIMAL_INFEASIBLE, STATUS_SOLVED,
                   STATUS_UNSOLVED, Settings, default_settings)
from .problem import QP, Csc

__all__ = ["QP", "Csc", "Settings", "default_settings", "Solver", "BatchSolver", "Solution",
           "STATUS_NAMES", "PRECISION_FP64", "PRECISION_MIXED"]


def __getattr__(name):
    # The solver classes need the built library; importing them fails loudly when it is missing.
    if name in ("Solver", "BatchSolver", "Solution", "device_count"):
        from . import solver
        return getattr(solver, name)
    raise AttributeError(name)
