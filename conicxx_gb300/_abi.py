"""ctypes mirror of include/conicxx_gb300.h (struct layouts and constants).

Shared by the product binding (conicxx_gb300._lib) and the test-side oracle binding; it holds
no compute.
"""
import ctypes as C

import numpy as np

OK = 0
E_INVALID, E_PATTERN, E_NOT_SETUP, E_CUDA, E_NOMEM, E_UNSUPPORTED, E_INTERNAL = -1, -2, -3, -4, -5, -6, -7

STATUS_UNSOLVED = 0
STATUS_SOLVED = 1
STATUS_PRIMAL_INFEASIBLE = 2
STATUS_DUAL_INFEASIBLE = 3
STATUS_MAX_ITERATIONS = 4
STATUS_NUMERICAL_ERROR = 5
STATUS_NAMES = {
    0: "Unsolved", 1: "Solved", 2: "PrimalInfeasible", 3: "DualInfeasible",
    4: "MaxIterations", 5: "NumericalError",
}

LINSOLVER_EIGEN, LINSOLVER_QDLDL, LINSOLVER_REGULARIZED = 0, 1, 2
PRECISION_FP64, PRECISION_MIXED = 0, 1


class Settings(C.Structure):
    """cxg_settings: the reference's Settings (include/conicxx/settings.h:21-62) plus additions."""

    _fields_ = [
        ("tol_feas", C.c_double),
        ("tol_gap_abs", C.c_double),
        ("tol_gap_rel", C.c_double),
        ("tol_infeas", C.c_double),
        ("max_iter", C.c_int),
        ("static_reg_P", C.c_double),
        ("static_reg_A", C.c_double),
        ("dynamic_reg_eps", C.c_double),
        ("dynamic_reg_delta", C.c_double),
        ("refine_max_iter", C.c_int),
        ("refine_tol", C.c_double),
        ("max_step_fraction", C.c_double),
        ("equilibrate", C.c_int),
        ("equilibrate_max_iter", C.c_int),
        ("equilibrate_min_scale", C.c_double),
        ("equilibrate_max_scale", C.c_double),
        ("warm_start", C.c_int),
        ("verbose", C.c_int),
        ("record_timings", C.c_int),
        ("validate_inputs", C.c_int),
        ("linear_solver", C.c_int),
        ("precision", C.c_int),
        ("mixed_refine_max_iter", C.c_int),
        ("mixed_fallback_tol", C.c_double),
        ("threads_per_instance", C.c_int),
        ("differentiable", C.c_int),
        ("whole_gpu_root", C.c_int),
        ("fault_factor_failures", C.c_int),
        ("fault_nonfinite_solves", C.c_int),
        ("soc_reference_dense", C.c_int),
    ]


def default_settings(**overrides):
    """Reference defaults (include/conicxx/settings.h:21-62) plus GB300 additions."""
    s = Settings(
        tol_feas=1e-8, tol_gap_abs=1e-8, tol_gap_rel=1e-8, tol_infeas=1e-7, max_iter=200,
        static_reg_P=1e-8, static_reg_A=1e-8, dynamic_reg_eps=1e-14, dynamic_reg_delta=1e-7,
        refine_max_iter=3, refine_tol=1e-12, max_step_fraction=0.99, equilibrate=1,
        equilibrate_max_iter=10, equilibrate_min_scale=1e-4, equilibrate_max_scale=1e4,
        warm_start=1, verbose=0, record_timings=0, validate_inputs=1,
        linear_solver=LINSOLVER_QDLDL, precision=PRECISION_FP64, mixed_refine_max_iter=4,
        mixed_fallback_tol=1e-10, threads_per_instance=0, differentiable=0,
        whole_gpu_root=0, fault_factor_failures=0, fault_nonfinite_solves=0, soc_reference_dense=1,
    )
    for k, v in overrides.items():
        if not hasattr(s, k):
            raise AttributeError(f"unknown setting {k!r}")
        setattr(s, k, int(v) if isinstance(v, bool) else v)
    return s


class Info(C.Structure):
    """cxg_info: the reference's Info (include/conicxx/solution.h:18-26) + status/objective."""

    _fields_ = [
        ("status", C.c_int),
        ("iterations", C.c_int),
        ("objective", C.c_double),
        ("primal_residual", C.c_double),
        ("dual_residual", C.c_double),
        ("duality_gap", C.c_double),
        ("mu", C.c_double),
        ("setup_time_s", C.c_double),
        ("solve_time_s", C.c_double),
        ("fp64_fallbacks", C.c_int),
        ("refine_steps", C.c_int),
        ("max_relres", C.c_double),
        ("time_factor_s", C.c_double),
        ("time_kkt_solve_s", C.c_double),
        ("time_other_s", C.c_double),
        ("time_assemble_s", C.c_double),
        ("time_ldlt_s", C.c_double),
        ("time_dense_solve_s", C.c_double),
        ("time_residual_s", C.c_double),
        ("factor_attempts", C.c_int),
        ("time_start_s", C.c_double),
        ("time_end_s", C.c_double),
        ("escalations", C.c_int),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


INFO_DTYPE = np.dtype([(name, np.int32 if t is C.c_int else np.float64) for name, t in Info._fields_],
                      align=True)
assert INFO_DTYPE.itemsize == C.sizeof(Info)


class Problem(C.Structure):
    """cxg_problem: one instance as plain pointers (caller-owned, copied by the library)."""

    _fields_ = [
        ("n", C.c_int), ("m", C.c_int),
        ("Pp", C.POINTER(C.c_int)), ("Pi", C.POINTER(C.c_int)), ("Px", C.POINTER(C.c_double)),
        ("q", C.POINTER(C.c_double)),
        ("Ap", C.POINTER(C.c_int)), ("Ai", C.POINTER(C.c_int)), ("Ax", C.POINTER(C.c_double)),
        ("b", C.POINTER(C.c_double)),
        ("zero_dim", C.c_int), ("nonneg_dim", C.c_int), ("n_soc", C.c_int),
        ("soc_dims", C.POINTER(C.c_int)),
    ]


def iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def make_problem_struct(qp):
    """Build a cxg_problem view of a QP (see conicxx_gb300.problem.QP). The returned tuple keeps
    the numpy buffers alive; element 0 is the struct."""
    keep = [
        np.ascontiguousarray(qp.P.indptr, dtype=np.int32), np.ascontiguousarray(qp.P.indices, dtype=np.int32),
        np.ascontiguousarray(qp.P.data, dtype=np.float64), np.ascontiguousarray(qp.q, dtype=np.float64),
        np.ascontiguousarray(qp.A.indptr, dtype=np.int32), np.ascontiguousarray(qp.A.indices, dtype=np.int32),
        np.ascontiguousarray(qp.A.data, dtype=np.float64), np.ascontiguousarray(qp.b, dtype=np.float64),
        np.ascontiguousarray(np.asarray(qp.soc, dtype=np.int32).reshape(-1)),
    ]
    socs = keep[8] if keep[8].size else np.zeros(1, np.int32)
    keep[8] = socs
    m = int(qp.A.shape[0])  # A's own row count; the library checks it against the cone spec
    if keep[7].shape[0] != m or keep[3].shape[0] != qp.n or qp.A.shape[1] != qp.n:
        raise ValueError("b/q/A sizes are inconsistent")
    st = Problem(
        n=qp.n, m=m, Pp=iptr(keep[0]), Pi=iptr(keep[1]), Px=dptr(keep[2]), q=dptr(keep[3]),
        Ap=iptr(keep[4]), Ai=iptr(keep[5]), Ax=dptr(keep[6]), b=dptr(keep[7]),
        zero_dim=qp.zero, nonneg_dim=qp.nonneg, n_soc=len(qp.soc), soc_dims=iptr(socs),
    )
    return st, keep
