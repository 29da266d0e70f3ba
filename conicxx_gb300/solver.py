"""Host-side mirror of ConicXX's operator interface for the interior-point path.

`Solver` keeps conicxx::Solver's API and semantics (include/conicxx/solver.h:33-95): setup
returns False on invalid input, update_data returns False when a matrix's sparsity pattern
changed (the caller then re-runs setup), solve always returns a Solution with a definite status.
`BatchSolver` is the batched form (many independent instances per call) the reference lacks.
Both run on the GPU through the C-ABI; there is no CPU path.
"""
import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._abi import Info, Settings, default_settings, dptr, iptr, make_problem_struct
from ._lib import CxgError, check, lib
from .problem import QP, Csc

# columns of an iteration-trace row (cxg_batch_trace / cxg_solver_trace)
TRACE_COLS = 12
TRACE_NAMES = ["mu", "norm_rx", "norm_rz", "pobj", "dobj", "alpha_aff", "sigma", "alpha", "tau", "kappa", "relres",
               "attempts"]


@dataclass
class Solution:
    """conicxx::Solution (include/conicxx/solution.h:28-39)."""

    status: int = _abi.STATUS_UNSOLVED
    x: np.ndarray = field(default_factory=lambda: np.zeros(0))
    s: np.ndarray = field(default_factory=lambda: np.zeros(0))
    z: np.ndarray = field(default_factory=lambda: np.zeros(0))
    objective: float = 0.0
    info: dict = field(default_factory=dict)

    def ok(self):
        return self.status == _abi.STATUS_SOLVED

    @property
    def status_name(self):
        return _abi.STATUS_NAMES.get(self.status, "Unknown")


def _settings(settings, default_precision, **kw):
    if settings is None:
        settings = default_settings(precision=default_precision)
    for k, v in kw.items():
        setattr(settings, k, v)
    return settings


class Solver:
    """Single-instance solver (FP64 factorisation by default: the plain per-instance GPU form).
    A root of more than 512 rows (n + zero_dim) is spread over every SM (whole_gpu_root setting:
    0 automatic, 1 always, -1 never)."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().cxg_solver_create(C.byref(h)), "cxg_solver_create")
        self._h = h
        self._qp = None
        self._solution = Solution()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().cxg_solver_destroy(h)
            self._h = None

    def setup(self, qp: QP, settings: Settings = None, **kw) -> bool:
        kw.setdefault("differentiable", 1)
        st = _settings(settings, _abi.PRECISION_FP64, **kw)
        prob, keep = make_problem_struct(qp)
        rc = lib().cxg_solver_setup(self._h, C.byref(prob), C.byref(st))
        if rc == _abi.E_INVALID:
            self._qp = None
            return False
        check(rc, "cxg_solver_setup")
        self._qp = qp
        self._solution = Solution()
        return True

    def setup_dense(self, P, q, A, b, zero=0, nonneg=0, soc=(), settings: Settings = None, **kw) -> bool:
        """The dense-input setup overloads (src/conicxx/solver.cpp:17-30): P and/or A as numpy
        arrays (or Csc), converted as the reference converts them (QP.from_dense)."""
        return self.setup(QP.from_dense(P, q, A, b, zero, nonneg, soc), settings, **kw)

    def update_data(self, P: Csc = None, q=None, A: Csc = None, b=None) -> bool:
        keep = []

        def arr(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a

        rc = lib().cxg_solver_update_data(
            self._h,
            iptr(arr(P.indptr, np.int32) if P is not None else None),
            iptr(arr(P.indices, np.int32) if P is not None else None),
            dptr(arr(P.data, np.float64) if P is not None else None),
            dptr(arr(q, np.float64)),
            iptr(arr(A.indptr, np.int32) if A is not None else None),
            iptr(arr(A.indices, np.int32) if A is not None else None),
            dptr(arr(A.data, np.float64) if A is not None else None),
            dptr(arr(b, np.float64)))
        if rc in (_abi.E_PATTERN, _abi.E_INVALID, _abi.E_NOT_SETUP):
            return False
        check(rc, "cxg_solver_update_data")
        return True

    def set_warm_start(self, x, s, z):
        x, s, z = (np.ascontiguousarray(v, dtype=np.float64) for v in (x, s, z))
        check(lib().cxg_solver_set_warm_start(self._h, dptr(x), dptr(s), dptr(z)), "cxg_solver_set_warm_start")

    def set_settings(self, settings: Settings):
        check(lib().cxg_solver_set_settings(self._h, C.byref(settings)), "cxg_solver_set_settings")

    def settings(self) -> Settings:
        st = Settings()
        check(lib().cxg_solver_get_settings(self._h, C.byref(st)), "cxg_solver_get_settings")
        return st

    def solve(self) -> Solution:
        info = Info()
        if self._qp is None:
            check(lib().cxg_solver_solve(self._h, None, None, None, C.byref(info)), "cxg_solver_solve")
            self._solution = Solution(status=info.status, info=info.as_dict())
            return self._solution
        n, m = self._qp.n, self._qp.m
        x, s, z = np.zeros(n), np.zeros(m), np.zeros(m)
        check(lib().cxg_solver_solve(self._h, dptr(x), dptr(s), dptr(z), C.byref(info)), "cxg_solver_solve")
        self._solution = Solution(status=info.status, x=x, s=s, z=z, objective=info.objective,
                                  info=info.as_dict())
        return self._solution

    def solution(self) -> Solution:
        return self._solution

    def trace(self):
        """Per-iteration trace of the last solve made with record_timings=1: an array of rows with
        the oracle's trace columns (oracle.TRACE_COLS)."""
        cap = max(1, self.settings().max_iter)
        out = np.zeros((cap, TRACE_COLS))
        k = lib().cxg_solver_trace(self._h, dptr(out), cap)
        if k < 0:
            check(k, "cxg_solver_trace")
        return out[:k]

    def backward(self, dl_dx):
        """Adjoint of the last Solved solution: dL/dq, dL/db, dL/d(P values), dL/d(A values)."""
        qp = self._qp
        dl = np.ascontiguousarray(dl_dx, dtype=np.float64)
        dq, db = np.zeros(qp.n), np.zeros(qp.m)
        dP, dA = np.zeros(qp.P.nnz), np.zeros(qp.A.nnz)
        check(lib().cxg_solver_backward(self._h, dptr(dl), dptr(dq), dptr(db), dptr(dP), dptr(dA)),
              "cxg_solver_backward")
        return dq, db, dP, dA


class BatchSolver:
    """Many independent instances solved per call (mixed precision by default)."""

    def __init__(self, qps, settings: Settings = None, **kw):
        st = _settings(settings, _abi.PRECISION_MIXED, **kw)
        structs, self._keep = [], []
        for qp in qps:
            s, k = make_problem_struct(qp)
            structs.append(s)
            self._keep.append(k)
        arr = (_abi.Problem * len(qps))(*structs)
        h = C.c_void_p()
        check(lib().cxg_batch_create(C.byref(h), len(qps), arr, C.byref(st)), "cxg_batch_create")
        self._h = h
        self.qps = list(qps)
        self.count = len(qps)
        self._keep = None  # the library copied everything
        self._offsets()

    def _offsets(self):
        qps = self.qps
        self.n_off = np.zeros(self.count + 1, np.int64)
        self.m_off = np.zeros(self.count + 1, np.int64)
        self.p_off = np.zeros(self.count + 1, np.int64)
        self.a_off = np.zeros(self.count + 1, np.int64)
        for i, qp in enumerate(qps):
            self.n_off[i + 1] = self.n_off[i] + qp.n
            self.m_off[i + 1] = self.m_off[i] + qp.m
            self.p_off[i + 1] = self.p_off[i] + qp.P.nnz
            self.a_off[i + 1] = self.a_off[i] + qp.A.nnz
        self.nnzP, self.n_total, self.nnzA, self.m_total = (int(self.p_off[-1]), int(self.n_off[-1]),
                                                            int(self.a_off[-1]), int(self.m_off[-1]))

    def replace(self, indices, qps):
        """A new set-up of instances indices[j] as qps[j] (new patterns and sizes allowed), the
        others kept with their values and warm starts (cxg_batch_replace). Returns the seconds the
        call took (host planning of the replaced instances, device re-layout)."""
        import time

        indices = [int(i) for i in indices]
        structs, keep = [], []
        for qp in qps:
            s_, k_ = make_problem_struct(qp)
            structs.append(s_)
            keep.append(k_)
        arr = (_abi.Problem * max(1, len(qps)))(*structs)
        idx = np.ascontiguousarray(indices, dtype=np.int32)
        t0 = time.perf_counter()
        check(lib().cxg_batch_replace(self._h, len(indices), iptr(idx), arr), "cxg_batch_replace")
        dt = time.perf_counter() - t0
        for i, qp in zip(indices, qps):
            self.qps[i] = qp
        self._offsets()
        a, b, c_, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().cxg_batch_sizes(self._h, C.byref(a), C.byref(b), C.byref(c_), C.byref(d)), "cxg_batch_sizes")
        assert (a.value, b.value, c_.value, d.value) == (self.nnzP, self.n_total, self.nnzA, self.m_total)
        return dt

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().cxg_batch_destroy(h)
            self._h = None

    def concat_values(self, qps=None):
        """Concatenated (Px, q, Ax, b) of instances (default: the set-up ones)."""
        qps = qps or self.qps
        return (np.concatenate([qp.P.data for qp in qps]), np.concatenate([qp.q for qp in qps]),
                np.concatenate([qp.A.data for qp in qps]), np.concatenate([qp.b for qp in qps]))

    def update_values(self, Px=None, q=None, Ax=None, b=None):
        keep = [None if v is None else np.ascontiguousarray(v, dtype=np.float64) for v in (Px, q, Ax, b)]
        check(lib().cxg_batch_update_values(self._h, *(dptr(v) for v in keep)), "cxg_batch_update_values")

    def solve(self):
        """Returns (x, s, z, infos): concatenated solutions and a structured info array."""
        x, s, z = np.zeros(self.n_total), np.zeros(self.m_total), np.zeros(self.m_total)
        infos = np.zeros(self.count, dtype=_abi.INFO_DTYPE)
        check(lib().cxg_batch_solve(self._h, dptr(x), dptr(s), dptr(z),
                                    infos.ctypes.data_as(C.POINTER(Info))), "cxg_batch_solve")
        return x, s, z, infos

    def trace(self, instance):
        """Per-iteration trace of one instance of the last solve made with record_timings=1."""
        cap = 1024
        out = np.zeros((cap, TRACE_COLS))
        k = lib().cxg_batch_trace(self._h, int(instance), dptr(out), cap)
        if k < 0:
            check(k, "cxg_batch_trace")
        return out[:k]

    def backward(self, dl_dx):
        """Adjoint of every instance at its last solution (needs differentiable=1): returns the
        concatenated (dL/dq, dL/db, dL/d(P values), dL/d(A values))."""
        g = np.ascontiguousarray(dl_dx, dtype=np.float64)
        dq, db = np.zeros(self.n_total), np.zeros(self.m_total)
        dP, dA = np.zeros(self.nnzP), np.zeros(self.nnzA)
        check(lib().cxg_batch_backward(self._h, dptr(g), dptr(dq), dptr(db), dptr(dP), dptr(dA)),
              "cxg_batch_backward")
        return dq, db, dP, dA

    def backward_device(self, gx_ptr, dq_ptr, db_ptr, dP_ptr, dA_ptr, stream_ptr):
        check(lib().cxg_batch_backward_device(self._h, gx_ptr, dq_ptr, db_ptr, dP_ptr, dA_ptr, stream_ptr),
              "cxg_batch_backward_device")

    def solve_device(self, x_ptr, s_ptr, z_ptr, stream_ptr, infos=None):
        """Enqueue a solve writing device buffers (raw pointers) on a CUDA stream handle."""
        ip_ = infos.ctypes.data_as(C.POINTER(Info)) if infos is not None else None
        check(lib().cxg_batch_solve_device(self._h, x_ptr, s_ptr, z_ptr, ip_, stream_ptr),
              "cxg_batch_solve_device")

    def solve_device_noalloc(self, x_ptr, s_ptr, z_ptr, stream_ptr, infos=None):
        """Like solve_device, through the allocation-free entry point (fixed device workspace,
        buckets launched one after another on the stream, no graph)."""
        ip_ = infos.ctypes.data_as(C.POINTER(Info)) if infos is not None else None
        check(lib().cxg_batch_solve_device_noalloc(self._h, x_ptr, s_ptr, z_ptr, ip_, stream_ptr),
              "cxg_batch_solve_device_noalloc")

    def update_values_device(self, Px_ptr, q_ptr, Ax_ptr, b_ptr, stream_ptr):
        check(lib().cxg_batch_update_values_device(self._h, Px_ptr, q_ptr, Ax_ptr, b_ptr, stream_ptr),
              "cxg_batch_update_values_device")

    def autotune(self, trials=3):
        """Pick threads per instance for every size bucket by timing each bucket's launch alone
        (cxg_batch_autotune); returns the per-bucket report."""
        buf = C.create_string_buffer(8192)
        check(lib().cxg_batch_autotune(self._h, int(trials), buf, len(buf)), "cxg_batch_autotune")
        return buf.value.decode()

    def last_launches(self):
        return lib().cxg_batch_last_launches(self._h)

    def footprint(self):
        """(plan bytes, value bytes, scratch bytes) resident on the device."""
        a, b, c_ = C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().cxg_batch_footprint(self._h, C.byref(a), C.byref(b), C.byref(c_)), "cxg_batch_footprint")
        return a.value, b.value, c_.value

    def algorithmic_bytes(self):
        """HBM bytes one solve must move at minimum: every instance's plan and values read once,
        solutions and results written once."""
        plan, values, _ = self.footprint()
        return plan + values

    def describe(self):
        buf = C.create_string_buffer(8192)
        lib().cxg_batch_describe(self._h, buf, len(buf))
        return buf.value.decode()

    def split(self, x, s, z):
        """Per-instance views of concatenated solutions."""
        return [(x[self.n_off[i]:self.n_off[i + 1]], s[self.m_off[i]:self.m_off[i + 1]],
                 z[self.m_off[i]:self.m_off[i + 1]]) for i in range(self.count)]


def device_count():
    return lib().cxg_device_count()
