"""ctypes binding of the oracle (oracle/oracle.cpp).

ORACLE -- TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg, and there only as the checker / the timed CPU restatement of the reference.
The product package (conicxx_gb300) never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from conicxx_gb300 import _abi
from conicxx_gb300._abi import Info, Settings, default_settings, dptr, iptr, make_problem_struct

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (g++ only; seconds)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.orc_create.restype = vp
        L.orc_destroy.argtypes = [vp]
        L.orc_setup.argtypes = [vp, C.POINTER(_abi.Problem), C.POINTER(Settings)]
        L.orc_update.argtypes = [vp, ip, ip, dp, dp, ip, ip, dp, dp]
        L.orc_set_warm_start.argtypes = [vp, dp, dp, dp]
        L.orc_solve.argtypes = [vp, dp, dp, dp, C.POINTER(Info)]
        L.orc_adjoint.argtypes = [vp, dp, dp, dp, dp, dp]
        L.orc_trace_len.argtypes = [vp]
        L.orc_trace.argtypes = [vp, dp]
        L.orc_equilibration.argtypes = [vp, dp, dp, dp]
        L.orc_nnz_l.argtypes = [vp]
        L.orc_kkt_solve.argtypes = [C.POINTER(_abi.Problem), C.POINTER(Settings), dp, dp, dp, dp]
        L.orc_kkt_solve.restype = C.c_double
        L.orc_cones_create.restype = vp
        L.orc_cones_create.argtypes = [C.c_int, C.c_int, C.c_int, ip]
        L.orc_cones_destroy.argtypes = [vp]
        L.orc_cones_dim.argtypes = [vp]
        L.orc_cones_degree.argtypes = [vp]
        L.orc_cones_identity.argtypes = [vp, dp]
        L.orc_cones_update_scaling.argtypes = [vp, dp, dp]
        L.orc_cones_apply.argtypes = [vp, C.c_int, dp, dp, dp]
        L.orc_cones_max_step.argtypes = [vp, dp, dp, C.c_double]
        L.orc_cones_max_step.restype = C.c_double
        L.orc_cones_margins.argtypes = [vp, dp, dp, dp]
        L.orc_cones_shift.argtypes = [vp, dp, C.c_double]
        L.orc_cones_scaling.argtypes = [vp, dp, dp, dp]
        L.orc_batch_solve.argtypes = [C.c_int, C.POINTER(_abi.Problem), C.POINTER(Settings), C.c_int, ip, ip]
        L.orc_batch_solve.restype = C.c_double
        L.orc_batch_solve_x.argtypes = [C.c_int, C.POINTER(_abi.Problem), C.POINTER(Settings), C.c_int, ip, ip,
                                        dp, dp, dp]
        L.orc_batch_solve_x.restype = C.c_double
        _lib = L
    return _lib


TRACE_COLS = ["mu", "norm_rx", "norm_rz", "pobj", "dobj", "alpha_aff", "sigma", "alpha", "tau",
              "kappa", "relres", "attempts"]


class OracleSolver:
    """conicxx::Solver semantics (include/conicxx/solver.h) on the CPU oracle."""

    def __init__(self):
        self._h = lib().orc_create()
        self.qp = None

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def setup(self, qp, settings=None, **kw):
        st = settings if settings is not None else default_settings(**kw)
        prob, keep = make_problem_struct(qp)
        ok = lib().orc_setup(self._h, C.byref(prob), C.byref(st))
        self.qp = qp
        return bool(ok)

    def update_data(self, P=None, q=None, A=None, b=None):
        keep = []

        def arr(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a

        Pp = arr(P.indptr, np.int32) if P is not None else None
        Pi = arr(P.indices, np.int32) if P is not None else None
        Px = arr(P.data, np.float64) if P is not None else None
        Ap = arr(A.indptr, np.int32) if A is not None else None
        Ai = arr(A.indices, np.int32) if A is not None else None
        Ax = arr(A.data, np.float64) if A is not None else None
        return bool(lib().orc_update(self._h, iptr(Pp), iptr(Pi), dptr(Px), dptr(arr(q, np.float64)),
                                     iptr(Ap), iptr(Ai), dptr(Ax), dptr(arr(b, np.float64))))

    def set_warm_start(self, x, s, z):
        x, s, z = (np.ascontiguousarray(v, dtype=np.float64) for v in (x, s, z))
        lib().orc_set_warm_start(self._h, dptr(x), dptr(s), dptr(z))

    def solve(self):
        n, m = self.qp.n, self.qp.m
        x, s, z = np.zeros(n), np.zeros(m), np.zeros(m)
        info = Info()
        lib().orc_solve(self._h, dptr(x), dptr(s), dptr(z), C.byref(info))
        return x, s, z, info.as_dict()

    def trace(self):
        L = lib()
        k = L.orc_trace_len(self._h)
        out = np.zeros((k, len(TRACE_COLS)))
        if k:
            L.orc_trace(self._h, dptr(out))
        return out

    def adjoint(self, dl_dx):
        """FP64 adjoint at the last Solved solution: (dL/dq, dL/db, dL/dPx, dL/dAx)."""
        qp = self.qp
        g = np.ascontiguousarray(dl_dx, dtype=np.float64)
        dq, db, dP, dA = np.zeros(qp.n), np.zeros(qp.m), np.zeros(qp.P.nnz), np.zeros(qp.A.nnz)
        if not lib().orc_adjoint(self._h, dptr(g), dptr(dq), dptr(db), dptr(dP), dptr(dA)):
            raise ValueError("adjoint needs a Solved solution")
        return dq, db, dP, dA

    def equilibration(self):
        d, e, c = np.zeros(self.qp.n), np.zeros(self.qp.m), C.c_double()
        lib().orc_equilibration(self._h, dptr(d), dptr(e), C.byref(c))
        return d, e, c.value

    def nnz_l(self):
        return lib().orc_nnz_l(self._h)


def solve(qp, settings=None, **kw):
    """One-shot oracle solve -> (x, s, z, info dict, trace)."""
    S = OracleSolver()
    if not S.setup(qp, settings, **kw):
        raise ValueError("oracle setup() returned false")
    x, s, z, info = S.solve()
    return x, s, z, info, S.trace()


def kkt_solve(qp, rhs, s=None, z=None, settings=None, **kw):
    """KktSystem::setup + optional updateScaling(s,z) + solve (reference KKT layer)."""
    st = settings if settings is not None else default_settings(equilibrate=0, **kw)
    prob, keep = make_problem_struct(qp)
    rhs = np.ascontiguousarray(rhs, dtype=np.float64)
    out = np.zeros(qp.n + qp.m)
    sa = np.ascontiguousarray(s, dtype=np.float64) if s is not None else None
    za = np.ascontiguousarray(z, dtype=np.float64) if z is not None else None
    rel = lib().orc_kkt_solve(C.byref(prob), C.byref(st), dptr(sa), dptr(za), dptr(rhs), dptr(out))
    return out, rel


class OracleCones:
    """ConeSet (include/conicxx/cones/cone_set.h) on the CPU oracle."""

    OPS = {"product": 0, "inverse_product": 1, "apply_w": 2, "apply_w_inv": 3, "mul_hs": 4}

    def __init__(self, zero, nonneg, soc):
        self.soc = np.ascontiguousarray(np.asarray(soc, np.int32).reshape(-1))
        if self.soc.size == 0:
            self.soc = np.zeros(1, np.int32)
            nsoc = 0
        else:
            nsoc = len(soc)
        self._h = lib().orc_cones_create(zero, nonneg, nsoc, iptr(self.soc))
        self.m = lib().orc_cones_dim(self._h)
        self.degree = lib().orc_cones_degree(self._h)
        self.nsoc = nsoc

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_cones_destroy(self._h)
            self._h = None

    def identity(self):
        out = np.zeros(self.m)
        lib().orc_cones_identity(self._h, dptr(out))
        return out

    def update_scaling(self, s, z):
        s, z = np.ascontiguousarray(s, np.float64), np.ascontiguousarray(z, np.float64)
        lib().orc_cones_update_scaling(self._h, dptr(s), dptr(z))

    def apply(self, op, u, v=None):
        u = np.ascontiguousarray(u, np.float64)
        v = np.ascontiguousarray(v if v is not None else u, np.float64)
        out = np.zeros(self.m)
        lib().orc_cones_apply(self._h, self.OPS[op], dptr(u), dptr(v), dptr(out))
        return out

    def max_step(self, x, dx, amax):
        x, dx = np.ascontiguousarray(x, np.float64), np.ascontiguousarray(dx, np.float64)
        return lib().orc_cones_max_step(self._h, dptr(x), dptr(dx), float(amax))

    def margins(self, x):
        x = np.ascontiguousarray(x, np.float64)
        a, b = C.c_double(), C.c_double()
        lib().orc_cones_margins(self._h, dptr(x), C.byref(a), C.byref(b))
        return a.value, b.value

    def shift(self, x, alpha):
        x = np.array(x, dtype=np.float64)
        lib().orc_cones_shift(self._h, dptr(x), float(alpha))
        return x

    def scaling(self):
        tot = int(sum(int(d) * int(d) for d in self.soc[: self.nsoc]))
        w = np.zeros(self.m)
        W, H = np.zeros(max(tot, 1)), np.zeros(max(tot, 1))
        lib().orc_cones_scaling(self._h, dptr(w), dptr(W), dptr(H))
        return w, W[:tot], H[:tot]


def batch_solve(qps, nthreads, settings=None, **kw):
    """Solve each instance on its own CPU solver with `nthreads` worker threads.
    Returns (wall seconds of the solve phase, statuses, iterations)."""
    st = settings if settings is not None else default_settings(**kw)
    structs, keeps = [], []
    for qp in qps:
        s, k = make_problem_struct(qp)
        structs.append(s)
        keeps.append(k)
    arr = (_abi.Problem * len(qps))(*structs)
    stat = np.zeros(len(qps), np.int32)
    iters = np.zeros(len(qps), np.int32)
    wall = lib().orc_batch_solve(len(qps), arr, C.byref(st), int(nthreads), iptr(stat), iptr(iters))
    return wall, stat, iters


def batch_solve_x(qps, nthreads, settings=None, **kw):
    """batch_solve plus the concatenated solutions: (wall, statuses, iterations, x, s, z)."""
    st = settings if settings is not None else default_settings(**kw)
    structs, keeps = [], []
    for qp in qps:
        s_, k = make_problem_struct(qp)
        structs.append(s_)
        keeps.append(k)
    arr = (_abi.Problem * len(qps))(*structs)
    stat = np.zeros(len(qps), np.int32)
    iters = np.zeros(len(qps), np.int32)
    x = np.zeros(sum(q.n for q in qps))
    s = np.zeros(sum(q.m for q in qps))
    z = np.zeros(sum(q.m for q in qps))
    wall = lib().orc_batch_solve_x(len(qps), arr, C.byref(st), int(nthreads), iptr(stat), iptr(iters), dptr(x),
                                   dptr(s), dptr(z))
    return wall, stat, iters, x, s, z


def perturb_q(qp, seed):
    """A copy of qp whose linear cost q is changed by a relative 2^-52 (one or two units in the
    last place), in a seeded random direction per entry (q_j (1 +- 2^-52), rounded): a change of
    the input at the rounding level of FP64."""
    import dataclasses

    rng = np.random.default_rng(seed)
    sign = rng.choice(np.array([-1.0, 1.0]), qp.n)
    return dataclasses.replace(qp, q=np.asarray(qp.q, dtype=np.float64) * (1.0 + sign * 2.0 ** -52))


def rounding_ensemble(qps, nthreads, members=4, seed=0, settings=None, **kw):
    """The oracle's own sensitivity to rounding, per instance: the batch solved as given (the
    base) and `members` more times with q perturbed at the last bit (perturb_q, seeds seed + 1 ...).

    Returns a dict:
      base: (statuses, iterations, x, s, z) of the unperturbed solves (concatenated vectors);
      statuses, iterations: (members + 1, N) arrays, row 0 the base;
      spread_x, spread_s, spread_z: per instance, the largest max-norm-relative difference
        max |v_k - v_base| / max(1, max |v_base|) over the members that Solved where the base did
        (0 where none did);
      sensitive: per instance, True when the members' statuses differ from the base's or their
        iteration counts span more than one.
    Where a last-bit change of the input moves the reference's own status, iterations or solution,
    the same movement in another implementation's result is rounding, not a difference in the
    algorithm."""
    st = settings if settings is not None else default_settings(**kw)
    n_off = np.concatenate([[0], np.cumsum([q.n for q in qps])]).astype(np.int64)
    m_off = np.concatenate([[0], np.cumsum([q.m for q in qps])]).astype(np.int64)
    runs = [batch_solve_x(qps, nthreads, settings=st)]
    for k in range(members):
        runs.append(batch_solve_x([perturb_q(q, seed + 1 + 1000003 * k + i) for i, q in enumerate(qps)], nthreads,
                                  settings=st))
    stat = np.stack([r[1] for r in runs]).astype(int)
    iters = np.stack([r[2] for r in runs]).astype(int)
    N = len(qps)
    spreads = {key: np.zeros(N) for key in ("x", "s", "z")}
    base = runs[0]
    for key, col, off in (("x", 3, n_off), ("s", 4, m_off), ("z", 5, m_off)):
        bv = base[col]
        for r_ in runs[1:]:
            rv = r_[col]
            for i in range(N):
                if stat[0, i] != 1:
                    continue
                a, b = off[i], off[i + 1]
                if b == a:
                    continue
                u, v = bv[a:b], rv[a:b]
                e = float(np.max(np.abs(u - v)) / max(1.0, float(np.max(np.abs(u)))))
                spreads[key][i] = max(spreads[key][i], e)
        # members that did not Solve where the base did: their distance is not defined; the
        # instance is then marked sensitive by its status
    sensitive = np.any(stat != stat[0], axis=0) | ((iters.max(axis=0) - iters.min(axis=0)) > 1)
    return {"base": (stat[0], iters[0], base[3], base[4], base[5]), "statuses": stat, "iterations": iters,
            "spread_x": spreads["x"], "spread_s": spreads["s"], "spread_z": spreads["z"], "sensitive": sensitive}
