"""GPU parity tests: the CUDA path (through the C-ABI) against the CPU oracle and the reference's
known answers.

Criteria (FP64 oracle as the reference): same status; iteration count within +-1 (a GPU count
lower than the oracle's by more is reported, as the reduced-KKT factorisation can converge
where the reference's numerics stall); solutions within the stated relative tolerance; primal
and dual residuals within tol_feas for Solved instances.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import kat_qp, rel
from conicxx_gb300 import _abi, _lib, generators
from conicxx_gb300._abi import dptr, iptr
from conicxx_gb300.problem import sym_upper_matvec

pytestmark = pytest.mark.gpu

# Relative tolerance of GPU vs FP64-oracle solutions. Both runs stop at the 1e-8 residual/gap
# tests, so their final iterates differ by what that stopping rule leaves undetermined: measured
# up to ~2e-6 for x and ~2e-5 for the duals z (and s) on the contact instances.
X_TOL = 1e-5
SZ_TOL = 1e-4


def _solvers():
    from conicxx_gb300 import BatchSolver, Solver

    return Solver, BatchSolver


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if _lib.lib().cxg_device_count() < 1:
        pytest.fail("a CUDA device is required for the -m gpu tests")


# ---- reference known-answer tests ------------------------------------------------------------
@pytest.mark.parametrize("linear_solver", [_abi.LINSOLVER_EIGEN, _abi.LINSOLVER_QDLDL, _abi.LINSOLVER_REGULARIZED])
@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
@pytest.mark.parametrize("idx", range(8))
def test_kats(kats, idx, precision, linear_solver):
    """Every known-answer problem, in both precisions and with each LinearSolverBackend value
    (the reference runs its KKT tests over all three, test/kkt/test_kkt_system_backends.cpp:32-135)."""
    Solver, _ = _solvers()
    k = kats[idx]
    qp = kat_qp(k)
    S = Solver()
    assert S.setup(qp, precision=precision, linear_solver=linear_solver)
    sol = S.solve()
    assert sol.status == k["status"], (k["name"], sol.status_name)
    if k["x"] is not None:
        assert np.allclose(sol.x, k["x"], atol=k["tol"]), (k["name"], sol.x)
    if k["objective"] is not None:
        assert abs(sol.objective - k["objective"]) < k["tol"]
    if k["status"] == _abi.STATUS_SOLVED:
        st, fe, sz = qp.kkt_residuals(sol.x, sol.s, sol.z)
        tol = max(k["tol"], 1e-6)
        assert st < tol and fe < tol and abs(sz) < tol


def test_kats_as_one_batch(kats):
    """All known-answer problems in one batched launch (mixed sizes and cone types)."""
    _, BatchSolver = _solvers()
    qps = [kat_qp(k) for k in kats]
    B = BatchSolver(qps)
    x, s, z, infos = B.solve()
    for i, (xi, si, zi) in enumerate(B.split(x, s, z)):
        k = kats[i]
        assert infos[i]["status"] == k["status"], k["name"]
        if k["x"] is not None:
            assert np.allclose(xi, k["x"], atol=k["tol"]), k["name"]


def _box(c):
    from conicxx_gb300.problem import QP, Csc

    n = len(c)
    P = Csc.from_triplets(n, n, [(0, 0, 1.0), (1, 1, 1.0)])
    A = Csc.from_triplets(n, n, [(0, 0, -1.0), (1, 1, -1.0)])
    return QP(P, -np.asarray(c, float), A, np.zeros(n), nonneg=n)


def test_update_reuse_and_pattern_mismatch():
    """test/solver/test_update_reuse.cpp:32-89 through the C-ABI."""
    from conicxx_gb300.problem import QP, Csc

    Solver, _ = _solvers()
    targets = [(1.0, 2.0), (-1.0, 3.0), (0.5, -0.5)]
    S = Solver()
    assert S.setup(_box(targets[0]))
    for t, c in enumerate(targets):
        p = _box(c)
        if t > 0:
            assert S.update_data(q=p.q)
        sol = S.solve()
        assert sol.ok()
        F = Solver()
        assert F.setup(p)
        assert np.allclose(sol.x, F.solve().x, atol=1e-6)
        assert np.allclose(sol.x, np.maximum(c, 0), atol=1e-6)
    A_bad = Csc.from_triplets(2, 2, [(0, 0, -1.0), (0, 1, 0.3), (1, 1, -1.0)])
    assert not S.update_data(A=A_bad)
    assert S.setup(QP(_box((1.0, 1.0)).P, -np.ones(2), A_bad, np.zeros(2), nonneg=2))
    assert S.solve().ok()


def test_warm_start_and_update_data_matrices(oracle_mod):
    """updateData of P and A values (same pattern) and an explicit setWarmStart against the oracle."""
    Solver, _ = _solvers()
    qp = generators.contact_qp(21, contacts=12)
    qp2 = generators.contact_qp(22, contacts=12)
    S = Solver()
    assert S.setup(qp)
    assert S.solve().ok()
    if np.array_equal(qp.P.indptr, qp2.P.indptr) and np.array_equal(qp.P.indices, qp2.P.indices):
        assert S.update_data(P=qp2.P, q=qp2.q)
    else:
        assert not S.update_data(P=qp2.P)  # pattern differs: rejected, like the reference
    O = oracle_mod.OracleSolver()
    assert O.setup(qp)
    xo, so, zo, _ = O.solve()
    S2 = Solver()
    assert S2.setup(qp)
    S2.set_warm_start(xo, so, zo)
    O2 = oracle_mod.OracleSolver()
    O2.setup(qp)
    O2.set_warm_start(xo, so, zo)
    sol = S2.solve()
    x2, _, _, i2 = O2.solve()
    assert sol.ok() and i2["status"] == 1
    assert abs(sol.info["iterations"] - i2["iterations"]) <= 1
    assert rel(sol.x, x2) < X_TOL


# ---- device cone algebra against the oracle --------------------------------------------------
def _interior(rng, zero, nn, soc, near=None):
    parts = [np.zeros(zero), rng.uniform(0.2, 2.0, nn)]
    for d in soc:
        u1 = rng.standard_normal(d - 1)
        gap = rng.uniform(0.05, 1.0) if near is None else near
        parts.append(np.concatenate([[np.linalg.norm(u1) + gap], u1]))
    return np.concatenate(parts)


def _cones_eval(op, zero, nn, soc, s, z, u, v=None, a=0.0):
    m = zero + nn + sum(soc)
    socs = np.asarray(soc if soc else [1], np.int32)
    out, sc, par = np.zeros(m), np.zeros(2), np.zeros(8 * max(len(soc), 1))
    vv = np.ascontiguousarray(v if v is not None else u, dtype=np.float64)
    s, z, u = (np.ascontiguousarray(t, dtype=np.float64) for t in (s, z, u))
    rc = _lib.lib().cxg_cones_eval(op, zero, nn, len(soc), iptr(socs), dptr(s), dptr(z), dptr(u), dptr(vv), a,
                                   dptr(out), dptr(sc), dptr(par))
    assert rc == 0, _lib.lib().cxg_last_error()
    return out, sc, par


@pytest.mark.parametrize("soc", [[3] * 6, [2, 4, 17, 3], [1, 3, 5]])
@pytest.mark.parametrize("near", [None, 1e-4, 1e-9])
def test_cone_algebra_matches_oracle(oracle_mod, soc, near):
    rng = np.random.default_rng(len(soc) * 7 + (0 if near is None else int(-np.log10(near))))
    zero, nn = 2, 5
    C_ = oracle_mod.OracleCones(zero, nn, soc)
    s = _interior(rng, zero, nn, soc, near)
    z = _interior(rng, zero, nn, soc, near)
    u = rng.standard_normal(len(s))
    v = rng.standard_normal(len(s))
    C_.update_scaling(s, z)
    _, Wcat, _ = C_.scaling()
    conds, off = [1.0], 0
    for d in soc:
        conds.append(np.linalg.cond(Wcat[off:off + d * d].reshape(d, d)))
        off += d * d
    cond = max(conds)
    # the scaling starts from a = sqrt(s0^2 - |s1|^2) and b = sqrt(z0^2 - |z1|^2): near the cone's
    # boundary the subtraction cancels, and each implementation's a, b carry a relative rounding
    # error of about eps x s0^2 / (s0^2 - |s1|^2) (different for each, as their operation orders
    # and fused multiply-adds differ)
    kap, off = 1.0, zero + nn
    for d in soc:
        for w in (s[off:off + d], z[off:off + d]):
            kap = max(kap, w[0] ** 2 / max(abs(w[0] ** 2 - w[1:] @ w[1:]), 1e-300))
        off += d
    for op, name in [(0, "apply_w"), (1, "apply_w_inv"), (2, "mul_hs")]:
        g = _cones_eval(op, zero, nn, soc, s, z, u)[0]
        o = C_.apply(name, u)
        scale = max(np.abs(o).max(), 1e-300)
        # the device eigen-form vs the oracle's dense W, W*W and LU(W): both are FP64-exact up to
        # the conditioning of W, so they agree to ~cond(W)^2 * eps relative to the result's size,
        # plus the cancellation in a and b above
        tol = 1e-12 + 1e-15 * cond * cond + 1e-15 * kap
        assert np.abs(g - o).max() / scale < tol, (name, np.abs(g - o).max(), scale, cond, kap)
    # the inverse Jordan product divides by rho = u0^2 - |u1|^2: its conditioning is u0^2/|rho|
    cond_ip, off = 1.0, zero + nn
    for d in soc:
        ub = s[off:off + d]
        cond_ip = max(cond_ip, ub[0] ** 2 / max(abs(ub[0] ** 2 - ub[1:] @ ub[1:]), 1e-300))
        off += d
    for op, name, tol in [(3, "product", 1e-12), (4, "inverse_product", 1e-12 * cond_ip)]:
        g = _cones_eval(op, zero, nn, soc, s, z, s, v)[0]
        o = C_.apply(name, s, v)
        assert np.abs(g - o).max() <= tol * max(np.abs(o).max(), 1.0), (name, np.abs(g - o).max(), cond_ip)
    dx = rng.standard_normal(len(s))
    g = _cones_eval(5, zero, nn, soc, s, z, s, dx, 10.0)[1][0]
    assert abs(g - C_.max_step(s, dx, 10.0)) <= 1e-12 * max(1.0, abs(g))
    g = _cones_eval(6, zero, nn, soc, s, z, u)[1]
    mn, pos = C_.margins(u)
    assert abs(g[0] - mn) < 1e-12 and abs(g[1] - pos) < 1e-12


def test_cone_kats_on_device():
    """test/cones/test_second_order_cone.cpp:46-119 and test_nonnegative_cone.cpp:33-71 on the
    device cone functions."""
    s, z = np.array([3.0, 1.0, 1.0]), np.array([2.0, 0.5, 0.5])
    assert np.allclose(_cones_eval(2, 0, 0, [3], s, z, z)[0], s, atol=1e-10)  # Hs z = s
    assert np.allclose(_cones_eval(1, 0, 0, [3], s, z, s)[0], _cones_eval(0, 0, 0, [3], s, z, z)[0], atol=1e-10)
    e = np.array([1.0, 0, 0])
    for dx, exp in [((-1.0, 0, 0), 1.0), ((1.0, 1.0, 0), 10.0), ((0.0, 1.0, 0), 1.0)]:
        assert abs(_cones_eval(5, 0, 0, [3], e, e, e, np.array(dx), 10.0)[1][0] - exp) < 1e-12
    sn, zn = np.array([1.0, 4, 0.5, 9]), np.array([2.0, 1, 2, 3])
    assert np.allclose(_cones_eval(2, 0, 4, [], sn, zn, zn)[0], sn, atol=1e-12)
    x, dxn = np.array([1.0, 2, 3]), np.array([-2.0, -1, 5])
    assert abs(_cones_eval(5, 0, 3, [], x, x, x, dxn, 10.0)[1][0] - 0.5) < 1e-14


def test_cone_identity_fallback_on_device(oracle_mod):
    """Degenerate SOC blocks take the identity scaling exactly like second_order_cone.cpp:152-156."""
    s = np.array([1.0, 1.0 - 1e-13, 0.0])  # numerically on the boundary
    z = np.array([1e-3, 0.0, 0.0])
    C_ = oracle_mod.OracleCones(0, 0, [3])
    C_.update_scaling(s, z)
    _, W, _ = C_.scaling()
    u = np.array([0.3, -0.7, 1.1])
    out, _, par = _cones_eval(0, 0, 0, [3], s, z, u)
    if np.allclose(W.reshape(3, 3), np.eye(3)):
        assert par[0] == 0.0 and np.allclose(out, u)
    assert rel(out, C_.apply("apply_w", u)) < 1e-6


# ---- instances: golden fixtures and live oracle ----------------------------------------------
@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
def test_golden_instances(golden_instances, precision):
    Solver, _ = _solvers()
    for name, qp, exp in golden_instances:
        S = Solver()
        assert S.setup(qp, precision=precision)
        sol = S.solve()
        assert sol.status == exp["status"], (name, sol.status_name)
        assert abs(sol.info["iterations"] - exp["iterations"]) <= 1, (name, sol.info["iterations"], exp["iterations"])
        for a, b, tol in ((sol.x, exp["x"], X_TOL), (sol.s, exp["s"], SZ_TOL), (sol.z, exp["z"], SZ_TOL)):
            assert rel(a, b) < tol, (name, rel(a, b))
        assert sol.info["primal_residual"] < 1e-8 and sol.info["dual_residual"] < 1e-8


@pytest.mark.parametrize("family", ["contact", "cfg3"])
def test_batch_against_live_oracle(oracle_mod, family):
    _, BatchSolver = _solvers()
    if family == "contact":
        qps = [generators.contact_qp(1000 + i) for i in range(48)]
    else:
        qps = [generators.config3_qp(100 + i) for i in range(16)]
    B = BatchSolver(qps)
    x, s, z, infos = B.solve()
    diffs = []
    for i, (xi, si, zi) in enumerate(B.split(x, s, z)):
        xo, so, zo, io, _ = oracle_mod.solve(qps[i])
        assert infos[i]["status"] == io["status"], (i, infos[i]["status"], io["status"])
        diffs.append(int(infos[i]["iterations"]) - io["iterations"])
        if io["status"] == 1:
            assert rel(xi, xo) < X_TOL, (i, rel(xi, xo))
    diffs = np.array(diffs)
    assert np.all(diffs <= 1), diffs
    assert np.mean(np.abs(diffs) <= 1) >= 0.9, diffs


def test_full_size_contact_batch_properties():
    """4096 contact instances (c ~ U{4..64}): size-independent properties of every result --
    definite statuses, and for Solved instances the original problem's KKT conditions, cone
    membership of s and z, and the reported residuals within tolerance."""
    _, BatchSolver = _solvers()
    qps = generators.contact_batch(4096)
    B = BatchSolver(qps, warm_start=0)
    x, s, z, infos = B.solve()
    st = infos["status"]
    assert set(np.unique(st)) <= {1, 4}
    assert np.mean(st == 1) > 0.99
    for i, (xi, si, zi) in enumerate(B.split(x, s, z)):
        if st[i] != 1:
            continue
        qp = qps[i]
        a, b, c = qp.kkt_residuals(xi, si, zi)
        scale = 1.0 + np.abs(qp.q).max()
        obj = abs(infos[i]["objective"])
        # stationarity/feasibility absolute; complementarity relative to the objective (the
        # stopping rule is a relative gap, src/conicxx/solver_impl.cpp checkConvergence)
        assert a < 1e-5 * scale and b < 1e-5 * scale and abs(c) < 1e-6 * max(1.0, obj), (i, a, b, c, obj)
        assert qp.cone_margins(si)[0] > -1e-7 and qp.cone_margins(zi)[0] > -1e-7
    ok = st == 1
    assert np.all(infos["primal_residual"][ok] < 1e-8) and np.all(infos["dual_residual"][ok] < 1e-8)


@pytest.fixture(scope="module")
def contact_ensemble(oracle_mod):
    """The 4096-instance contact batch on the oracle, as given and with q moved at the last bit in four
    seeded directions (oracle.rounding_ensemble): the reference's own status, iterations and
    solution, and how far each moves under a change of the input at the rounding level."""
    qps = generators.contact_batch(4096)
    E = oracle_mod.rounding_ensemble(qps, os.cpu_count() or 1, members=4, warm_start=0)
    return qps, E


def _max_rel(a, b):
    return float(np.max(np.abs(a - b)) / max(1.0, float(np.max(np.abs(b))))) if len(b) else 0.0


@pytest.mark.parametrize("precision", [_abi.PRECISION_MIXED, _abi.PRECISION_FP64])
def test_full_size_contact_batch_agrees_with_oracle(contact_ensemble, precision):
    """The 4096-instance contact batch against the oracle on every instance, measured against the
    reference's own rounding sensitivity. On this family a last-bit change of q (or compiling the
    reference with fused multiply-adds) moves the reference's own status on about ten instances,
    its iteration count by more than one on about 3% and its x beyond 1e-6 on about 5% (measured
    on the CPU): P = J Minv J' + 1e-6 I is rank deficient up to the shift, many contacts sit at
    the friction cone's apex with a vanishing normal force, and instances whose last iterates sit
    at the 1e-8 tolerance are Solved or run to MaxIterations as the rounding falls. An instance is
    rounding-sensitive when any of four last-bit perturbations of its q changes the oracle's status
    or moves its iterations by more than one (about 250 of the 4096). Asserted:
    - status: equal to the oracle's on every instance that is not rounding-sensitive, up to the
      number of status changes one perturbation alone makes (its mean over the four);
    - iterations within +-1 on every instance both solve that is not rounding-sensitive, up to 1%
      of them (the reference built with fused multiply-adds misses this on 0.5%);
    - x, s and z on every instance both solve: within max(1e-6, 10 x the oracle's own spread over
      the perturbations) of the oracle's, max-norm relative, or else the device's (x, s, z) is a
      solution of the original problem of the oracle's quality: stationarity and feasibility
      within 1e-6 of the data's scale, s'z within 10 x the oracle's own or 1e-7 of the objective.
      (The reference built with fused multiply-adds needs the second form on 3 instances for x
      and on 23 for z, whose duals are not unique where a normal force vanishes.)"""
    _, BatchSolver = _solvers()
    qps, E = contact_ensemble
    B = BatchSolver(qps, warm_start=0, precision=precision)
    x, s, z, infos = B.solve()
    st, it = infos["status"].astype(int), infos["iterations"].astype(int)
    ost, oit, ox, os_, oz = E["base"]
    sens = E["sensitive"]
    member_flips = [int(np.sum(E["statuses"][k] != ost)) for k in range(1, E["statuses"].shape[0])]
    mism = np.where(st != ost)[0]
    outside = [int(i) for i in mism if not sens[i]]
    print("rounding-sensitive instances: %d; oracle status changes per last-bit perturbation: %s"
          % (int(sens.sum()), member_flips))
    print("status mismatches: %d (%d outside the sensitive set: %s)" % (len(mism), len(outside), outside))
    assert len(outside) <= int(np.ceil(np.mean(member_flips))), outside
    both = (st == 1) & (ost == 1)
    d = it - oit
    ns = both & ~sens
    bad_it = np.where(ns & (np.abs(d) > 1))[0]
    print("iterations within +-1 on %d of %d non-sensitive instances both solve; exact on %.4f"
          % (int(ns.sum()) - len(bad_it), int(ns.sum()), float(np.mean(d[ns] == 0))))
    assert len(bad_it) <= 0.01 * ns.sum(), bad_it[:20]
    gs, os2 = B.split(x, s, z), B.split(ox, os_, oz)
    errs = {"x": [], "s": [], "z": []}
    kkt_route = {"x": [], "s": [], "z": []}
    failed = []
    for i in np.where(both)[0]:
        beyond = []
        for k, key in enumerate(("x", "s", "z")):
            e = _max_rel(gs[i][k], os2[i][k])
            errs[key].append(e)
            if e > max(1e-6, 10.0 * E["spread_" + key][i]):
                beyond.append(key)
        if not beyond:
            continue
        g_res = qps[i].kkt_residuals(*gs[i])
        o_res = qps[i].kkt_residuals(*os2[i])
        scale = max(1.0, np.linalg.norm(qps[i].q), np.linalg.norm(qps[i].b))
        obj = abs(float(0.5 * gs[i][0] @ sym_upper_matvec(qps[i].P, gs[i][0]) + qps[i].q @ gs[i][0]))
        ok = (g_res[0] < 1e-6 * scale and g_res[1] < 1e-6 * scale
              and abs(g_res[2]) <= max(10.0 * abs(o_res[2]), 1e-7 * max(1.0, obj)))
        for key in beyond:
            kkt_route[key].append(int(i))
        if not ok:
            failed.append((int(i), beyond, g_res, o_res))
    for k, v in errs.items():
        v = np.array(v)
        print("%s vs oracle over %d instances: median %.2e p99 %.2e max %.2e, <= 1e-6: %.4f; beyond the rounding "
              "bound (checked as KKT points): %d %s" % (k, v.size, np.median(v), np.percentile(v, 99), v.max(),
                                                       np.mean(v <= 1e-6), len(kkt_route[k]), kkt_route[k][:8]))
    assert not failed, failed[:10]


@pytest.mark.parametrize("precision", [_abi.PRECISION_MIXED, _abi.PRECISION_FP64])
def test_layer_batch_agrees_with_oracle(oracle_mod, precision):
    """The 1024-instance differentiable-layer batch (n=100, m=150, Zero^10 x R^100_+ x 10 Q^4)
    against the oracle: same status on >= 99%, iterations within +-1 on >= 95% of the instances
    both solve."""
    _, BatchSolver = _solvers()
    qps = generators.config3_batch(1024)
    B = BatchSolver(qps, warm_start=0, precision=precision)
    _, _, _, infos = B.solve()
    st, it = infos["status"], infos["iterations"]
    _, ost, oit = oracle_mod.batch_solve(qps, os.cpu_count() or 1, warm_start=0)
    agree = st == ost
    print("layer batch: status agreement %d/%d" % (agree.sum(), len(qps)))
    assert agree.mean() >= 0.99, (agree.sum(), np.where(~agree)[0][:20])
    both = agree & (st == 1)
    d = it[both] - oit[both]
    assert np.mean(np.abs(d) <= 1) >= 0.95, dict(zip(*np.unique(d, return_counts=True)))


def test_autotune_keeps_results():
    """After cxg_batch_autotune picks the launch shapes, a solve gives the same statuses and
    solutions to solver precision (the dense solves split their dot products by block size, so
    the last bits may differ)."""
    _, BatchSolver = _solvers()
    qps = generators.contact_batch(256, base_seed=5000)
    B = BatchSolver(qps, warm_start=0)
    x0, s0, z0, i0 = B.solve()
    rep = B.autotune(trials=2)
    assert rep.count("bucket") == len(B.describe().strip().splitlines()), rep
    x1, s1, z1, i1 = B.solve()
    same = i0["status"] == i1["status"]
    assert same.mean() >= 0.99
    ok = same & (i0["status"] == 1)
    for i in np.where(ok)[0]:
        a, b = B.split(x0, s0, z0)[i][0], B.split(x1, s1, z1)[i][0]
        assert np.max(np.abs(a - b)) <= 1e-5 * max(1.0, np.max(np.abs(b))), i


def test_dense_input_setup_solves_readme_example():
    """The README example through the dense-input setup (P and A as numpy arrays, every entry
    explicit as the reference's toSparse keeps them): x = (0.5, 0.5, sqrt(0.5))."""
    from conicxx_gb300 import Solver

    S = Solver()
    A = np.array([[1.0, 1, 0], [0, 0, -1], [0, 0, -1], [-1, 0, 0], [0, -1, 0]])
    assert S.setup_dense(np.eye(3), np.array([-1.0, -1, -0.3]), A, np.array([1.0, 0, 0, 0, 0]), zero=1, nonneg=1,
                         soc=[3])
    sol = S.solve()
    assert sol.ok(), sol.status_name
    assert np.allclose(sol.x, [0.5, 0.5, np.sqrt(0.5)], atol=1e-6), sol.x


def test_history_ordered_queues_keep_results():
    """The bucket queues are re-ordered after every solve (the instances that ran longest go
    first); each instance's arithmetic does not depend on its place in the queue, so repeated
    solves of the same values give the same bits, iterations and statuses."""
    _, BatchSolver = _solvers()
    qps = generators.contact_batch(512, base_seed=9000)
    B = BatchSolver(qps, warm_start=0)
    x0, s0, z0, i0 = B.solve()
    x1, s1, z1, i1 = B.solve()  # queue order now from the first solve's iteration counts
    x2, s2, z2, i2 = B.solve()
    for xa, sa, za, ia in ((x1, s1, z1, i1), (x2, s2, z2, i2)):
        assert np.array_equal(ia["status"], i0["status"]) and np.array_equal(ia["iterations"], i0["iterations"])
        assert np.array_equal(xa, x0) and np.array_equal(sa, s0) and np.array_equal(za, z0)


@pytest.mark.parametrize("whole_gpu_root", [-1, 1])
@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
def test_larger_instance_root_in_scratch(oracle_mod, precision, whole_gpu_root):
    """One instance with a 550-row root (n = 500, m = 600: Zero^50 x R^400_+ x 50 Q^3): the root
    and its factor live in the CTA's scratch rather than shared memory, and the triangular solve
    takes its block-parallel form (more than six tiles); with whole_gpu_root = 1 the root is
    spread over every SM instead. Same status as the oracle, iterations within +-1, x within 1e-6
    relative."""
    from conicxx_gb300 import Solver

    qp = generators.random_conic_qp(3, n=500, m_zero=50, m_nonneg=400, soc=(3,) * 50, density=0.02)
    S = Solver()
    assert S.setup(qp, precision=precision, warm_start=0, whole_gpu_root=whole_gpu_root)
    sol = S.solve()
    xo, _, _, io, _ = oracle_mod.solve(qp, warm_start=0)
    assert sol.status == io["status"] == 1
    assert abs(sol.info["iterations"] - io["iterations"]) <= 1
    assert np.max(np.abs(sol.x - xo)) <= 1e-6 * max(1.0, np.max(np.abs(xo)))


@pytest.mark.parametrize("linear_solver", [_abi.LINSOLVER_QDLDL, _abi.LINSOLVER_REGULARIZED])
@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
def test_rank_deficient_equalities_stay_finite(oracle_mod, precision, linear_solver):
    """A rank-deficient Zero-cone block (two identical equality rows, the case of
    test/kkt/test_kkt_system.cpp:137-158) inside a full solve: regularisation keeps every KKT solve
    finite, and the consistent system is Solved as by the oracle."""
    from conicxx_gb300 import Solver
    from conicxx_gb300.problem import QP, Csc

    P = Csc.from_triplets(3, 3, [(0, 0, 1.0), (1, 1, 1.0), (2, 2, 1.0)])
    A = Csc.from_triplets(4, 3, [(0, 0, 1.0), (0, 1, 1.0), (1, 0, 1.0), (1, 1, 1.0), (2, 2, -1.0), (3, 0, -1.0)])
    qp = QP(P, np.array([-1.0, 0.5, 0.2]), A, np.array([1.0, 1.0, 0.0, 0.0]), 2, 2, [])
    S = Solver()
    assert S.setup(qp, precision=precision, linear_solver=linear_solver)
    sol = S.solve()
    xo, _, _, io, _ = oracle_mod.solve(qp, linear_solver=linear_solver)
    assert sol.status == io["status"] == _abi.STATUS_SOLVED
    assert np.all(np.isfinite(sol.x)) and np.allclose(sol.x, xo, atol=1e-6)
