"""Pins the CPU oracle to the reference's own known-answer tests (CPU only).

Each test cites the reference test it re-expresses; tolerances are the reference's.
"""
import os

import numpy as np
import pytest

from conftest import kat_qp, rel
from conicxx_gb300 import _abi
from conicxx_gb300.problem import QP, Csc


def _kkt_optimal(qp, x, s, z, tol):
    """expectKktOptimal (test/utils/test_helpers.h:32-48)."""
    st, fe, sz = qp.kkt_residuals(x, s, z)
    assert st < tol and fe < tol and abs(sz) < tol, (st, fe, sz)
    assert qp.cone_margins(s)[0] > -tol and qp.cone_margins(z)[0] > -tol


@pytest.mark.parametrize("idx", range(8))
def test_solver_kats(oracle_mod, kats, idx):
    k = kats[idx]
    qp = kat_qp(k)
    x, s, z, info, _ = oracle_mod.solve(qp)
    assert info["status"] == k["status"], (k["name"], info["status"])
    if k["x"] is not None:
        assert np.allclose(x, k["x"], atol=k["tol"]), (k["name"], x)
    if k["objective"] is not None:
        assert abs(info["objective"] - k["objective"]) < k["tol"]
    if k["status"] == 1 and k["name"] != "readme_example":
        _kkt_optimal(qp, x, s, z, k["tol"])


def test_dense_input_matches_sparse(oracle_mod, kats):
    """test/solver/test_solve_dense_input.cpp:35-71: explicit zeros of a dense conversion keep the
    same solution."""
    qp = kat_qp(kats[1])
    Pd = np.eye(2)
    Ad = -np.eye(2)
    qd = QP(Csc.from_dense(Pd, keep_zeros=True, upper=True), qp.q, Csc.from_dense(Ad, keep_zeros=True), qp.b,
            nonneg=2)
    x1 = oracle_mod.solve(qp)[0]
    x2 = oracle_mod.solve(qd)[0]
    assert np.allclose(x1, x2, atol=1e-6) and np.allclose(x2, [0, 2], atol=1e-6)


def _box(c):
    n = len(c)
    P = Csc.from_triplets(n, n, [(0, 0, 1.0), (1, 1, 1.0)])
    A = Csc.from_triplets(n, n, [(0, 0, -1.0), (1, 1, -1.0)])
    return QP(P, -np.asarray(c, float), A, np.zeros(n), nonneg=n)


def test_update_reuse_matches_fresh_setup(oracle_mod):
    """test/solver/test_update_reuse.cpp:32-73 (updateData(q) + auto warm start)."""
    targets = [(1.0, 2.0), (-1.0, 3.0), (0.5, -0.5)]
    S = oracle_mod.OracleSolver()
    assert S.setup(_box(targets[0]))
    for t, c in enumerate(targets):
        p = _box(c)
        if t > 0:
            assert S.update_data(q=p.q)
        x = S.solve()[0]
        xf = oracle_mod.solve(p)[0]
        assert np.allclose(x, xf, atol=1e-6)
        assert np.allclose(x, np.maximum(c, 0.0), atol=1e-6)


def test_pattern_mismatch_rejected(oracle_mod):
    """test/solver/test_update_reuse.cpp:75-89."""
    p = _box((1.0, 1.0))
    S = oracle_mod.OracleSolver()
    assert S.setup(p)
    A_bad = Csc.from_triplets(2, 2, [(0, 0, -1.0), (0, 1, 0.3), (1, 1, -1.0)])
    assert not S.update_data(A=A_bad)
    p2 = QP(p.P, p.q, A_bad, p.b, nonneg=2)
    assert S.setup(p2)
    assert S.solve()[3]["status"] == _abi.STATUS_SOLVED


# ---- cones (test/cones/*) -------------------------------------------------------------------
def test_soc_product_inverse_roundtrip(oracle_mod):
    """test/cones/test_second_order_cone.cpp:19-35, 37-44."""
    C = oracle_mod.OracleCones(0, 0, [4])
    u = np.array([3.0, 0.5, -0.2, 0.1])
    v = np.array([2.0, 0.3, 0.4, -0.1])
    w = C.apply("product", u, v)
    exp = np.concatenate([[u @ v], u[0] * v[1:] + v[0] * u[1:]])
    assert np.allclose(w, exp, atol=1e-13)
    assert np.allclose(C.apply("inverse_product", u, w), v, atol=1e-10)
    u2 = np.array([2.0, 0.3, -0.1, 0.4])
    assert np.allclose(C.apply("product", u2, C.identity()), u2, atol=1e-13)


def test_soc_nt_scaling_identities(oracle_mod):
    """test/cones/test_second_order_cone.cpp:46-80: Hs z = s, W^-1 s = W z, W W x = Hs x."""
    C = oracle_mod.OracleCones(0, 0, [3])
    s = np.array([3.0, 1.0, 1.0])
    z = np.array([2.0, 0.5, 0.5])
    C.update_scaling(s, z)
    assert np.allclose(C.apply("mul_hs", z), s, atol=1e-10)
    assert np.allclose(C.apply("apply_w_inv", s), C.apply("apply_w", z), atol=1e-10)
    _, W, H = C.scaling()
    assert np.allclose(H.reshape(3, 3), H.reshape(3, 3).T, atol=1e-12)
    x = np.array([0.4, -0.2, 0.7])
    assert np.allclose(C.apply("apply_w", C.apply("apply_w", x)), C.apply("mul_hs", x), atol=1e-10)


def test_soc_margin_shift_maxstep(oracle_mod):
    """test/cones/test_second_order_cone.cpp:82-119."""
    C = oracle_mod.OracleCones(0, 0, [3])
    x = np.array([3.0, 1.0, 1.0])
    assert abs(C.margins(x)[0] - (3 - np.sqrt(2))) < 1e-14
    assert np.allclose(C.shift(x, 2.0), [5.0, 1.0, 1.0], atol=1e-14)
    e = np.array([1.0, 0.0, 0.0])
    assert abs(C.max_step(e, np.array([-1.0, 0, 0]), 10.0) - 1.0) < 1e-12
    assert abs(C.max_step(e, np.array([1.0, 1.0, 0]), 10.0) - 10.0) < 1e-12
    assert abs(C.max_step(e, np.array([0.0, 1.0, 0]), 10.0) - 1.0) < 1e-12


def test_nonnegative_cone(oracle_mod):
    """test/cones/test_nonnegative_cone.cpp:9-71."""
    C = oracle_mod.OracleCones(0, 4, [])
    u, v = np.array([1.0, 2, 3, 4]), np.array([5.0, 6, 7, 8])
    w = C.apply("product", u, v)
    assert np.allclose(w, u * v, atol=1e-14)
    assert np.allclose(C.apply("inverse_product", u, w), v, atol=1e-12)
    s, z = np.array([1.0, 4, 0.5, 9]), np.array([2.0, 1, 2, 3])
    C.update_scaling(s, z)
    assert np.allclose(C.apply("mul_hs", z), s, atol=1e-12)
    assert np.allclose(C.apply("apply_w_inv", s), C.apply("apply_w", z), atol=1e-12)
    C3 = oracle_mod.OracleCones(0, 3, [])
    assert C3.margins(np.array([-1.0, 2, 0.5]))[0] == -1.0
    assert np.allclose(C3.shift(np.array([-1.0, 2, 0.5]), 2.0), [1, 4, 2.5])
    assert abs(C3.max_step(np.array([1.0, 2, 3]), np.array([-2.0, -1, 5]), 10.0) - 0.5) < 1e-14


def test_zero_cone_and_cone_set(oracle_mod):
    """test/cones/test_zero_cone.cpp:7-58, test/cones/test_cone_set.cpp:12-94."""
    Z = oracle_mod.OracleCones(3, 0, [])
    x = np.array([0.3, -1.0, 2.0])
    assert np.allclose(Z.apply("product", x, x), 0) and np.allclose(Z.apply("apply_w", x), 0)
    assert Z.max_step(x, x, 0.73) == 0.73
    L = oracle_mod.OracleCones(2, 3, [3, 4])
    assert L.m == 12 and L.degree == 5
    I = oracle_mod.OracleCones(1, 2, [3])
    assert np.allclose(I.identity(), [0, 1, 1, 1, 0, 0])
    s = np.array([0.0, 1, 4, 3, 1, 1])
    z = np.array([0.0, 2, 1, 2, 0.5, 0.5])
    I.update_scaling(s, z)
    out = I.apply("mul_hs", z)
    assert abs(out[0]) < 1e-14 and np.allclose(out[1:], s[1:], atol=1e-10)
    M = oracle_mod.OracleCones(2, 2, [])
    assert M.margins(np.array([100.0, -100, -1, 3])) == (-1.0, 0.0)
    M2 = oracle_mod.OracleCones(0, 2, [3, 3])
    mn, pos = M2.margins(np.array([1.0, 2, 3, 1, 1, 0.5, 0.4, 0.4]))
    ms = [1.0, 3 - np.sqrt(2), 0.5 - np.sqrt(0.32)]
    assert abs(mn - min(ms)) < 1e-12 and abs(pos - sum(max(v, 0) for v in ms)) < 1e-12


# ---- KKT (test/kkt/test_kkt_system.cpp) ------------------------------------------------------
def _dense_k(Pd, Ad, Hs, regP=1e-8, regA=1e-8):
    n, m = Pd.shape[0], Ad.shape[0]
    K = np.zeros((n + m, n + m))
    K[:n, :n] = Pd + regP * np.eye(n)
    K[:n, n:] = Ad.T
    K[n:, :n] = Ad
    K[n:, n:] = -Hs - regA * np.eye(m)
    return K


def test_kkt_matches_dense_reference(oracle_mod):
    """test/kkt/test_kkt_system.cpp:32-92."""
    P = Csc.from_triplets(2, 2, [(0, 0, 2.0), (1, 1, 3.0)])
    A = Csc.from_triplets(2, 2, [(0, 0, 1.0), (1, 1, 1.0)])
    qp = QP(P, np.zeros(2), A, np.zeros(2), nonneg=2)
    rhs = np.array([1.0, 2, 3, 4])
    x, relres = oracle_mod.kkt_solve(qp, rhs)
    K = _dense_k(np.diag([2.0, 3]), np.eye(2), np.eye(2))
    assert relres < 1e-10 and np.allclose(x, np.linalg.solve(K, rhs), atol=1e-8)
    s, z = np.array([4.0, 9.0]), np.array([1.0, 1.0])
    rhs2 = np.array([1.0, -1, 0.5, 2])
    x2, _ = oracle_mod.kkt_solve(qp, rhs2, s=s, z=z)
    K2 = _dense_k(np.diag([2.0, 3]), np.eye(2), np.diag(s / z))
    assert np.allclose(x2, np.linalg.solve(K2, rhs2), atol=1e-8)


def test_kkt_rank_deficient_equalities(oracle_mod):
    """test/kkt/test_kkt_system.cpp:137-158."""
    P = Csc.from_triplets(2, 2, [(0, 0, 1.0), (1, 1, 1.0)])
    A = Csc.from_triplets(2, 2, [(0, 0, 1.0), (0, 1, 1.0), (1, 0, 1.0), (1, 1, 1.0)])
    qp = QP(P, np.zeros(2), A, np.zeros(2), zero=2)
    x, relres = oracle_mod.kkt_solve(qp, np.array([1.0, 1, 0, 0]))
    assert np.all(np.isfinite(x)) and relres < 1e-6


# ---- equilibration (test/kkt/test_equilibration.cpp) -----------------------------------------
def test_equilibration_roundtrip_and_soc_uniform(oracle_mod):
    """test/kkt/test_equilibration.cpp:11-110."""
    P = Csc.from_triplets(3, 3, [(0, 0, 1e6), (1, 1, 1e-4), (2, 2, 50.0)])
    A = Csc.from_triplets(4, 3, [(0, 0, 1e5), (1, 1, 1e-3), (2, 2, 20.0), (3, 0, 1e5), (3, 1, 1e-3), (3, 2, 20.0)])
    qp = QP(P, np.array([3.0, -2, 1]), A, np.array([1.0, 2, 3, 4]), zero=1, nonneg=3)
    S = oracle_mod.OracleSolver()
    assert S.setup(qp)
    d, e, c = S.equilibration()
    assert np.all(d > 0) and np.all(e > 0) and c > 0
    S2 = oracle_mod.OracleSolver()
    assert S2.setup(qp, equilibrate=0)
    d2, e2, c2 = S2.equilibration()
    assert np.allclose(d2, 1) and np.allclose(e2, 1) and c2 == 1.0
    P3 = Csc.from_triplets(3, 3, [(0, 0, 1.0), (1, 1, 1.0), (2, 2, 1.0)])
    A3 = Csc.from_triplets(3, 3, [(0, 0, 100.0), (1, 1, 1.0), (2, 2, 0.01)])
    S3 = oracle_mod.OracleSolver()
    assert S3.setup(QP(P3, np.zeros(3), A3, np.zeros(3), soc=[3]))
    e3 = S3.equilibration()[1]
    assert abs(e3[0] - e3[1]) < 1e-12 and abs(e3[1] - e3[2]) < 1e-12


def test_golden_instances_reproduce(oracle_mod, golden_instances):
    """The oracle re-solves the committed golden instances to the committed results."""
    for name, qp, exp in golden_instances:
        x, s, z, info, _ = oracle_mod.solve(qp)
        assert info["status"] == exp["status"] and info["iterations"] == exp["iterations"], name
        assert rel(x, exp["x"]) < 1e-9, name


def test_oracle_adjoint_closed_form(oracle_mod, kats):
    """The FP64 adjoint (new; no reference counterpart) on the equality QP of
    test/solver/test_solve_qp.cpp:9-34, whose solution map is affine: x = -q + (b+q0+q1)/2 (1,1)."""
    qp = kat_qp(kats[0])
    S = oracle_mod.OracleSolver()
    assert S.setup(qp)
    x, s, z, info = S.solve()
    t = np.array([0.3, -1.2])
    g = x - t
    dq, db, dP, dA = S.adjoint(g)
    J = -np.eye(2) + 0.5 * np.ones((2, 2))
    assert np.allclose(dq, J @ g, atol=1e-7) and np.allclose(db, [0.5 * g.sum()], atol=1e-7)
    # dL/dP (upper diagonal entries): -(u_i x_i) with u = -dq
    assert np.allclose(dP, -(-dq) * x, atol=1e-7)


def test_oracle_rounding_ensemble_moves_statuses():
    """The rounding ensemble used by the full-batch parity tests: the perturbations of q change each
    entry by a relative 2^-52 (one or two units in its last place), and on 512 instances of the contact family they move the
    oracle's own status or iteration count on some instances (the reference's rounding
    sensitivity the device results are measured against)."""
    import oracle as orc
    from conicxx_gb300 import generators

    orc.build()
    qps = generators.contact_batch(512)
    q2 = orc.perturb_q(qps[0], 7)
    assert np.all(np.abs(q2.q - qps[0].q) <= 2.0 * np.spacing(np.abs(qps[0].q)))
    assert np.any(q2.q != qps[0].q)
    E = orc.rounding_ensemble(qps, os.cpu_count() or 1, members=2, warm_start=0)
    assert E["statuses"].shape == (3, 512) and E["spread_x"].shape == (512,)
    assert E["sensitive"].sum() >= 1
    assert np.all(E["spread_x"][E["statuses"][0] == 1] < 1e-3)
