"""GPU tests of backward(): the adjoint of the KKT conditions at the solution (one extra KKT
solve with the saved final factorisation).

Checked against (i) the closed-form gradient of the equality-constrained QP of the reference's
test suite, (ii) the FP64 oracle's adjoint computed with its own CPU factorisation at its own
solution, (iii) central finite differences of the oracle's forward map, and (iv) the torch
autograd layer end to end. Gradient vectors are compared by relative 2-norm.

The adjoint is evaluated at the final interior iterate, where the NT scaling still smooths every
degenerate cone: at the default 1e-8 tolerance it differs from the exact derivative by ~3e-3 on
the friction-projection problem, identically for the oracle's CPU factorisation and the GPU. On
degenerate problems the adjoint at the final iterate therefore moves with the iterate itself:
on the differentiable-layer problems (configuration 3) the oracle's own adjoint moves by 4-32%
when q is changed at its last bit (oracle.perturb_q), with the same iteration count. Those
comparisons are bounded per instance and per gradient by that measured spread
(oracle_adjoint_with_spread: max(GRAD_TOL, 2 x the spread over six perturbations)). The tight
checks use strictly complementary problems (strict_qp), where the adjoint equals the derivative:
the GPU adjoint matches the oracle's and central finite differences to GRAD_TOL_STRICT there.
"""
import numpy as np
import pytest

from conftest import kat_qp, rel
from conicxx_gb300 import _abi, _lib, generators
from conicxx_gb300.problem import QP, Csc

pytestmark = pytest.mark.gpu
GRAD_TOL_STRICT = 1e-5  # nondegenerate problems: the adjoint is stable to ~1e-7 across tolerances
GRAD_TOL = 1e-3


def oracle_adjoint_with_spread(oracle_mod, qp, target, members=6):
    """The oracle's adjoint (dq, db, dP, dA) of L = 1/2 |x - target|^2 at its own solution, and per
    gradient the largest relative 2-norm change of that adjoint over `members` solves with q
    changed at its last bit (each at its own solution; members that do not Solve are skipped)."""
    O = oracle_mod.OracleSolver()
    assert O.setup(qp, warm_start=0)
    xo, _, _, io = O.solve()
    if io["status"] != 1:
        return None, None
    go = O.adjoint(xo - target)
    spread = np.zeros(4)
    for k in range(members):
        Ok = oracle_mod.OracleSolver()
        assert Ok.setup(oracle_mod.perturb_q(qp, 1000 + k), warm_start=0)
        xk, _, _, ik = Ok.solve()
        if ik["status"] != 1:
            continue
        gk = Ok.adjoint(xk - target)
        spread = np.maximum(spread, [rel(a, b) for a, b in zip(gk, go)])
    return go, spread


def adjoint_bound(spread):
    """Per gradient: the rounding-level spread of the oracle's own adjoint, doubled, or GRAD_TOL."""
    return np.maximum(GRAD_TOL, 2.0 * spread)


def strict_qp(seed, n=30, p=5, l=40):
    """Strictly convex QP (P = M'M + I) over Zero^p x R^l_+ with a strictly complementary
    solution (x0, s0, z0): each inequality row is either active (s = 0, z in [1, 2]) or inactive
    (s in [1, 2], z = 0). The solution map is smooth there, so the adjoint at the final iterate
    equals the derivative to ~1e-7 at the default tolerance."""
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((n, n)) / np.sqrt(n)
    P = M.T @ M + np.eye(n)
    m = p + l
    A = rng.standard_normal((m, n))
    x0 = rng.standard_normal(n)
    s0, z0 = np.zeros(m), np.zeros(m)
    z0[:p] = rng.standard_normal(p)
    act = rng.random(l) < 0.5
    s0[p:][~act] = rng.uniform(1, 2, int((~act).sum()))
    z0[p:][act] = rng.uniform(1, 2, int(act.sum()))
    return QP(Csc.from_dense(np.triu(P), keep_zeros=False), -P @ x0 - A.T @ z0,
              Csc.from_dense(A, keep_zeros=False), A @ x0 + s0, p, l, [])


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if _lib.lib().cxg_device_count() < 1:
        pytest.fail("a CUDA device is required for the -m gpu tests")


def test_closed_form_equality_qp(kats):
    """min 1/2|x|^2 + q'x s.t. x0 + x1 = b (test/solver/test_solve_qp.cpp:9-34): x = -q + (b+q0+q1)/2 (1,1),
    so for L = 1/2|x - t|^2: dL/dq = (-I + 11'/2)(x - t), dL/db = ((x0-t0) + (x1-t1))/2."""
    from conicxx_gb300 import Solver

    qp = kat_qp(kats[0])
    t = np.array([0.3, -1.2])
    for precision in (_abi.PRECISION_FP64, _abi.PRECISION_MIXED):
        S = Solver()
        assert S.setup(qp, precision=precision)
        sol = S.solve()
        assert sol.ok()
        g = sol.x - t
        dq, db, dP, dA = S.backward(g)
        J = -np.eye(2) + 0.5 * np.ones((2, 2))
        assert np.allclose(dq, J @ g, atol=1e-6), dq
        assert np.allclose(db, [0.5 * g.sum()], atol=1e-6), db
        # dL/dA_0j = -(z0 u_j + v0 x_j) with u = -dq, v = db (the reference's A = [1 1])
        z0 = sol.z[0]
        assert np.allclose(dA, -(z0 * (-dq) + db[0] * sol.x), atol=1e-6), dA


@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
def test_adjoint_matches_oracle_on_nondegenerate_problems(oracle_mod, precision):
    """Tight: on strictly complementary problems the GPU adjoint equals the oracle's FP64 adjoint
    (computed with its own CPU factorisation at its own solution) to GRAD_TOL_STRICT."""
    from conicxx_gb300 import Solver

    for seed in range(4):
        qp = strict_qp(seed)
        t = np.linspace(-1.0, 1.0, qp.n)
        S = Solver()
        assert S.setup(qp, precision=precision)
        sol = S.solve()
        O = oracle_mod.OracleSolver()
        assert O.setup(qp)
        xo, _, _, io = O.solve()
        assert sol.ok() and io["status"] == 1
        g = S.backward(sol.x - t)
        go = O.adjoint(xo - t)
        for name, a, b in zip(("dq", "db", "dP", "dA"), g, go):
            assert rel(a, b) < GRAD_TOL_STRICT, (seed, name, rel(a, b))


@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
def test_adjoint_matches_oracle_on_degenerate_layer_problems(oracle_mod, precision):
    """The differentiable-layer problems (n=100, m=150, Zero^10 x R^100_+ x 10 Q^4) are
    degenerate: the adjoint at the final iterate moves with the iterate itself. Each gradient is
    compared with the oracle's within twice the oracle's own spread under last-bit changes of q."""
    from conicxx_gb300 import Solver

    checked = 0
    for seed in range(3):
        qp = generators.config3_qp(seed)
        t = generators.x_target(seed, qp.n)
        S = Solver()
        assert S.setup(qp, precision=precision, warm_start=0)
        sol = S.solve()
        go, spread = oracle_adjoint_with_spread(oracle_mod, qp, t)
        assert sol.ok() and go is not None
        g = S.backward(sol.x - t)
        bound = adjoint_bound(spread)
        for k, (name, a, b) in enumerate(zip(("dq", "db", "dP", "dA"), g, go)):
            print(seed, name, "device vs oracle %.3e, oracle's own spread %.3e" % (rel(a, b), spread[k]))
            assert rel(a, b) < bound[k], (seed, name, rel(a, b), spread[k])
        checked += 1
    assert checked == 3


def test_batched_adjoint_matches_single_and_oracle(oracle_mod):
    """The batched adjoint equals, per instance, the single-instance Solver's adjoint (the same
    device computation on the same iterates: tight), and the oracle's within twice the oracle's
    own spread under last-bit changes of q, per instance and gradient."""
    from conicxx_gb300 import BatchSolver, Solver

    qps = [generators.config3_qp(10 + i) for i in range(8)] + [generators.contact_qp(300 + i, cmax=24) for i in range(8)]
    B = BatchSolver(qps, differentiable=1, warm_start=0, precision=_abi.PRECISION_FP64)
    x, s, z, infos = B.solve()
    targets = [generators.x_target(i, qp.n) for i, qp in enumerate(qps)]
    xs = B.split(x, s, z)
    gx = np.concatenate([xs[i][0] - targets[i] for i in range(len(qps))])
    dq, db, dP, dA = B.backward(gx)
    worst = []
    for i, qp in enumerate(qps):
        if infos[i]["status"] != 1:
            continue
        sl = [slice(B.n_off[i], B.n_off[i + 1]), slice(B.m_off[i], B.m_off[i + 1]),
              slice(B.p_off[i], B.p_off[i + 1]), slice(B.a_off[i], B.a_off[i + 1])]
        S = Solver()
        assert S.setup(qp, warm_start=0, precision=_abi.PRECISION_FP64)
        sol = S.solve()
        assert sol.info["iterations"] == infos[i]["iterations"]
        gs = S.backward(sol.x - targets[i])
        for name, full, ref, sli in zip(("dq", "db", "dP", "dA"), (dq, db, dP, dA), gs, sl):
            assert rel(full[sli], ref) < 1e-9, (i, name, rel(full[sli], ref))
        go, spread = oracle_adjoint_with_spread(oracle_mod, qp, targets[i])
        if go is None:
            continue
        bound = adjoint_bound(spread)
        for k, (full, ref, sli) in enumerate(zip((dq, db, dP, dA), go, sl)):
            assert rel(full[sli], ref) < bound[k], (i, k, rel(full[sli], ref), spread[k])
        worst.append(max(rel(full[sli], ref) for full, ref, sli in zip((dq, db, dP, dA), go, sl)))
    assert len(worst) >= 12, len(worst)


def test_adjoint_against_central_differences(kats, oracle_mod):
    """Central finite differences (step 1e-6, tight-tolerance oracle solves) of the forward map on
    problems whose solution map is smooth (the box QP with one active bound and the friction
    projection), within the 1e-8-iterate smoothing (<1e-2 relative)."""
    from conicxx_gb300 import Solver

    tight = dict(tol_feas=1e-12, tol_gap_abs=1e-12, tol_gap_rel=1e-12)
    for idx in (1, 4):
        qp = kat_qp(kats[idx])
        t = np.linspace(-1.0, 1.0, qp.n)
        S = Solver()
        assert S.setup(qp)
        sol = S.solve()
        dq, db, _, _ = S.backward(sol.x - t)
        L = lambda p: 0.5 * np.sum((oracle_mod.solve(p, **tight)[0] - t) ** 2)  # noqa: E731
        h = 1e-6
        for vec, grad in (("q", dq), ("b", db)):
            for i in range(len(grad)):
                vp, vm = getattr(qp, vec).copy(), getattr(qp, vec).copy()
                vp[i] += h
                vm[i] -= h
                mk = lambda v: QP(qp.P, v if vec == "q" else qp.q, qp.A, v if vec == "b" else qp.b,  # noqa: E731
                                  qp.zero, qp.nonneg, qp.soc)
                fd = (L(mk(vp)) - L(mk(vm))) / (2 * h)
                assert abs(fd - grad[i]) < 1e-2 * max(1.0, abs(fd)), (kats[idx]["name"], vec, i, fd, grad[i])


def test_adjoint_against_central_differences_nondegenerate(oracle_mod):
    """Central finite differences (step 1e-6, tight-tolerance oracle solves) against the GPU
    adjoint on strictly complementary problems, to GRAD_TOL_STRICT relative."""
    from conicxx_gb300 import Solver

    tight = dict(tol_feas=1e-12, tol_gap_abs=1e-12, tol_gap_rel=1e-12)
    for seed in range(2):
        qp = strict_qp(seed)
        t = np.linspace(-1.0, 1.0, qp.n)
        S = Solver()
        assert S.setup(qp)
        sol = S.solve()
        dq, db, _, _ = S.backward(sol.x - t)
        L = lambda p: 0.5 * np.sum((oracle_mod.solve(p, **tight)[0] - t) ** 2)  # noqa: E731
        h = 1e-6
        for vec, grad in (("q", dq), ("b", db)):
            for i in range(0, len(grad), 7):
                vp, vm = getattr(qp, vec).copy(), getattr(qp, vec).copy()
                vp[i] += h
                vm[i] -= h
                mk = lambda v: QP(qp.P, v if vec == "q" else qp.q, qp.A, v if vec == "b" else qp.b,  # noqa: E731
                                  qp.zero, qp.nonneg, qp.soc)
                fd = (L(mk(vp)) - L(mk(vm))) / (2 * h)
                assert abs(fd - grad[i]) < GRAD_TOL_STRICT * max(1.0, abs(fd)), (seed, vec, i, fd, grad[i])


def test_torch_layer_autograd(oracle_mod):
    torch = pytest.importorskip("torch")
    from conicxx_gb300.torch_layer import QPLayer

    qps = [generators.config3_qp(20 + i) for i in range(4)]
    layer = QPLayer(qps)
    dev = torch.device("cuda", 0)
    Px = torch.tensor(np.concatenate([q.P.data for q in qps]), device=dev, requires_grad=True)
    q = torch.tensor(np.concatenate([q_.q for q_ in qps]), device=dev, requires_grad=True)
    Ax = torch.tensor(np.concatenate([q_.A.data for q_ in qps]), device=dev, requires_grad=True)
    b = torch.tensor(np.concatenate([q_.b for q_ in qps]), device=dev, requires_grad=True)
    tgt = torch.tensor(np.concatenate([generators.x_target(i, q_.n) for i, q_ in enumerate(qps)]), device=dev)
    x = layer(Px, q, Ax, b)
    loss = 0.5 * ((x - tgt) ** 2).sum()
    loss.backward()
    # exact consistency with the batch adjoint through the C-ABI (same device computation)
    gref = layer.solver.backward((x - tgt).detach().cpu().numpy())
    for got, ref in zip((q.grad, b.grad, Px.grad, Ax.grad), gref):
        assert rel(got.cpu().numpy(), ref) < 1e-12
    for i, qp in enumerate(qps):
        go, spread = oracle_adjoint_with_spread(oracle_mod, qp, generators.x_target(i, qp.n))
        assert go is not None
        bound = adjoint_bound(spread)
        s = layer.solver
        got = (q.grad[s.n_off[i]:s.n_off[i + 1]], b.grad[s.m_off[i]:s.m_off[i + 1]],
               Px.grad[s.p_off[i]:s.p_off[i + 1]], Ax.grad[s.a_off[i]:s.a_off[i + 1]])
        for k, (gv, ref) in enumerate(zip(got, go)):
            assert rel(gv.cpu().numpy(), ref) < bound[k], (i, k, rel(gv.cpu().numpy(), ref), spread[k])
