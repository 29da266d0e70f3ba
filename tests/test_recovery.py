"""The numerical recovery paths of the KKT layer, driven by host-side fault injection
(cxg_settings::fault_factor_failures / fault_nonfinite_solves; nothing faults on the GPU):

- factorizeWithRetry's x10 regularisation ladder (src/conicxx/kkt/kkt_system.cpp:242-264): the
  first k factorisation attempts of a solve report failure;
- escalateAndResolve's x1000 bumps (kkt_system.cpp:266-294): the first k solves with the factor
  return a non-finite vector;
- a ladder that runs out (18 failed attempts) ends in NumericalError
  (SolverImpl::solve, src/conicxx/solver_impl.cpp:445-448);
- a NaN in one instance's data ends that instance in NumericalError and leaves every other
  instance of the batch bit-identical.

The oracle carries the same injection, so the device path is checked against it attempt for
attempt: same status, the same number of attempts and escalations, iterations within +-1.
"""
import numpy as np
import pytest

from conftest import kat_qp
from conicxx_gb300 import _abi, generators

X_TOL = 1e-5


def _oracle_solve(orc, qp, **kw):
    S = orc.OracleSolver()
    assert S.setup(qp, warm_start=0, **kw)
    return S.solve()


# ---- the oracle's own injection (CPU) ------------------------------------------------------------
def test_oracle_factor_ladder_injection(oracle_mod, kats):
    """k injected failures add exactly k attempts, and the solve still ends Solved at the KAT's x."""
    k = kats[0]
    qp = kat_qp(k)
    _, _, _, base = _oracle_solve(oracle_mod, qp)
    for inj in (1, 3, 5):
        x, _, _, info = _oracle_solve(oracle_mod, qp, fault_factor_failures=inj)
        assert info["status"] == _abi.STATUS_SOLVED
        assert info["factor_attempts"] == base["factor_attempts"] + inj
        assert np.allclose(x, k["x"], atol=k["tol"])


def test_oracle_escalation_injection(oracle_mod, kats):
    """Each injected non-finite solve costs one x1000 escalation; the solve recovers."""
    k = kats[0]
    qp = kat_qp(k)
    _, _, _, base = _oracle_solve(oracle_mod, qp)
    assert base["escalations"] == 0
    for inj in (1, 2):
        x, _, _, info = _oracle_solve(oracle_mod, qp, fault_nonfinite_solves=inj)
        assert info["status"] == _abi.STATUS_SOLVED
        assert info["escalations"] == inj
        assert np.allclose(x, k["x"], atol=k["tol"])


def test_oracle_ladder_exhausted(oracle_mod, kats):
    """18 failed attempts: the initial point cannot be computed -> NumericalError."""
    qp = kat_qp(kats[0])
    _, _, _, info = _oracle_solve(oracle_mod, qp, fault_factor_failures=18)
    assert info["status"] == _abi.STATUS_NUMERICAL_ERROR
    assert info["factor_attempts"] == 18


# ---- the device path against the oracle (GPU) --------------------------------------------------
def _instances():
    qps = [generators.contact_qp(i, cmin=6, cmax=20) for i in range(3)]
    qps.append(generators.random_conic_qp(0, n=60, m_zero=6, m_nonneg=40, soc=(3,) * 8))
    return qps


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
@pytest.mark.parametrize("inj", [dict(fault_factor_failures=2), dict(fault_factor_failures=4),
                                 dict(fault_nonfinite_solves=1), dict(fault_nonfinite_solves=2),
                                 dict(fault_factor_failures=3, fault_nonfinite_solves=1)])
def test_recovery_paths_match_oracle(oracle_mod, inj, precision):
    from conicxx_gb300 import BatchSolver, Solver

    qps = _instances()
    # single instances (cxg_solver, one CTA) and the same instances as one batch
    B = BatchSolver(qps, precision=precision, warm_start=0, **inj)
    xb, sb, zb, infos = B.solve()
    parts = B.split(xb, sb, zb)
    for i, qp in enumerate(qps):
        xo, so, zo, io = _oracle_solve(oracle_mod, qp, **inj)
        S = Solver()
        assert S.setup(qp, precision=precision, warm_start=0, **inj)
        sol = S.solve()
        for got, x in ((sol.info, sol.x), (infos[i], parts[i][0])):
            assert int(got["status"]) == io["status"] == _abi.STATUS_SOLVED, (i, inj, got["status"], io["status"])
            assert int(got["factor_attempts"]) == io["factor_attempts"] or precision == _abi.PRECISION_MIXED, \
                (i, inj, got["factor_attempts"], io["factor_attempts"])
            if "fault_nonfinite_solves" in inj:
                assert int(got["escalations"]) == io["escalations"] == inj["fault_nonfinite_solves"], \
                    (i, inj, got["escalations"], io["escalations"])
            assert abs(int(got["iterations"]) - io["iterations"]) <= 1, (i, inj, got["iterations"], io["iterations"])
            err = np.max(np.abs(x - xo)) / max(1.0, np.max(np.abs(xo)))
            assert err < X_TOL, (i, inj, err)


@pytest.mark.gpu
def test_injected_attempts_counted_on_device(oracle_mod):
    """FP64 device attempts = clean attempts + injected failures (the ladder was taken)."""
    from conicxx_gb300 import Solver

    qp = _instances()[0]
    S = Solver()
    assert S.setup(qp, warm_start=0)
    base = S.solve().info["factor_attempts"]
    S = Solver()
    assert S.setup(qp, warm_start=0, fault_factor_failures=3)
    sol = S.solve()
    assert sol.info["status"] == _abi.STATUS_SOLVED
    assert sol.info["factor_attempts"] == base + 3


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
def test_ladder_exhausted_is_numerical_error(oracle_mod, precision):
    from conicxx_gb300 import Solver

    qp = _instances()[0]
    _, _, _, io = _oracle_solve(oracle_mod, qp, fault_factor_failures=18)
    S = Solver()
    assert S.setup(qp, precision=precision, warm_start=0, fault_factor_failures=18)
    sol = S.solve()
    assert sol.status == io["status"] == _abi.STATUS_NUMERICAL_ERROR


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
def test_nan_instance_isolated_in_batch(precision):
    """A NaN in one instance's q (set through updateData's value copy, which does not screen
    values): that instance ends NumericalError; every other instance's status, iterations and
    x, s, z are bit-identical to the clean batch."""
    from conicxx_gb300 import BatchSolver

    qps = [generators.contact_qp(i, cmin=4, cmax=24) for i in range(12)]
    B = BatchSolver(qps, precision=precision, warm_start=0)
    x0, s0, z0, i0 = B.solve()
    q = np.concatenate([qp.q for qp in qps])
    bad = 5
    q[B.n_off[bad] + 1] = np.nan
    B.update_values(q=q)
    x1, s1, z1, i1 = B.solve()
    assert int(i1[bad]["status"]) == _abi.STATUS_NUMERICAL_ERROR
    for i in range(len(qps)):
        if i == bad:
            continue
        assert int(i1[i]["status"]) == int(i0[i]["status"]) and int(i1[i]["iterations"]) == int(i0[i]["iterations"])
        sl, ml = slice(B.n_off[i], B.n_off[i + 1]), slice(B.m_off[i], B.m_off[i + 1])
        assert np.array_equal(x1[sl], x0[sl]) and np.array_equal(s1[ml], s0[ml]) and np.array_equal(z1[ml], z0[ml])
