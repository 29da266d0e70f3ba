"""GPU tests of cxg_batch_replace: a new set-up of some instances of a batch (the per-timestep
contact-pattern change), the others kept with their values and device-resident warm starts."""
import numpy as np
import pytest

from conftest import rel
from conicxx_gb300 import _abi, _lib, generators

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if _lib.lib().cxg_device_count() < 1:
        pytest.fail("a CUDA device is required for the -m gpu tests")


def _batch(qps, **kw):
    from conicxx_gb300 import BatchSolver

    return BatchSolver(qps, **kw)


@pytest.mark.parametrize("precision", [_abi.PRECISION_MIXED, _abi.PRECISION_FP64])
def test_replace_equals_fresh_batch(precision):
    """Replacing 9 of 64 contact instances by instances of other sizes and patterns gives, on every
    instance, the statuses, iterations and x, s, z of a batch set up from the final list (cold
    starts; the same plans, buckets and per-instance arithmetic)."""
    qps = [generators.contact_qp(4000 + i) for i in range(64)]
    B = _batch(qps, warm_start=0, precision=precision)
    B.solve()
    idx = [0, 5, 6, 17, 31, 32, 40, 62, 63]
    new = [generators.contact_qp(9000 + j) for j in range(len(idx))]
    assert any(new[j].n != qps[i].n for j, i in enumerate(idx))
    B.replace(idx, new)
    final = list(qps)
    for j, i in enumerate(idx):
        final[i] = new[j]
    x1, s1, z1, inf1 = B.solve()
    F = _batch(final, warm_start=0, precision=precision)
    x2, s2, z2, inf2 = F.solve()
    np.testing.assert_array_equal(inf1["status"], inf2["status"])
    np.testing.assert_array_equal(inf1["iterations"], inf2["iterations"])
    for a, b in ((x1, x2), (s1, s2), (z1, z2)):
        assert a.shape == b.shape and rel(a, b) < 1e-12


def test_replace_keeps_values_and_warm_starts():
    """The kept instances keep the values last set (update_values) and their warm starts: after a
    warm re-solve they take the same iterations as in a batch without the replacement, and the
    replaced instances start cold (the iterations of a cold solve of the new instance)."""
    qps = [generators.contact_qp(5000 + i) for i in range(32)]
    B = _batch(qps, warm_start=1)
    R = _batch(qps, warm_start=1)
    # new values for every instance (q scaled), then two solves: the second is warm
    for S in (B, R):
        Px, q, Ax, b = S.concat_values()
        S.update_values(Px, 1.1 * q, Ax, b)
        S.solve()
    idx = [3, 11, 20]
    new = [generators.contact_qp(9100 + j) for j in range(len(idx))]
    B.replace(idx, new)
    _, _, _, infB = B.solve()
    _, _, _, infR = R.solve()
    keep = np.setdiff1d(np.arange(32), idx)
    np.testing.assert_array_equal(infB["iterations"][keep], infR["iterations"][keep])
    np.testing.assert_array_equal(infB["status"][keep], infR["status"][keep])
    C_ = _batch(new, warm_start=1)
    _, _, _, infC = C_.solve()
    np.testing.assert_array_equal(infB["iterations"][idx], infC["iterations"])


def test_replace_rejects_bad_arguments_and_stale_backward():
    """Indices out of range or repeated are refused before anything changes; after a replacement a
    differentiable batch needs a solve before backward."""
    import ctypes as C

    from conicxx_gb300._abi import iptr, make_problem_struct

    qps = [generators.config3_qp(60 + i) for i in range(6)]
    B = _batch(qps, warm_start=0, differentiable=1, precision=_abi.PRECISION_FP64)
    x, s, z, _ = B.solve()
    new = generators.config3_qp(70)
    st, keep = make_problem_struct(new)
    arr = (_abi.Problem * 2)(st, st)
    L = _lib.lib()
    for bad in ([6, 0], [2, 2], [-1, 0]):
        idx = np.array(bad, dtype=np.int32)
        assert L.cxg_batch_replace(B._h, 2, iptr(idx), arr) == _abi.E_INVALID
    B.backward(x - 0.5)  # still valid: nothing was replaced
    B.replace([4], [new])
    with pytest.raises(Exception):
        B.backward(np.zeros(B.n_total))
    x, s, z, infos = B.solve()
    assert np.all(infos["status"] == _abi.STATUS_SOLVED)
    g = B.backward(x - 0.5)
    assert all(np.all(np.isfinite(v)) for v in g)
