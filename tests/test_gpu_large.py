"""GPU tests of the whole-GPU root: one large instance whose root is assembled, factored and
solved by every SM (cooperative launch), CTA 0 running the interior-point iteration.

- The factor itself (cxg_dense_ldlt, threads = -1) gives the same L and D bits as the one-CTA
  root in FP64 and double-float (every tile receives the same updates in the same order); in FP32
  the trailing update runs on the tensor cores (3xTF32), and L and D agree to FP32 accuracy.
- Full solves (whole_gpu_root = 1) against the oracle: same status, iterations within +-1,
  x within 1e-6 relative; and against the one-CTA form of the same instance.
- The large single-instance workloads at full size (n = 20000, m = 30000 sparse QP): status and
  the KKT residuals of the returned point, which the oracle cannot reach at that size.
"""
import numpy as np
import pytest

from conftest import rel
from conicxx_gb300 import _abi, _lib, generators

pytestmark = pytest.mark.gpu
ARITH = {"fp64": 0, "fp32": 1, "df64": 2}
# x of the GPU solve against the FP64 oracle's, relative to max |x| (the criterion of the
# batched parity tests)
X_TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if _lib.lib().cxg_device_count() < 1:
        pytest.fail("a CUDA device is required for the -m gpu tests")


def _quasi_definite(nr, nx, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((nx, nx))
    P = B @ B.T / nx + np.eye(nx)
    AZ = rng.standard_normal((nr - nx, nx)) * 0.5
    K = np.zeros((nr, nr))
    K[:nx, :nx] = P
    K[nx:, :nx] = AZ
    K[:nx, nx:] = AZ.T
    K[nx:, nx:] = -np.eye(nr - nx) * 0.5
    return K


def _probe(K, nx, b, arith, threads):
    nr = K.shape[0]
    Kc = np.asfortranarray(K)
    L = np.zeros((nr, nr), order="F")
    D = np.zeros(nr)
    x = np.zeros(nr)
    cyc = np.zeros(2, np.int64)
    flags = np.zeros(3, np.int32)
    rc = _lib.lib().cxg_dense_ldlt(nr, nx, Kc.ctypes.data, b.ctypes.data, ARITH[arith], threads,
                                   _abi.LINSOLVER_QDLDL, L.ctypes.data, D.ctypes.data, x.ctypes.data,
                                   cyc.ctypes.data, flags.ctypes.data)
    assert rc == _abi.OK, _lib.lib().cxg_last_error()
    return L, D, x, flags


@pytest.mark.parametrize("arith", ["fp64", "fp32", "df64"])
@pytest.mark.parametrize("nr,nx", [(40, 30), (150, 120), (190, 160)])
def test_grid_factor_equals_one_cta(arith, nr, nx):
    """The whole-GPU LDL' is bit-identical to the one-CTA LDL' in FP64 (same tile operations in
    the same order per tile); in FP32 its trailing updates run on the tensor cores as 3xTF32
    products, so L and D agree to FP32 accuracy; in double-float (at these sizes the one-column
    form, whose trailing update runs on the CUDA cores) L and D agree to 1e-11. Its solve agrees
    with numpy to the arithmetic's accuracy. Sizes up to six tiles, the largest 8-byte root the
    one-CTA probe holds in shared memory."""
    K = _quasi_definite(nr, nx, nr + 7)
    b = np.random.default_rng(nr).standard_normal(nr)
    L1, D1, x1, f1 = _probe(K, nx, b, arith, 256)
    Lg, Dg, xg, fg = _probe(K, nx, b, arith, -1)
    assert fg[2] == 0 and fg[0] == 0 and fg[1] == 0 and f1[0] == 0 and f1[1] == 0
    if arith == "fp64":
        assert np.array_equal(L1, Lg) and np.array_equal(D1, Dg)
    else:
        # FP32: FP32-level agreement (a single TF32 product would differ by ~1e-3); double-float:
        # the sliced tensor-core products against the CUDA-core double-float products
        lt = 1e-5 if arith == "fp32" else 1e-11
        assert np.max(np.abs(L1 - Lg)) < lt * max(1.0, np.max(np.abs(L1))), np.max(np.abs(L1 - Lg))
        assert np.max(np.abs(D1 - Dg) / np.abs(D1)) < lt, np.max(np.abs(D1 - Dg) / np.abs(D1))
    xs = np.linalg.solve(K, b)
    tol = {"fp64": 1e-10, "df64": 1e-8, "fp32": 1e-3}[arith]
    assert rel(xg, xs) < tol and rel(x1, xs) < tol


@pytest.mark.parametrize("arith", ["fp64", "fp32", "df64"])
def test_grid_factor_large_root(arith):
    """A 1500-row root (47 tile columns) on the whole GPU against numpy."""
    nr, nx = 1500, 1300
    K = _quasi_definite(nr, nx, 11)
    b = np.random.default_rng(12).standard_normal(nr)
    L, D, x, f = _probe(K, nx, b, arith, -1)
    assert f[2] == 0 and f[0] == 0 and f[1] == 0
    xs = np.linalg.solve(K, b)
    tol = {"fp64": 1e-10, "df64": 1e-8, "fp32": 1e-3}[arith]
    assert rel(x, xs) < tol
    # FP32 (tensor-core 3xTF32 trailing updates): the reconstruction at FP32 accuracy, well below
    # the ~1e-3 of a single TF32 product; double-float: at the level of an FP64 factor
    recon = rel(L @ np.diag(D) @ L.T, K)
    print(arith, "reconstruction", recon, "solve", rel(x, xs))
    assert recon < {"fp64": 1e-10, "df64": 1e-12, "fp32": 1e-5}[arith]


@pytest.mark.parametrize("arith,nr", [("fp32", 12832), ("df64", 5216)])
def test_grid_factor_pair_form(arith, nr):
    """Roots above the pair threshold (352 tile columns in FP32, 160 in double-float) factor over
    column pairs, the trailing update fed by the TF32 parts or BF16 slices written per row pair:
    the solve against numpy and the residual."""
    nx = nr - 256
    K = _quasi_definite(nr, nx, 21)
    b = np.random.default_rng(22).standard_normal(nr)
    L, D, x, f = _probe(K, nx, b, arith, -1)
    assert f[2] == 0 and f[0] == 0 and f[1] == 0
    xs = np.linalg.solve(K, b)
    res = np.linalg.norm(K @ x - b) / np.linalg.norm(b)
    print(arith, nr, "solve", rel(x, xs), "residual", res)
    assert rel(x, xs) < {"df64": 1e-10, "fp32": 1e-4}[arith]
    assert res < {"df64": 1e-11, "fp32": 1e-4}[arith]


@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
@pytest.mark.parametrize("idx", range(8))
def test_kats_whole_gpu(kats, idx, precision):
    """Every known-answer problem through the whole-GPU form (roots of one tile: the one-block
    edge of the solve, and the infeasibility statuses)."""
    from conftest import kat_qp
    from conicxx_gb300 import Solver

    k = kats[idx]
    qp = kat_qp(k)
    S = Solver()
    assert S.setup(qp, precision=precision, whole_gpu_root=1)
    sol = S.solve()
    assert sol.status == k["status"], (k["name"], sol.status_name)
    if k["x"] is not None:
        assert np.allclose(sol.x, k["x"], atol=k["tol"]), (k["name"], sol.x)
    if k["objective"] is not None:
        assert abs(sol.objective - k["objective"]) < k["tol"]


def _small_large_qp():
    # the large sparse QP family (P = M'M + 1e-3 I, 3 nnz per column of M; A 8 nnz per row) at
    # n = 1000, m = 1500: root of 1100 rows, 35 tile columns
    return generators.large_sparse_qp(0, n=1000, m_zero=100, m_nonneg=1200, n_soc=100)


def oracle_band(oracle_mod, qp, members=4):
    """The oracle's solve of qp and its rounding band: the same solve with q changed at its last
    bit (oracle.perturb_q) `members` times. Returns (x, info, statuses, iterations of every run,
    largest max-norm-relative change of x over the Solved perturbed runs)."""
    xo, _, _, io, _ = oracle_mod.solve(qp, warm_start=0)
    sts, its, spread = [io["status"]], [io["iterations"]], 0.0
    for k in range(members):
        xk, _, _, ik, _ = oracle_mod.solve(oracle_mod.perturb_q(qp, 500 + k), warm_start=0)
        sts.append(ik["status"])
        its.append(ik["iterations"])
        if ik["status"] == io["status"] == _abi.STATUS_SOLVED:
            spread = max(spread, float(np.max(np.abs(xk - xo)) / max(1.0, float(np.max(np.abs(xo))))))
    return xo, io, sts, its, spread


def assert_within_band(sol, band):
    """Status the oracle's; iterations within one of the oracle's band (its iteration count under
    last-bit changes of q: on configuration 2's family at n = 1000 it runs 12 to 17 iterations
    as the rounding falls); x within max(X_TOL, 10 x the band's spread of x)."""
    xo, io, sts, its, spread = band
    assert sol.status == io["status"] == _abi.STATUS_SOLVED, (sol.status, sts)
    assert min(its) - 1 <= sol.info["iterations"] <= max(its) + 1, (sol.info["iterations"], its)
    assert np.max(np.abs(sol.x - xo)) <= max(X_TOL, 10.0 * spread) * max(1.0, np.max(np.abs(xo))), spread


@pytest.fixture(scope="module")
def small_large_band(oracle_mod):
    qp = _small_large_qp()
    return qp, oracle_band(oracle_mod, qp)


@pytest.fixture(scope="module")
def group_lasso_band(oracle_mod):
    qp = generators.group_lasso_socp(0, groups=60)
    return qp, oracle_band(oracle_mod, qp)


@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
def test_whole_gpu_root_agrees_with_oracle(small_large_band, precision):
    """Configuration 2's family at n = 1000 on the whole-GPU root against the oracle's band."""
    from conicxx_gb300 import Solver

    qp, band = small_large_band
    S = Solver()
    assert S.setup(qp, precision=precision, warm_start=0, whole_gpu_root=1)
    sol = S.solve()
    print("device iterations", sol.info["iterations"], "oracle band", band[3], "x spread %.2e" % band[4])
    assert_within_band(sol, band)
    st, fe, sz = qp.kkt_residuals(sol.x, sol.s, sol.z)
    assert fe < 1e-6 and sz < 1e-6


@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
def test_group_lasso_whole_gpu_agrees_with_oracle(group_lasso_band, precision):
    """The block-sparse group-lasso SOCP (60 groups of 16: n = 1020, SOC blocks of dimension 17)."""
    from conicxx_gb300 import Solver

    qp, band = group_lasso_band
    S = Solver()
    assert S.setup(qp, precision=precision, warm_start=0, whole_gpu_root=1)
    sol = S.solve()
    print("device iterations", sol.info["iterations"], "oracle band", band[3], "x spread %.2e" % band[4])
    assert_within_band(sol, band)


def test_whole_gpu_and_one_cta_forms_agree():
    """The same instance through both forms: same status and iterations, x to 1e-8 relative
    (the forms differ only in the summation order of the dense triangular solves)."""
    from conicxx_gb300 import Solver

    qp = _small_large_qp()
    out = []
    for whole in (1, -1):
        S = Solver()
        assert S.setup(qp, precision=_abi.PRECISION_MIXED, warm_start=0, whole_gpu_root=whole)
        sol = S.solve()
        out.append((sol.status, sol.info["iterations"], sol.x.copy()))
    assert out[0][0] == out[1][0] == _abi.STATUS_SOLVED
    assert out[0][1] == out[1][1]
    assert rel(out[0][2], out[1][2]) < 1e-8


def test_whole_gpu_warm_start_and_backward(oracle_mod):
    """setWarmStart at the oracle's solution on the whole-GPU form against the oracle started the
    same way (same status, iterations within +-1); the adjoint (one-CTA solve with the saved
    factor) agreeing with the one-CTA form's gradient. (A warm start after a change of q sends
    the reference's iteration to MaxIterations on these families, so it is no parity case.)"""
    from conicxx_gb300 import Solver

    qp = generators.group_lasso_socp(1, groups=40)
    O = oracle_mod.OracleSolver()
    assert O.setup(qp)
    x0, s0, z0, _ = O.solve()
    O2 = oracle_mod.OracleSolver()
    assert O2.setup(qp)
    O2.set_warm_start(x0, s0, z0)
    xo, _, _, io = O2.solve()
    grads = []
    for whole in (1, -1):
        S = Solver()
        assert S.setup(qp, precision=_abi.PRECISION_FP64, whole_gpu_root=whole)
        S.set_warm_start(x0, s0, z0)
        sol = S.solve()
        assert sol.status == io["status"] == _abi.STATUS_SOLVED
        assert abs(sol.info["iterations"] - io["iterations"]) <= 1
        assert np.max(np.abs(sol.x - xo)) <= X_TOL * max(1.0, np.max(np.abs(xo)))
        grads.append(S.backward(np.ones(qp.P.shape[0]))[0])
    assert rel(grads[0], grads[1]) < 1e-6


def test_large_sparse_qp_full_size_mixed():
    """Configuration 2 at full size: the n = 20000, m = 30000 sparse QP (root of 22000 rows) in
    mixed precision on the whole GPU is Solved, and the returned point meets the tolerances on the
    unscaled KKT conditions (a property independent of the oracle, which takes hours at this
    size; its parity cases are the same family at n = 2000 and 3000, below)."""
    from conicxx_gb300 import Solver

    qp = generators.large_sparse_qp(0)
    S = Solver()
    assert S.setup(qp, precision=_abi.PRECISION_MIXED, warm_start=0)
    sol = S.solve()
    assert sol.status == _abi.STATUS_SOLVED, (sol.status_name, sol.info["iterations"])
    assert sol.info["iterations"] <= 40
    st, fe, sz = qp.kkt_residuals(sol.x, sol.s, sol.z)
    scale = max(1.0, np.linalg.norm(qp.q), np.linalg.norm(qp.b))
    assert st < 1e-6 * scale and fe < 1e-6 * scale and abs(sz) < 1e-6 * max(1.0, abs(sol.objective)), (st, fe, sz)
    assert np.all(qp.cone_margins(sol.s)[0] >= -1e-9) and np.all(qp.cone_margins(sol.z)[0] >= -1e-9)


def _golden_large():
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_large.npz")
    return np.load(path)


@pytest.mark.parametrize("precision", [_abi.PRECISION_FP64, _abi.PRECISION_MIXED])
@pytest.mark.parametrize("n", [2000, 3000])
def test_large_family_agrees_with_oracle_golden(n, precision):
    """Configuration 2's family at n = 2000 and 3000 (roots of 2200 and 3300 rows) on the whole
    GPU against the oracle's solutions (tests/golden/oracle_large.npz): both Solved; x, s and z
    within 5e-5 relative to their max-norm, the size of the 1e-8 stopping ball on this family
    (P = M'M + 1e-3 I): the oracle's own solutions at 1e-8 and at 1e-10 differ by 1.6e-5 (x),
    4.6e-5 (s) and 3.3e-5 (z) at n = 2000 (its 1e-10 solution is kept in the fixture as n2000t).
    Iteration counts are not compared: past the point where the reference's dense SOC blocks
    lose their small eigenvalue, its path depends on their rounding (the device holds those
    blocks at the dense form's resolution instead; 12-13 iterations against the oracle's 20-26)."""
    from conicxx_gb300 import Solver

    g = _golden_large()
    f = n / 20000  # the proportions of n = 20000 (tests/golden/make_golden.py, large_family)
    qp = generators.large_sparse_qp(0, n=n, m_zero=int(2000 * f), m_nonneg=int(24000 * f), n_soc=int(2000 * f))
    checksum = [qp.P.data.sum(), qp.A.data.sum(), qp.q.sum(), qp.b.sum(), qp.P.nnz, qp.A.nnz]
    np.testing.assert_allclose(checksum, g[f"n{n}/checksum"], rtol=1e-12)
    S = Solver()
    assert S.setup(qp, precision=precision, warm_start=0, whole_gpu_root=1)
    sol = S.solve()
    status_o = int(g[f"n{n}/info"][0])
    assert sol.status == status_o == _abi.STATUS_SOLVED, (sol.status_name, sol.info["iterations"])
    for name, v in (("x", sol.x), ("s", sol.s), ("z", sol.z)):
        vo = g[f"n{n}/{name}"]
        err = np.max(np.abs(v - vo)) / max(1.0, np.max(np.abs(vo)))
        print("n=%d %s error vs oracle %.2e" % (n, name, err))
        assert err < 5e-5, (name, err)


def test_large_family_mixed_equals_fp64_factor():
    """FP32 factorisation with FP64 refinement against the FP64 factorisation on the same
    instance of configuration 2's family (n = 4000): both Solved, x, s and z within 1e-6
    (measured 3e-12, 3e-10, 5e-12: the two runs take the same path)."""
    from conicxx_gb300 import Solver

    f = 4000 / 20000
    qp = generators.large_sparse_qp(0, n=4000, m_zero=int(2000 * f), m_nonneg=int(24000 * f), n_soc=int(2000 * f))
    sols = []
    for precision in (_abi.PRECISION_MIXED, _abi.PRECISION_FP64):
        S = Solver()
        assert S.setup(qp, precision=precision, warm_start=0)
        sol = S.solve()
        assert sol.status == _abi.STATUS_SOLVED, (precision, sol.status_name)
        sols.append(sol)
    for name in ("x", "s", "z"):
        a, b = getattr(sols[0], name), getattr(sols[1], name)
        err = np.max(np.abs(a - b)) / max(1.0, np.max(np.abs(b)))
        print("mixed vs FP64 factor, %s: %.2e" % (name, err))
        assert err < 1e-6, name


def test_grid_barrier_wait_runs_out_and_reports():
    """The whole-GPU root's barrier wait is bounded. With one CTA that never arrives, the others'
    first wait runs out after the limit (0.2 s here), the error flag is set and every CTA returns;
    the context stays usable. With every CTA arriving, all barriers are passed."""
    import ctypes as C

    L = _lib.lib()
    err, mx, el = C.c_int(), C.c_int(), C.c_double()
    assert L.cxg_grid_barrier_selftest(1, 3, 0.2, C.byref(err), C.byref(mx), C.byref(el)) == _abi.OK
    assert err.value == 1 and mx.value == 0 and 0.15 < el.value < 5.0, (err.value, mx.value, el.value)
    # the device is still usable: a whole-GPU factorisation right after
    K = _quasi_definite(64, 48, 3)
    b = np.ones(64)
    _, _, x, f = _probe(K, 48, b, "fp64", -1)
    assert f[2] == 0 and rel(x, np.linalg.solve(K, b)) < 1e-10
    assert L.cxg_grid_barrier_selftest(-1, 200, 0.2, C.byref(err), C.byref(mx), C.byref(el)) == _abi.OK
    assert err.value == 0 and mx.value == 200, (err.value, mx.value)
