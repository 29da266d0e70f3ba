"""GPU tests of the IPM kernel's dense root factorisation (cxg_dense_ldlt): the tiled LDL' and its
triangular solves in FP64, FP32 and double-float against numpy on quasi-definite matrices of
the reduced-KKT shape [P + A'GA, A_Z'; A_Z, -eps I], sizes spanning one to six 32-row tiles."""
import ctypes as C

import numpy as np
import pytest

from conicxx_gb300 import _abi, _lib

pytestmark = pytest.mark.gpu
ARITH = {"fp64": 0, "fp32": 1, "df64": 2}
# relative tolerances on L, D and x for well-conditioned (cond ~ 1e3) matrices
TOL = {"fp64": 1e-11, "df64": 1e-9, "fp32": 2e-3}


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if _lib.lib().cxg_device_count() < 1:
        pytest.fail("a CUDA device is required for the -m gpu tests")


def quasi_definite(nr, nx, seed):
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


def ldlt_ref(K):
    n = K.shape[0]
    A = K.copy()
    L = np.eye(n)
    D = np.zeros(n)
    for j in range(n):
        D[j] = A[j, j]
        L[j + 1:, j] = A[j + 1:, j] / D[j]
        A[j + 1:, j + 1:] -= np.outer(L[j + 1:, j], A[j + 1:, j])
    return L, D


def probe(K, nx, b, arith, threads=256, linear_solver=_abi.LINSOLVER_QDLDL):
    nr = K.shape[0]
    Kc = np.asfortranarray(K)
    L = np.zeros((nr, nr), order="F")
    D = np.zeros(nr)
    x = np.zeros(nr)
    cyc = np.zeros(2, np.int64)
    flags = np.zeros(2, np.int32)
    rc = _lib.lib().cxg_dense_ldlt(nr, nx, Kc.ctypes.data, b.ctypes.data, ARITH[arith], threads, linear_solver,
                                   L.ctypes.data, D.ctypes.data, x.ctypes.data, cyc.ctypes.data, flags.ctypes.data)
    assert rc == _abi.OK, _lib.lib().cxg_last_error()
    return L, D, x, cyc, flags


@pytest.mark.parametrize("arith", ["fp64", "df64", "fp32"])
@pytest.mark.parametrize("nr,nx", [(12, 12), (32, 30), (45, 40), (64, 64), (100, 90), (189, 189), (192, 170)])
def test_dense_ldlt_matches_numpy(arith, nr, nx):
    K = quasi_definite(nr, nx, seed=nr * 7 + nx)
    b = np.random.default_rng(nr).standard_normal(nr)
    L, D, x, cyc, flags = probe(K, nx, b, arith)
    Lr, Dr = ldlt_ref(K)
    tol = TOL[arith]
    assert flags[0] == 0 and flags[1] == 0
    assert np.all(np.sign(D) == np.sign(Dr))
    assert np.max(np.abs(D - Dr) / np.abs(Dr)) < tol
    assert np.max(np.abs(L - Lr)) < tol * max(1.0, np.max(np.abs(Lr)))
    xr = np.linalg.solve(K, b)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 10 * tol
    assert cyc[0] > 0 and cyc[1] > 0


@pytest.mark.parametrize("threads", [64, 128, 256])
def test_dense_ldlt_block_sizes_agree(threads):
    """The factor does not depend on the block size (same arithmetic order per entry); the solve
    splits its dot products by block size, so x agrees to rounding."""
    K = quasi_definite(100, 96, seed=3)
    b = np.ones(100)
    ref = probe(K, 96, b, "fp64", threads=256)
    got = probe(K, 96, b, "fp64", threads=threads)
    np.testing.assert_array_equal(got[0], ref[0])
    np.testing.assert_array_equal(got[1], ref[1])
    assert np.linalg.norm(got[2] - ref[2]) / np.linalg.norm(ref[2]) < 1e-13


def test_dense_ldlt_regularized_pivot_rule():
    """A zero pivot: plain QDLDL semantics report it; the regularised rule replaces it by +delta
    (RegularizedLdlt::regularizePivot, regularized_ldlt.cpp:132-139)."""
    K = np.diag(np.arange(1.0, 41.0))
    K[1, 1] = 0.0
    b = np.ones(40)
    _, D, _, _, flags = probe(K, 40, b, "fp64", linear_solver=_abi.LINSOLVER_QDLDL)
    assert flags[0] == 1
    _, D, _, _, flags = probe(K, 40, b, "fp64", linear_solver=_abi.LINSOLVER_REGULARIZED)
    assert flags[0] == 0 and D[1] == pytest.approx(1e-7)
