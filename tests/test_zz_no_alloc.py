"""GPU tests of cxg_batch_solve_device_noalloc, the allocation-free batch solve whose IPM working
memory is a fixed device array instead of the batch's own scratch.

The file name sorts last, so in a full run these tests also run after every other GPU test of
the same process; they must pass alone in a fresh process too.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel
from conicxx_gb300 import _abi, _lib, generators
from conicxx_gb300.problem import QP, Csc

pytestmark = pytest.mark.gpu
SOL_TOL = 1e-10  # same kernel on the same inputs: only the CTA that runs an instance differs


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if _lib.lib().cxg_device_count() < 1 or not torch.cuda.is_available():
        pytest.fail("a CUDA device is required for the -m gpu tests")
    return torch


def _buffers(torch, B, fill):
    dev = torch.device("cuda", 0)
    N, M = int(B.n_off[-1]), int(B.m_off[-1])
    return [torch.full((k,), fill, dtype=torch.float64, device=dev) for k in (N, M, M)]


def _noalloc(B, bufs, infos, stream):
    return _lib.lib().cxg_batch_solve_device_noalloc(
        B._h, *[t.data_ptr() for t in bufs], infos.ctypes.data_as(C.POINTER(_abi.Info)), stream)


@pytest.mark.parametrize("precision", [_abi.PRECISION_MIXED, _abi.PRECISION_FP64])
def test_noalloc_matches_device_solve(torch_cuda, precision):
    """Two allocation-free solves in a row give the statuses, iteration counts and x, s, z of the
    regular device solve (warm start off, so every solve starts from the same point)."""
    from conicxx_gb300 import BatchSolver

    torch = torch_cuda
    qps = [generators.contact_qp(700 + i, cmax=40) for i in range(12)] + \
          [generators.config3_qp(40 + i) for i in range(4)]
    B = BatchSolver(qps, warm_start=0, precision=precision)
    stream = torch.cuda.current_stream().cuda_stream
    ref = _buffers(torch, B, 0.0)
    infos_ref = np.zeros(B.count, dtype=_abi.INFO_DTYPE)
    B.solve_device(*[t.data_ptr() for t in ref], stream, infos_ref)
    torch.cuda.synchronize()
    assert (infos_ref["status"] == _abi.STATUS_SOLVED).sum() >= B.count - 1
    ref_host = [t.cpu().numpy() for t in ref]
    for call in range(2):
        out = _buffers(torch, B, float("nan"))
        infos = np.zeros(B.count, dtype=_abi.INFO_DTYPE)
        rc = _noalloc(B, out, infos, stream)
        assert rc == _abi.OK, _lib.lib().cxg_last_error()
        torch.cuda.synchronize()
        assert B.last_launches() >= 1
        np.testing.assert_array_equal(infos["status"], infos_ref["status"])
        np.testing.assert_array_equal(infos["iterations"], infos_ref["iterations"])
        for name, got, want in zip("xsz", out, ref_host):
            got = got.cpu().numpy()
            assert np.all(np.isfinite(got)), (call, name)
            assert rel(got, want) < SOL_TOL, (call, name, rel(got, want))


def test_noalloc_rejects_oversized_instance(torch_cuda):
    """One FP64 instance whose root (nr = 2900: 4186 tiles of 32x33 doubles, 35 MB) exceeds the
    fixed working memory is refused before anything is launched."""
    from conicxx_gb300 import BatchSolver

    torch = torch_cuda
    n, m = 2900, 60
    rng = np.random.default_rng(0)
    P = Csc.from_coo(n, n, np.arange(n), np.arange(n), np.ones(n))
    rows = np.arange(m)
    A = Csc.from_coo(m, n, rows, rng.integers(0, n, m), -np.ones(m))
    qp = QP(P, rng.standard_normal(n), A, np.ones(m), 0, m, [])
    B = BatchSolver([qp], warm_start=0, precision=_abi.PRECISION_FP64)
    out = _buffers(torch, B, 0.0)
    infos = np.zeros(B.count, dtype=_abi.INFO_DTYPE)
    rc = _noalloc(B, out, infos, torch.cuda.current_stream().cuda_stream)
    assert rc == _abi.E_UNSUPPORTED
    assert b"fixed scratch" in _lib.lib().cxg_last_error()


def test_noalloc_grid_cut_to_the_fixed_array(torch_cuda):
    """128 FP64 instances of the n = 200, m = 300 random conic QP: their 220-row roots do not fit in
    shared memory, so each CTA's working memory (root included) is about 0.36 MB, and a grid of
    128 CTAs needs more than the fixed array holds; the entry point runs the bucket on fewer CTAs.
    Statuses, iterations and x, s, z still equal the regular device solve's."""
    from conicxx_gb300 import BatchSolver

    torch = torch_cuda
    qps = [generators.config0_qp(700 + i) for i in range(128)]
    B = BatchSolver(qps, warm_start=0, precision=_abi.PRECISION_FP64)
    cap = (32 << 20) - 256  # CXG_NOALLOC_SCRATCH_BYTES less the queue counters
    cut = [ln for ln in B.describe().splitlines()
           if int(ln.split("grid=")[1].split()[0]) * int(ln.split("scratchPerCTA=")[1].split()[0]) * 8 > cap]
    assert cut, B.describe()  # the grid cut is exercised
    stream = torch.cuda.current_stream().cuda_stream
    ref = _buffers(torch, B, 0.0)
    infos_ref = np.zeros(B.count, dtype=_abi.INFO_DTYPE)
    B.solve_device(*[t.data_ptr() for t in ref], stream, infos_ref)
    torch.cuda.synchronize()
    ref_host = [t.cpu().numpy() for t in ref]
    out = _buffers(torch, B, float("nan"))
    infos = np.zeros(B.count, dtype=_abi.INFO_DTYPE)
    rc = _noalloc(B, out, infos, stream)
    assert rc == _abi.OK, _lib.lib().cxg_last_error()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(infos["status"], infos_ref["status"])
    np.testing.assert_array_equal(infos["iterations"], infos_ref["iterations"])
    for name, got, want in zip("xsz", out, ref_host):
        assert rel(got.cpu().numpy(), want) < SOL_TOL, name
