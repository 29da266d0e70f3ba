"""CPU tests of the host side: the C-ABI surface, input validation, the host equilibration of the
set-up path against the oracle, generators, and multi-rank sharding over gloo."""
import ctypes as C
import os
import socket

import numpy as np
import pytest

from conftest import kat_qp, rel
from conicxx_gb300 import _abi, _lib, generators
from conicxx_gb300._abi import dptr, make_problem_struct
from conicxx_gb300.problem import QP, Csc, sym_upper_matvec
from conicxx_gb300.sharding import gather_solutions, instance_cost, shard_indices


def test_library_exports_every_header_symbol():
    L = _lib.lib()
    syms = _lib.header_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert L.cxg_version().startswith(b"conicxx_gb300")


def test_default_settings_match_reference():
    """include/conicxx/settings.h:21-62."""
    st = _abi.Settings()
    _lib.lib().cxg_default_settings(C.byref(st))
    ref = dict(tol_feas=1e-8, tol_gap_abs=1e-8, tol_gap_rel=1e-8, tol_infeas=1e-7, max_iter=200,
               static_reg_P=1e-8, static_reg_A=1e-8, dynamic_reg_eps=1e-14, dynamic_reg_delta=1e-7,
               refine_max_iter=3, refine_tol=1e-12, max_step_fraction=0.99, equilibrate=1,
               equilibrate_max_iter=10, equilibrate_min_scale=1e-4, equilibrate_max_scale=1e4,
               warm_start=1, linear_solver=_abi.LINSOLVER_QDLDL)
    for k, v in ref.items():
        assert getattr(st, k) == v, k
    py = _abi.default_settings()
    for name, _ in _abi.Settings._fields_:
        if name != "precision":
            assert getattr(py, name) == getattr(st, name), name


def test_status_strings():
    L = _lib.lib()
    assert [L.cxg_status_string(i).decode() for i in range(6)] == [
        "Unsolved", "Solved", "PrimalInfeasible", "DualInfeasible", "MaxIterations", "NumericalError"]


def _setup_rc(qp):
    h = C.c_void_p()
    L = _lib.lib()
    assert L.cxg_solver_create(C.byref(h)) == 0
    prob, keep = make_problem_struct(qp)
    rc = L.cxg_solver_setup(h, C.byref(prob), None)
    L.cxg_solver_destroy(h)
    return rc


def test_invalid_inputs_rejected_before_any_device_work():
    """SolverImpl::setup returns false on an invalid cone spec or mismatched dimensions
    (src/conicxx/solver_impl.cpp:11-16); the C-ABI returns CXG_E_INVALID, on any machine."""
    base = generators.contact_qp(0, contacts=4)
    bad_cone = QP(base.P, base.q, base.A, base.b, nonneg=base.nonneg + 1, soc=base.soc)
    assert _setup_rc(bad_cone) == _abi.E_INVALID
    bad_soc = QP(base.P, base.q, base.A, base.b, nonneg=base.nonneg, soc=[0] + base.soc[1:])
    assert _setup_rc(bad_soc) == _abi.E_INVALID
    A = base.A.copy()
    A.indices = A.indices.copy()
    A.indices[0] = base.m + 5  # row index out of range
    assert _setup_rc(QP(base.P, base.q, A, base.b, nonneg=base.nonneg, soc=base.soc)) == _abi.E_INVALID
    q = base.q.copy()
    q[0] = np.nan
    assert _setup_rc(QP(base.P, q, base.A, base.b, nonneg=base.nonneg, soc=base.soc)) == _abi.E_INVALID
    assert "non-finite" in _lib.lib().cxg_last_error().decode()


def test_solve_before_setup_is_numerical_error():
    """solver_impl.cpp:369-372 of the reference: NumericalError, never a crash."""
    L = _lib.lib()
    h = C.c_void_p()
    assert L.cxg_solver_create(C.byref(h)) == 0
    info = _abi.Info()
    assert L.cxg_solver_solve(h, None, None, None, C.byref(info)) == 0
    assert info.status == _abi.STATUS_NUMERICAL_ERROR
    L.cxg_solver_destroy(h)


@pytest.mark.parametrize("which", ["contact", "cfg3", "cfg0", "badly_scaled"])
def test_host_equilibration_matches_oracle(oracle_mod, which):
    """The set-up path's host equilibration (cxg_plan.cpp) equals the oracle's restatement of
    Equilibration::compute (src/conicxx/kkt/equilibration.cpp:8-100) bit for bit."""
    if which == "contact":
        qp = generators.contact_qp(5)
    elif which == "cfg3":
        qp = generators.config3_qp(2)
    elif which == "cfg0":
        qp = generators.config0_qp(1)
    else:
        P = Csc.from_triplets(3, 3, [(0, 0, 1e6), (1, 1, 1e-4), (2, 2, 50.0)])
        A = Csc.from_triplets(4, 3, [(0, 0, 1e5), (1, 1, 1e-3), (2, 2, 20.0), (3, 0, 1e5), (3, 1, 1e-3), (3, 2, 20.0)])
        qp = QP(P, np.array([3.0, -2, 1]), A, np.array([1.0, 2, 3, 4]), zero=1, nonneg=3)
    prob, keep = make_problem_struct(qp)
    st = _abi.default_settings()
    d, e, c = np.zeros(qp.n), np.zeros(qp.m), C.c_double()
    assert _lib.lib().cxg_equilibration(C.byref(prob), C.byref(st), dptr(d), dptr(e), C.byref(c)) == 0
    S = oracle_mod.OracleSolver()
    assert S.setup(qp)
    do, eo, co = S.equilibration()
    assert np.array_equal(d, do) and np.array_equal(e, eo) and c.value == co


def test_generators_deterministic_and_feasible():
    a, b = generators.contact_qp(3), generators.contact_qp(3)
    assert np.array_equal(a.P.data, b.P.data) and np.array_equal(a.q, b.q)
    for qp in (generators.config0_qp(0), generators.config3_qp(0), generators.contact_qp(1)):
        qp.validate()
        P = qp.P
        assert np.all(P.indices <= P.col_of_entries())  # upper triangle only
    qp = generators.config0_qp(0)
    assert qp.n == 200 and qp.m == 300 and qp.zero == 20 and qp.nonneg == 160 and qp.soc == [3] * 40
    qp = generators.config3_qp(0)
    assert qp.n == 100 and qp.m == 150 and qp.soc == [4] * 10
    c = generators.contact_qp(7)
    nc = c.n // 3
    assert 4 <= nc <= 64 and c.m == 4 * nc and c.nonneg == nc and c.soc == [3] * nc
    # P = J Minv J' + 1e-6 I is PSD with the regularisation as smallest eigenvalue bound
    Pd = c.P.to_dense()
    Pd = np.triu(Pd) + np.triu(Pd, 1).T
    assert np.linalg.eigvalsh(Pd).min() > 0.5e-6


def test_large_instance_generators():
    """The single large-instance families: shapes, structure and the primal-dual pair construction
    (b - A x0 interior to the cone, known from the generator's seeded draws) at reduced size, and
    the full configuration 2 shape."""
    qp = generators.large_sparse_qp(0, n=1000, m_zero=100, m_nonneg=1200, n_soc=100)
    assert qp.n == 1000 and qp.m == 1500 and qp.zero == 100 and qp.nonneg == 1200 and qp.soc == [2] * 100
    assert np.all(np.diff(qp.A.indptr) >= 0)
    rows_per = np.bincount(qp.A.indices, minlength=qp.m)
    assert np.all(rows_per == 8)  # 8 distinct nonzeros per row of A
    assert np.all(qp.P.indices <= qp.P.col_of_entries())
    Pd = qp.P.to_dense()
    Pd = np.triu(Pd) + np.triu(Pd, 1).T
    assert np.linalg.eigvalsh(Pd).min() > 0.9e-3  # M'M + 1e-3 I
    a, b = generators.large_sparse_qp(0, n=300, m_zero=30, m_nonneg=360, n_soc=30), \
        generators.large_sparse_qp(0, n=300, m_zero=30, m_nonneg=360, n_soc=30)
    assert np.array_equal(a.A.data, b.A.data) and np.array_equal(a.q, b.q)
    full = generators.large_sparse_qp(0)
    assert full.n == 20000 and full.m == 30000 and full.zero == 2000 and full.nonneg == 24000
    assert full.A.nnz == 240000
    g = generators.group_lasso_socp(0, groups=60)
    assert g.n == 60 * 17 and g.m == 60 * 17 and g.soc == [17] * 60 and g.zero == 0 and g.nonneg == 0
    # each SOC block is (t_j, x_Gj): rows -e on t_j and the group's 16 x entries
    assert g.A.nnz == 60 * 17 and np.all(g.A.data == -1.0)
    assert np.all(g.q[60 * 16:] == 0.1)


def test_whole_gpu_setting_rejections():
    """Roots above the one-CTA limit are refused when the whole-GPU form is switched off or the
    handle is a batch of several instances (host checks, no device work)."""
    n = 4200
    P = Csc.from_coo(n, n, np.arange(n), np.arange(n), np.ones(n))
    A = Csc.from_coo(1, n, [0], [0], [-1.0])
    qp = QP(P, np.zeros(n), A, np.ones(1), 0, 1, [])
    prob, keep = make_problem_struct(qp)
    st = _abi.default_settings(whole_gpu_root=-1)
    h = C.c_void_p()
    assert _lib.lib().cxg_batch_create(C.byref(h), 1, C.byref(prob), C.byref(st)) == _abi.E_UNSUPPORTED
    assert b"4096" in _lib.lib().cxg_last_error()
    arr = (_abi.Problem * 2)(prob, prob)
    st = _abi.default_settings()
    assert _lib.lib().cxg_batch_create(C.byref(h), 2, arr, C.byref(st)) == _abi.E_UNSUPPORTED
    # the whole-GPU root's limit (131072 rows; the scatter maps hold 64-bit root element offsets)
    n = 131073
    P = Csc.from_coo(n, n, np.arange(n), np.arange(n), np.ones(n))
    A = Csc.from_coo(1, n, [0], [0], [-1.0])
    big = QP(P, np.zeros(n), A, np.ones(1), 0, 1, [])
    prob, keep = make_problem_struct(big)
    st = _abi.default_settings(whole_gpu_root=1)
    assert _lib.lib().cxg_batch_create(C.byref(h), 1, C.byref(prob), C.byref(st)) == _abi.E_UNSUPPORTED
    assert b"131072" in _lib.lib().cxg_last_error()


def _root_idx(nr, i, j):
    """Element offset of root entry (i, j), i >= j: lower triangle of 32x32 tiles in column-major
    tile order, each tile column-major with leading dimension 33 (the device layout)."""
    T = -(-nr // 32)
    I, J = i // 32, j // 32
    return (J * T - J * (J - 1) // 2 + (I - J)) * 32 * 33 + (j % 32) * 33 + (i % 32)


def test_plan_root_offsets_above_2_31():
    """The plan of a 68000-row root (the full-size group-lasso root, 2.39e9 entries): scatter
    offsets above 2^31 come out exact and 8-byte aligned in the int pool (host planning only)."""
    n = 68000
    rows = list(range(n)) + [n - 2, 100]
    cols = list(range(n)) + [n - 1, n - 3]
    P = Csc.from_coo(n, n, rows, cols, np.ones(len(rows)))
    # Zero row 0 on column n - 10; NN row 1 on columns n - 5, n - 4; SOC (dim 2) rows 2, 3 on n - 7, n - 6
    A = Csc.from_coo(4, n, [0, 1, 1, 2, 3], [n - 10, n - 5, n - 4, n - 7, n - 6], [1.0, -1.0, -1.0, -1.0, -1.0])
    qp = QP(P, np.zeros(n), A, np.ones(4), 1, 1, [2])
    prob, keep = make_problem_struct(qp)
    st = _abi.default_settings()
    counts = np.zeros(9, np.int64)
    cap = 16
    plow, az, tgt = (np.zeros(cap, np.int64) for _ in range(3))
    ptr = lambda a: a.ctypes.data_as(_lib.i64p)  # noqa: E731
    assert _lib.lib().cxg_plan_inspect(C.byref(prob), C.byref(st), ptr(counts), ptr(plow), ptr(az), ptr(tgt), cap) == 0
    nr = n + 1
    T = -(-nr // 32)
    assert counts[0] == nr and counts[1] == T * (T + 1) // 2 * 32 * 33 > 2**31
    assert counts[8] == 1
    assert counts[2] == 2 and sorted(plow[:2].tolist()) == sorted([_root_idx(nr, n - 3, 100), _root_idx(nr, n - 1, n - 2)])
    assert max(plow[:2]) > 2**31
    assert counts[3] == 1 and az[0] == _root_idx(nr, n, n - 10) and az[0] > 2**31
    want = sorted({_root_idx(nr, i, j) for (i, j) in [(n - 5, n - 5), (n - 4, n - 5), (n - 4, n - 4),
                                                         (n - 7, n - 7), (n - 6, n - 7), (n - 6, n - 6)]})
    assert counts[4] == len(want) and tgt[:len(want)].tolist() == want and min(want) > 2**31


def test_plan_counts_beyond_32_bits_refused():
    """A plan count the device indexes with 32-bit ints is computed from the pattern and refused
    (CXG_E_UNSUPPORTED) before any plan array or device work: one SOC block of dimension 50000
    whose rows touch 50000 distinct columns densifies to 2.5e9 A-block entries."""
    n = 50000
    P = Csc.from_coo(n, n, np.arange(n), np.arange(n), np.ones(n))
    A = Csc.from_coo(n, n, np.arange(n), np.arange(n), -np.ones(n))
    qp = QP(P, np.zeros(n), A, np.concatenate([[1.0], np.zeros(n - 1)]), 0, 0, [n])
    prob, keep = make_problem_struct(qp)
    st = _abi.default_settings(whole_gpu_root=1)
    h = C.c_void_p()
    assert _lib.lib().cxg_batch_create(C.byref(h), 1, C.byref(prob), C.byref(st)) == _abi.E_UNSUPPORTED
    assert b"32-bit" in _lib.lib().cxg_last_error()
    counts = np.zeros(9, np.int64)
    assert _lib.lib().cxg_plan_inspect(C.byref(prob), C.byref(st), counts.ctypes.data_as(_lib.i64p), None, None, None,
                                       0) == _abi.E_UNSUPPORTED


def test_dense_inputs_convert_like_the_reference():
    """QP.from_dense (the dense-input setup overloads): P's upper triangle and all of A with every
    entry explicit, the same products as the sparse problem, and the reference's warning for an
    asymmetric P."""
    import warnings

    P = np.eye(3)
    A = np.array([[1.0, 1, 0], [0, 0, -1], [0, 0, -1], [-1, 0, 0], [0, -1, 0]])
    q, b = np.array([-1.0, -1, -0.3]), np.array([1.0, 0, 0, 0, 0])
    qp = QP.from_dense(P, q, A, b, zero=1, nonneg=1, soc=[3])
    assert qp.P.nnz == 6 and qp.A.nnz == 15  # upper triangle of 3x3, all 5x3 entries
    assert np.all(qp.P.indices <= qp.P.col_of_entries())
    x = np.array([0.3, -0.7, 1.1])
    assert np.allclose(sym_upper_matvec(qp.P, x), P @ x) and np.allclose(qp.A.matvec(x), A @ x)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        QP.from_dense(np.array([[1.0, 2.0], [0.0, 1.0]]), np.zeros(2), np.eye(2), np.ones(2), nonneg=2)
    assert any("symmetric" in str(x_.message) for x_ in w)


def test_sharding_balanced():
    qps = generators.contact_batch(64)
    costs = [instance_cost(q) for q in qps]
    shards = shard_indices(costs, 4)
    assert sorted(np.concatenate(shards).tolist()) == list(range(64))
    loads = [sum(costs[i] for i in s) for s in shards]
    assert max(loads) / min(loads) < 1.15


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _gloo_worker(rank, world, port, result_q):
    import sys

    import torch.distributed as dist

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    import oracle as orc
    from conicxx_gb300 import generators as G
    from conicxx_gb300.sharding import gather_solutions as gs
    from conicxx_gb300.sharding import instance_cost as ic
    from conicxx_gb300.sharding import shard_indices as si

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    qps = [G.contact_qp(i, cmin=4, cmax=10) for i in range(12)]
    mine = si([ic(q) for q in qps], world)[rank]
    xs, st = [], []
    for i in mine:  # each rank solves its shard (the oracle stands in for the GPU on CPU)
        x, s, z, info, _ = orc.solve(qps[i])
        xs.append(x)
        st.append(info["status"])
    allx, allst = gs(mine, xs, st, len(qps))
    if rank == 0:
        ref = [orc.solve(q) for q in qps]
        ok = all(np.allclose(a, r[0]) for a, r in zip(allx, ref))
        ok = ok and all(int(st) == r[3]["status"] for st, r in zip(allst, ref))
        result_q.put(bool(ok))
    dist.barrier()
    dist.destroy_process_group()


def test_multi_rank_sharded_solve_gloo():
    """world_size-2 run of the instance-sharded path over gloo: no data-path collective, results
    gathered on the host match a single-process solve."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gloo_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    assert q.get(timeout=10) is True
