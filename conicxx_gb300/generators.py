"""Seeded synthetic workload generators.

They restate the problem families of the benchmark configurations the reference's generators
(benchmarks/problem_generators.cpp:58-75, the feasible primal-dual pair construction, and
:300-343, the friction-cone row encoding of README.md:54-67) describe, with the sizes and value
distributions of the workloads this library is measured on. Every instance is a deterministic
function of its seed (numpy PCG64), so the CUDA path and the CPU oracle read identical bytes.
"""
import numpy as np

from .problem import QP, Csc, sym_upper_matvec


def _rng(*key):
    return np.random.Generator(np.random.PCG64(np.random.SeedSequence([int(k) & 0xFFFFFFFF for k in key])))


def _sparse_normal(rng, rows, cols, density, min_per_row=0):
    mask = rng.random((rows, cols)) < density
    if min_per_row:
        empty = np.where(~mask.any(axis=1))[0]
        mask[empty, rng.integers(0, cols, size=empty.size)] = True
    r, c = np.nonzero(mask)
    v = rng.standard_normal(r.size)
    return r, c, v


def _upper_from_structural(Pd, pattern):
    """Upper-triangle CSC of Pd restricted to the structural pattern (diagonal always kept)."""
    n = Pd.shape[0]
    pat = pattern | np.eye(n, dtype=bool)
    pat = np.triu(pat)
    r, c = np.nonzero(pat)
    return Csc.from_coo(n, n, r, c, Pd[r, c])


def _interior(rng, zero, nonneg, soc, free_zero):
    """A strictly interior cone point: Zero rows 0 (or N(0,1) when free_zero, for the dual),
    NN rows U(0.5,1.5), SOC blocks u1 ~ N(0,1), u0 = ||u1|| + U(0.5,1.5)."""
    parts = [rng.standard_normal(zero) if free_zero else np.zeros(zero), rng.uniform(0.5, 1.5, nonneg)]
    for d in soc:
        u1 = rng.standard_normal(d - 1)
        parts.append(np.concatenate([[np.linalg.norm(u1) + rng.uniform(0.5, 1.5)], u1]))
    return np.concatenate(parts) if parts else np.zeros(0)


def random_conic_qp(seed, n=200, m_zero=20, m_nonneg=160, soc=(3,) * 40, density=0.05, p_reg=1e-2,
                    family=0):
    """Random sparse conic QP with a known strictly feasible primal-dual pair.

    P = M'M + p_reg*I (M n x n, `density`, N(0,1); upper triangle stored), A m x n (`density`,
    N(0,1), at least one nonzero per row), x0 ~ N(0,1), interior s0/z0 (z0 free on the Zero
    rows), b = A x0 + s0, q = -P x0 - A' z0."""
    rng = _rng(family, seed)
    soc = list(soc)
    m = m_zero + m_nonneg + sum(soc)
    mr, mc, mv = _sparse_normal(rng, n, n, density)
    M = np.zeros((n, n))
    M[mr, mc] = mv
    Pd = M.T @ M + p_reg * np.eye(n)
    Mb = M != 0
    pattern = (Mb.T.astype(np.int32) @ Mb.astype(np.int32)) > 0
    P = _upper_from_structural(Pd, pattern)
    ar, ac, av = _sparse_normal(rng, m, n, density, min_per_row=1)
    A = Csc.from_coo(m, n, ar, ac, av)
    x0 = rng.standard_normal(n)
    s0 = _interior(rng, m_zero, m_nonneg, soc, free_zero=False)
    z0 = _interior(rng, m_zero, m_nonneg, soc, free_zero=True)
    b = A.matvec(x0) + s0
    q = -sym_upper_matvec(P, x0) - A.rmatvec(z0)
    qp = QP(P=P, q=q, A=A, b=b, zero=m_zero, nonneg=m_nonneg, soc=soc, name=f"random_qp[{seed}]")
    qp.validate()
    return qp


def config0_qp(seed=0):
    """n=200, m=300, K = Zero^20 x R^160_+ x 40 Q^3, 5% density, P reg 1e-2."""
    return random_conic_qp(seed, n=200, m_zero=20, m_nonneg=160, soc=(3,) * 40, family=0)


def config3_qp(seed):
    """n=100, m=150, K = Zero^10 x R^100_+ x 10 Q^4 (the differentiable-layer instances)."""
    return random_conic_qp(seed, n=100, m_zero=10, m_nonneg=100, soc=(4,) * 10, family=3)


def contact_qp(seed, contacts=None, cmin=4, cmax=64):
    """One friction-contact QP (the per-timestep multibody use case).

    c contacts (U{cmin..cmax} unless given), n = 3c forces, k = ceil(c/4) bodies; each contact
    touches 2 distinct random bodies (1 when k = 1) through N(0,1) 3x6 Jacobian blocks;
    Minv is block-diagonal SPD 6x6 per body; P = J Minv J' + 1e-6 I (upper triangle, block
    pattern of contacts sharing a body); q = 0.1 N(0,1). Cones: R^c_+ with rows -e_n (b = 0),
    then c Q^3 with rows [-mu e_n; -e_t1; -e_t2] (b = 0), mu ~ U(0.2, 1.0)."""
    rng = _rng(1, seed)
    c = int(contacts) if contacts is not None else int(rng.integers(cmin, cmax + 1))
    n = 3 * c
    k = (c + 3) // 4
    J = np.zeros((n, 6 * k))
    touch = np.zeros((c, k), dtype=bool)
    for i in range(c):
        bodies = rng.choice(k, size=2, replace=False) if k >= 2 else np.array([0])
        for bd in bodies:
            J[3 * i:3 * i + 3, 6 * bd:6 * bd + 6] = rng.standard_normal((3, 6))
            touch[i, bd] = True
    Minv = np.zeros((6 * k, 6 * k))
    for bd in range(k):
        G = rng.standard_normal((6, 6))
        Minv[6 * bd:6 * bd + 6, 6 * bd:6 * bd + 6] = G @ G.T / 6.0 + 0.5 * np.eye(6)
    Pd = J @ Minv @ J.T + 1e-6 * np.eye(n)
    share = (touch.astype(np.int32) @ touch.T.astype(np.int32)) > 0
    pattern = np.kron(share, np.ones((3, 3), dtype=bool))
    P = _upper_from_structural(Pd, pattern)
    q = 0.1 * rng.standard_normal(n)
    mu = rng.uniform(0.2, 1.0, c)
    rows, cols, vals = [], [], []
    for i in range(c):  # normal non-penetration rows: -f_n + s = 0, s >= 0
        rows.append(i); cols.append(3 * i); vals.append(-1.0)
    for i in range(c):  # friction cone rows: s = (mu f_n, f_t1, f_t2) in Q^3
        r0 = c + 3 * i
        rows += [r0, r0 + 1, r0 + 2]
        cols += [3 * i, 3 * i + 1, 3 * i + 2]
        vals += [-mu[i], -1.0, -1.0]
    m = 4 * c
    A = Csc.from_coo(m, n, rows, cols, vals)
    b = np.zeros(m)
    qp = QP(P=P, q=q, A=A, b=b, zero=0, nonneg=c, soc=[3] * c, name=f"contact[{seed}]")
    qp.validate()
    return qp


def contact_batch(count=4096, base_seed=0, cmin=4, cmax=64):
    """`count` contact instances with c ~ U{cmin..cmax} (the batched contact workload)."""
    return [contact_qp(base_seed + i, cmin=cmin, cmax=cmax) for i in range(count)]


def config3_batch(count=1024, base_seed=0):
    return [config3_qp(base_seed + i) for i in range(count)]


def x_target(seed, n):
    """x_target ~ N(0,1) for the differentiable-layer loss L = 1/2 ||x* - x_target||^2."""
    return _rng(7, seed).standard_normal(n)


def _distinct_per_row(rng, count, upper, k):
    """(count, k) integers in [0, upper), distinct within each row."""
    idx = rng.integers(0, upper, size=(count, k))
    while True:
        srt = np.sort(idx, axis=1)
        dup = (np.diff(srt, axis=1) == 0).any(axis=1)
        if not dup.any():
            return idx
        idx[dup] = rng.integers(0, upper, size=(int(dup.sum()), k))


def _upper_of_gram(F, extra_diag):
    """Upper triangle (CSC) of F'F + extra_diag I for a scipy sparse F (structural pattern)."""
    import scipy.sparse as sp

    G = (F.T @ F + extra_diag * sp.identity(F.shape[1], format="csc")).tocoo()
    keep = G.row <= G.col
    return Csc.from_coo(F.shape[1], F.shape[1], G.row[keep], G.col[keep], G.data[keep])


def large_sparse_qp(seed, n=20000, m_zero=2000, m_nonneg=24000, n_soc=2000, soc_dim=2, m_col_nnz=3, a_row_nnz=8,
                    p_reg=1e-3):
    """One large sparse conic QP (the mixed-precision single-instance workload).

    P = M'M + p_reg I with M n x n holding m_col_nnz N(0,1) entries per column at distinct random
    rows (upper triangle stored); A m x n with a_row_nnz N(0,1) entries per row at distinct random
    columns; cones Zero^m_zero x R^m_nonneg_+ x n_soc Q^soc_dim. Feasible and bounded by the
    primal-dual pair construction of random_conic_qp (x0 ~ N(0,1), interior s0/z0,
    b = A x0 + s0, q = -P x0 - A' z0). Defaults: n = 20000, m = 30000."""
    import scipy.sparse as sp

    rng = _rng(2, seed)
    soc = [soc_dim] * n_soc
    m = m_zero + m_nonneg + soc_dim * n_soc
    mr = _distinct_per_row(rng, n, n, m_col_nnz)
    M = sp.csc_matrix((rng.standard_normal(n * m_col_nnz), (mr.ravel(), np.repeat(np.arange(n), m_col_nnz))),
                      shape=(n, n))
    P = _upper_of_gram(M, p_reg)
    ac = _distinct_per_row(rng, m, n, a_row_nnz)
    A = Csc.from_coo(m, n, np.repeat(np.arange(m), a_row_nnz), ac.ravel(), rng.standard_normal(m * a_row_nnz))
    x0 = rng.standard_normal(n)
    s0 = _interior(rng, m_zero, m_nonneg, soc, free_zero=False)
    z0 = _interior(rng, m_zero, m_nonneg, soc, free_zero=True)
    b = A.matvec(x0) + s0
    q = -sym_upper_matvec(P, x0) - A.rmatvec(z0)
    qp = QP(P=P, q=q, A=A, b=b, zero=m_zero, nonneg=m_nonneg, soc=soc, name=f"large_sparse_qp[{seed}]")
    qp.validate()
    return qp


def group_lasso_socp(seed, groups=4000, group_size=16, rows_per_group=20, row_nnz=12, blocks=64, coupling=0.05,
                     active=0.10, lam=0.1):
    """Group-sparse robust least squares as an SOCP (the block-sparse large-instance workload).

    minimise 1/2 ||F x - g||^2 + lam sum_j t_j  s.t.  ||x_Gj||_2 <= t_j, for `groups` groups of
    `group_size` variables. F is (groups*rows_per_group) x (groups*group_size) with row_nnz N(0,1)
    entries per row: `blocks` diagonal blocks, a fraction `coupling` of each row's entries at
    random columns outside its block. g = F x_true + 0.01 N(0,1), x_true nonzero (N(0,1)) on a
    fraction `active` of the groups. Standard form in the variables (x, t), n = groups *
    (group_size + 1): P = F'F (upper, on x), q = (-F'g, lam 1), one SOC block (t_j, x_Gj) of
    dimension group_size + 1 per group (rows -e, b = 0); the constant 1/2 ||g||^2 is dropped.
    Defaults: 4000 groups of 16, F 80000 x 64000, n = 68000."""
    import scipy.sparse as sp

    rng = _rng(4, seed)
    nx = groups * group_size
    rows = groups * rows_per_group
    blocks = max(1, min(blocks, groups))
    rb = -(-rows // blocks)
    cb = -(-nx // blocks)
    blk = np.minimum(np.arange(rows) // rb, blocks - 1)
    lo = blk * cb
    hi = np.minimum(lo + cb, nx)
    # within-block columns (distinct per row), a fraction replaced by random coupling columns
    width = hi - lo
    u = rng.random((rows, row_nnz))
    cols = lo[:, None] + np.floor(u * width[:, None]).astype(np.int64)
    far = rng.random((rows, row_nnz)) < coupling
    cols[far] = rng.integers(0, nx, size=int(far.sum()))
    F = sp.coo_matrix((rng.standard_normal(rows * row_nnz), (np.repeat(np.arange(rows), row_nnz), cols.ravel())),
                      shape=(rows, nx)).tocsc()
    F.sum_duplicates()
    x_true = np.zeros(nx)
    on = rng.random(groups) < active
    for j in np.where(on)[0]:
        x_true[j * group_size:(j + 1) * group_size] = rng.standard_normal(group_size)
    g = F @ x_true + 0.01 * rng.standard_normal(rows)
    n = nx + groups
    Px = _upper_of_gram(F, 0.0)
    P = Csc((n, n), np.concatenate([Px.indptr, np.full(groups, Px.indptr[-1], np.int32)]).astype(np.int32),
            Px.indices, Px.data)
    q = np.concatenate([-(F.T @ g), np.full(groups, lam)])
    d = group_size + 1
    r, c = [], []
    for j in range(groups):
        r.append(j * d)
        c.append(nx + j)
        for k in range(group_size):
            r.append(j * d + 1 + k)
            c.append(j * group_size + k)
    m = groups * d
    A = Csc.from_coo(m, n, np.asarray(r), np.asarray(c), -np.ones(len(r)))
    b = np.zeros(m)
    qp = QP(P=P, q=q, A=A, b=b, zero=0, nonneg=0, soc=[d] * groups, name=f"group_lasso[{seed}]")
    qp.validate()
    return qp
