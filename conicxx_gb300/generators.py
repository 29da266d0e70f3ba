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
