"""Regenerates the golden fixtures in this directory.

reference_kats.json  -- the known-answer tests of the reference's own test suite (ConicXX
                        test/solver/*.cpp, README.md), transcribed as problem data + expected
                        results with their file:line sources.
oracle_instances.npz -- seeded synthetic instances (contact, random conic QP) with the CPU
                        oracle's solutions (status, iterations, x, s, z, objective).
oracle_large.npz     -- configuration 2's family (generators.large_sparse_qp, seed 0) at n = 2000
                        and 3000: the oracle's solutions at the default tolerances (1e-8) and, at
                        n = 2000, at 1e-10 ("n2000t"), with a checksum of the generated problem
                        (the problem itself is regenerated from its seed by the tests).

Run from the repository root:  python tests/golden/make_golden.py [--large]
(--large writes oracle_large.npz only; its oracle solves take several minutes.)
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from conicxx_gb300 import generators  # noqa: E402


def kats():
    """Solver known-answer tests (problem as triplets; P given by its upper triangle)."""
    return [
        dict(name="eq_qp", source="test/solver/test_solve_qp.cpp:9-34", n=2, m=1,
             P=[[0, 0, 1.0], [1, 1, 1.0]], q=[0.0, 0.0], A=[[0, 0, 1.0], [0, 1, 1.0]], b=[1.0],
             zero=1, nonneg=0, soc=[], status=1, x=[0.5, 0.5], objective=0.25, tol=1e-6),
        dict(name="box_qp", source="test/solver/test_solve_qp.cpp:36-66", n=2, m=2,
             P=[[0, 0, 1.0], [1, 1, 1.0]], q=[1.0, -2.0], A=[[0, 0, -1.0], [1, 1, -1.0]], b=[0.0, 0.0],
             zero=0, nonneg=2, soc=[], status=1, x=[0.0, 2.0], objective=-2.0, tol=1e-6),
        dict(name="lp_vertex", source="test/solver/test_solve_lp.cpp:9-37", n=2, m=3,
             P=[], q=[-1.0, -2.0], A=[[0, 0, 1.0], [0, 1, 1.0], [1, 0, -1.0], [2, 1, -1.0]], b=[1.0, 0.0, 0.0],
             zero=0, nonneg=3, soc=[], status=1, x=[0.0, 1.0], objective=-2.0, tol=1e-6),
        dict(name="socp_min_first", source="test/solver/test_solve_socp.cpp:11-42", n=3, m=4,
             P=[], q=[1.0, 0.0, 0.0], A=[[0, 1, 1.0], [1, 0, -1.0], [2, 1, -1.0], [3, 2, -1.0]],
             b=[1.0, 0.0, 0.0, 0.0], zero=1, nonneg=0, soc=[3], status=1, x=[1.0, 1.0, 0.0], objective=1.0,
             tol=1e-5),
        dict(name="friction_projection", source="test/solver/test_solve_friction_qp_soc.cpp:17-51", n=3, m=3,
             P=[[0, 0, 1.0], [1, 1, 1.0], [2, 2, 1.0]], q=[-1.0, -3.0, -4.0],
             A=[[0, 0, -1.0], [1, 1, -1.0], [2, 2, -1.0]], b=[0.0, 0.0, 0.0], zero=0, nonneg=0, soc=[3],
             status=1, x=[3.0, 1.8, 2.4], objective=None, tol=1e-5),
        dict(name="primal_infeasible", source="test/solver/test_infeasible.cpp:9-29", n=1, m=2,
             P=[], q=[0.0], A=[[0, 0, -1.0], [1, 0, 1.0]], b=[-1.0, 0.0], zero=0, nonneg=2, soc=[],
             status=2, x=None, objective=None, tol=None),
        dict(name="dual_infeasible", source="test/solver/test_infeasible.cpp:31-50", n=1, m=1,
             P=[], q=[-1.0], A=[[0, 0, -1.0]], b=[0.0], zero=0, nonneg=1, soc=[],
             status=3, x=None, objective=None, tol=None),
        dict(name="readme_example", source="README.md:84-123", n=3, m=5,
             P=[[0, 0, 1.0], [1, 1, 1.0], [2, 2, 1.0]], q=[-1.0, -1.0, -0.3],
             A=[[0, 0, 1.0], [0, 1, 1.0], [1, 2, -1.0], [2, 2, -1.0], [3, 0, -1.0], [4, 1, -1.0]],
             b=[1.0, 0.0, 0.0, 0.0, 0.0], zero=1, nonneg=1, soc=[3], status=1,
             x=[0.5, 0.5, float(np.sqrt(0.5))], objective=None, tol=1e-6),
    ]


def instances():
    """(name, QP) pairs for the oracle golden file: contact instances of assorted sizes and the
    random conic QPs of the two small configurations."""
    out = []
    for seed, c in [(11, 4), (12, 9), (13, 17), (14, 33), (15, 48), (16, 64)]:
        out.append((f"contact_c{c}", generators.contact_qp(seed, contacts=c)))
    out.append(("cfg3_seed0", generators.config3_qp(0)))
    out.append(("cfg3_seed1", generators.config3_qp(1)))
    out.append(("cfg0_seed0", generators.config0_qp(0)))
    return out


def large_family(n):
    """Configuration 2's family scaled to n variables (the proportions of n = 20000)."""
    f = n / 20000
    return generators.large_sparse_qp(0, n=n, m_zero=int(2000 * f), m_nonneg=int(24000 * f), n_soc=int(2000 * f))


def problem_checksum(qp):
    return np.array([qp.P.data.sum(), qp.A.data.sum(), qp.q.sum(), qp.b.sum(), qp.P.nnz, qp.A.nnz])


def main_large():
    import oracle as orc

    orc.build()
    arrays = {}
    for n, tol in ((2000, 1e-8), (3000, 1e-8), (2000, 1e-10)):
        qp = large_family(n)
        x, s, z, info, _ = orc.solve(qp, warm_start=0, tol_feas=tol, tol_gap_abs=tol, tol_gap_rel=tol)
        p = f"n{n}/" if tol == 1e-8 else f"n{n}t/"
        arrays[p + "checksum"] = problem_checksum(qp)
        arrays[p + "x"], arrays[p + "s"], arrays[p + "z"] = x, s, z
        arrays[p + "info"] = np.array([info["status"], info["iterations"], info["objective"]])
        print("large family n", n, "tol", tol, "status", info["status"], "iterations", info["iterations"], flush=True)
    np.savez_compressed(os.path.join(HERE, "oracle_large.npz"), **arrays)


def main():
    import oracle as orc

    orc.build()
    with open(os.path.join(HERE, "reference_kats.json"), "w") as f:
        json.dump(kats(), f, indent=1)
    arrays = {}
    names = []
    for name, qp in instances():
        x, s, z, info, _ = orc.solve(qp)
        names.append(name)
        p = name + "/"
        arrays[p + "Pp"], arrays[p + "Pi"], arrays[p + "Px"] = qp.P.indptr, qp.P.indices, qp.P.data
        arrays[p + "Ap"], arrays[p + "Ai"], arrays[p + "Ax"] = qp.A.indptr, qp.A.indices, qp.A.data
        arrays[p + "q"], arrays[p + "b"] = qp.q, qp.b
        arrays[p + "cones"] = np.array([qp.zero, qp.nonneg] + list(qp.soc), np.int32)
        arrays[p + "x"], arrays[p + "s"], arrays[p + "z"] = x, s, z
        arrays[p + "info"] = np.array([info["status"], info["iterations"], info["objective"]])
        print(name, "n", qp.n, "m", qp.m, "status", info["status"], "iterations", info["iterations"])
    arrays["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "oracle_instances.npz"), **arrays)


if __name__ == "__main__":
    if "--large" in sys.argv:
        main_large()
    else:
        main()
