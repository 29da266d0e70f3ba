"""Regenerates the golden fixtures in this directory.

reference_kats.json  -- the known-answer tests of the reference's own test suite (ConicXX
                        test/solver/*.cpp, README.md), transcribed as problem data + expected
                        results with their file:line sources.
oracle_instances.npz -- seeded synthetic instances (contact, random conic QP) with the CPU
                        oracle's solutions (status, iterations, x, s, z, objective).

Run from the repository root:  python tests/golden/make_golden.py
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
    main()
