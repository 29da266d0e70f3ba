"""Shared test fixtures.

Tests marked `gpu` run on a GB300 through the C-ABI; everything else runs on the CPU (oracle
checks against the reference's known answers, host logic, ABI surface, multi-process gloo).
"""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

from conicxx_gb300.problem import QP, Csc  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def kat_qp(k):
    """QP of a known-answer test record (tests/golden/reference_kats.json)."""
    n, m = k["n"], k["m"]
    P = Csc.from_triplets(n, n, k["P"]) if k["P"] else Csc((n, n), np.zeros(n + 1, np.int32),
                                                          np.zeros(0, np.int32), np.zeros(0))
    A = Csc.from_triplets(m, n, k["A"])
    return QP(P, np.asarray(k["q"], float), A, np.asarray(k["b"], float), zero=k["zero"], nonneg=k["nonneg"],
              soc=list(k["soc"]), name=k["name"])


def load_kats():
    with open(os.path.join(GOLDEN, "reference_kats.json")) as f:
        return json.load(f)


def load_golden_instances():
    """[(name, QP, expected dict)] from tests/golden/oracle_instances.npz."""
    d = np.load(os.path.join(GOLDEN, "oracle_instances.npz"))
    out = []
    for name in d["names"]:
        name = str(name)
        g = lambda k: d[name + "/" + k]  # noqa: E731
        cones = g("cones")
        n = len(g("Pp")) - 1
        m = len(g("b"))
        qp = QP(Csc((n, n), g("Pp"), g("Pi"), g("Px")), g("q"), Csc((m, n), g("Ap"), g("Ai"), g("Ax")), g("b"),
                zero=int(cones[0]), nonneg=int(cones[1]), soc=[int(v) for v in cones[2:]], name=name)
        info = g("info")
        out.append((name, qp, dict(status=int(info[0]), iterations=int(info[1]), objective=float(info[2]),
                                   x=g("x"), s=g("s"), z=g("z"))))
    return out


@pytest.fixture(scope="session")
def kats():
    return load_kats()


@pytest.fixture(scope="session")
def golden_instances():
    return load_golden_instances()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build()
    return oracle


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-12))
