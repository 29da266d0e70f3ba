"""Diagnostic: time the dense root LDL' and triangular solve (cxg_dense_ldlt) on a seeded
quasi-definite matrix of the reduced-KKT shape [P, A_Z'; A_Z, -0.5 I].

    python -m conicxx_gb300.probe --nr 8192 --nx 7936 --arith fp32 --threads -1

--threads -1 runs the whole-GPU root (every SM); 32..256 the one-CTA root (roots that fit in
shared memory). Prints one JSON line: factor and solve time, multiply-adds per second, the
solution's relative error against a float64 solve (when --check), and the pivot flags.
"""
import argparse
import json

import numpy as np

from . import _abi, _lib

ARITH = {"fp64": 0, "fp32": 1, "df64": 2}


def quasi_definite(nr, nx, seed):
    """P = B B'/nx + I (nx x nx), A_Z ~ 0.5 N(0,1) ((nr - nx) x nx), -0.5 I on the Zero rows;
    column-major."""
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((nx, nx), dtype=np.float64)
    K = np.zeros((nr, nr), order="F")
    K[:nx, :nx] = B @ B.T / nx + np.eye(nx)
    AZ = rng.standard_normal((nr - nx, nx)) * 0.5
    K[nx:, :nx] = AZ
    K[:nx, nx:] = AZ.T
    K[nx:, nx:] = -0.5 * np.eye(nr - nx)
    return K


def run(nr, nx, arith, threads, seed=1, check=False, linear_solver=_abi.LINSOLVER_QDLDL):
    K = quasi_definite(nr, nx, seed)
    b = np.random.default_rng(seed + 1).standard_normal(nr)
    D, x = np.zeros(nr), np.zeros(nr)
    cyc = np.zeros(2, np.int64)
    flags = np.zeros(3, np.int32)
    rc = _lib.lib().cxg_dense_ldlt(nr, nx, K.ctypes.data, b.ctypes.data, ARITH[arith], threads, linear_solver,
                                   None, D.ctypes.data, x.ctypes.data, cyc.ctypes.data, flags.ctypes.data)
    if rc != _abi.OK:
        raise RuntimeError(_lib.lib().cxg_last_error().decode())
    out = {"nr": nr, "nx": nx, "arith": arith, "threads": threads, "flags": flags.tolist()}
    fma = nr ** 3 / 6.0
    if threads < 0:  # nanoseconds from the device global timer
        out.update(ldlt_ms=cyc[0] / 1e6, solve_ms=cyc[1] / 1e6, ldlt_fma_per_s=fma / (cyc[0] * 1e-9))
    else:  # SM clock cycles
        out.update(ldlt_cycles=int(cyc[0]), solve_cycles=int(cyc[1]))
    if check:
        xs = np.linalg.solve(K, b)
        out["x_rel_err"] = float(np.linalg.norm(x - xs) / np.linalg.norm(xs))
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--nr", type=int, default=8192)
    ap.add_argument("--nx", type=int, default=None, help="rows with positive pivots (default nr - 256)")
    ap.add_argument("--arith", choices=sorted(ARITH), default="fp32")
    ap.add_argument("--threads", type=int, default=-1)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--check", action="store_true")
    a = ap.parse_args()
    nx = a.nx if a.nx is not None else max(1, a.nr - 256)
    for _ in range(a.repeat):
        print(json.dumps(run(a.nr, nx, a.arith, a.threads, check=a.check)), flush=True)


if __name__ == "__main__":
    main()
