"""Host-side problem container: a conic QP in ConicXX's form (README.md:21-33).

    minimise 1/2 x'Px + q'x   s.t.  Ax + s = b,  s in Zero^zero x R^nonneg_+ x Q^soc[0] x ...

P is stored as its upper triangle in CSC, A in CSC, both with 32-bit indices, mirroring
conicxx::SparseMat (include/conicxx/types.h:18).
"""
from dataclasses import dataclass, field
from typing import List

import numpy as np


@dataclass
class Csc:
    """Compressed sparse column matrix (int32 indices, float64 values)."""

    shape: tuple
    indptr: np.ndarray
    indices: np.ndarray
    data: np.ndarray

    @staticmethod
    def from_dense(M, keep_zeros=True, upper=False):
        """Dense -> CSC. keep_zeros keeps explicit zeros (as conicxx::toSparse, convert.cpp:22-40);
        upper keeps only the upper triangle incl. the diagonal (toSparseUpperTriangular)."""
        M = np.asarray(M, dtype=np.float64)
        rows, cols = M.shape
        indptr = [0]
        indices, data = [], []
        for j in range(cols):
            rmax = min(j + 1, rows) if upper else rows
            for i in range(rmax):
                v = M[i, j]
                if keep_zeros or v != 0.0:
                    indices.append(i)
                    data.append(v)
            indptr.append(len(indices))
        return Csc((rows, cols), np.asarray(indptr, np.int32), np.asarray(indices, np.int32),
                   np.asarray(data, np.float64))

    @staticmethod
    def from_triplets(rows, cols, triplets):
        """Like Eigen's setFromTriplets: duplicates are summed, rows sorted per column."""
        acc = {}
        for i, j, v in triplets:
            acc[(j, i)] = acc.get((j, i), 0.0) + float(v)
        keys = sorted(acc)
        indptr = np.zeros(cols + 1, np.int32)
        for (j, _i) in keys:
            indptr[j + 1] += 1
        indptr = np.cumsum(indptr).astype(np.int32)
        indices = np.asarray([i for (_j, i) in keys], np.int32)
        data = np.asarray([acc[k] for k in keys], np.float64)
        return Csc((rows, cols), indptr, indices, data)

    @staticmethod
    def from_coo(rows, cols, r, c, v):
        """Vectorised COO -> CSC (duplicates summed)."""
        r = np.asarray(r, np.int64)
        c = np.asarray(c, np.int64)
        v = np.asarray(v, np.float64)
        key = c * rows + r
        order = np.argsort(key, kind="stable")
        key, v = key[order], v[order]
        uk, start = np.unique(key, return_index=True)
        vals = np.add.reduceat(v, start) if v.size else v
        cc = uk // rows
        rr = uk % rows
        indptr = np.zeros(cols + 1, np.int64)
        np.add.at(indptr, cc + 1, 1)
        indptr = np.cumsum(indptr)
        return Csc((rows, cols), indptr.astype(np.int32), rr.astype(np.int32), vals.astype(np.float64))

    @property
    def nnz(self):
        return int(self.indptr[-1])

    def to_dense(self):
        M = np.zeros(self.shape)
        for j in range(self.shape[1]):
            for k in range(self.indptr[j], self.indptr[j + 1]):
                M[self.indices[k], j] += self.data[k]
        return M

    def col_of_entries(self):
        return np.repeat(np.arange(self.shape[1], dtype=np.int32), np.diff(self.indptr))

    def matvec(self, x):
        y = np.zeros(self.shape[0])
        np.add.at(y, self.indices, self.data * x[self.col_of_entries()])
        return y

    def rmatvec(self, y):
        x = np.zeros(self.shape[1])
        np.add.at(x, self.col_of_entries(), self.data * y[self.indices])
        return x

    def copy(self):
        return Csc(self.shape, self.indptr.copy(), self.indices.copy(), self.data.copy())


def sym_upper_matvec(P: Csc, x):
    """P_sym x from the upper triangle (entries below the diagonal ignored), the product the
    reference forms with selfadjointView<Upper> (src/conicxx/solver_impl.cpp:102)."""
    cols = P.col_of_entries()
    rows = P.indices
    keep = rows <= cols
    r, c, v = rows[keep], cols[keep], P.data[keep]
    y = np.zeros(P.shape[0])
    np.add.at(y, r, v * x[c])
    off = r != c
    np.add.at(y, c[off], v[off] * x[r[off]])
    return y


@dataclass
class QP:
    """One problem instance: P (upper CSC), q, A (CSC), b, cone spec (zero, nonneg, soc dims)."""

    P: Csc
    q: np.ndarray
    A: Csc
    b: np.ndarray
    zero: int = 0
    nonneg: int = 0
    soc: List[int] = field(default_factory=list)
    name: str = ""

    @property
    def n(self):
        return int(self.P.shape[0])

    @property
    def m(self):
        return int(self.zero + self.nonneg + sum(self.soc))

    @staticmethod
    def from_dense(P, q, A, b, zero=0, nonneg=0, soc=(), name=""):
        """QP from dense (numpy) or Csc inputs: the dense-input Solver::setup overloads
        (src/conicxx/solver.cpp:17-30). A dense P becomes its upper triangle with every entry kept
        explicit (toSparseUpperTriangular, convert.cpp:43-70), a dense A every entry explicit
        (toSparse, convert.cpp:22-41), so the pattern stays the same across conversions of new
        values; an asymmetric dense P gets the reference's warning (only its upper triangle is
        read)."""
        if not isinstance(P, Csc):
            Pd = np.asarray(P, dtype=np.float64)
            if Pd.ndim == 2 and Pd.shape[0] == Pd.shape[1] and Pd.size:
                asym = np.max(np.abs(Pd - Pd.T))
                if asym > 1e-8 * max(1.0, np.max(np.abs(Pd))):
                    import warnings

                    warnings.warn("matrix passed as P is not numerically symmetric: only its upper "
                                  "triangle is read", stacklevel=2)
            P = Csc.from_dense(Pd, keep_zeros=True, upper=True)
        if not isinstance(A, Csc):
            A = Csc.from_dense(np.asarray(A, dtype=np.float64), keep_zeros=True)
        qp = QP(P=P, q=np.asarray(q, dtype=np.float64), A=A, b=np.asarray(b, dtype=np.float64), zero=int(zero),
                nonneg=int(nonneg), soc=[int(d) for d in soc], name=name)
        qp.validate()
        return qp

    def validate(self):
        assert self.P.shape == (self.n, self.n)
        assert self.A.shape == (self.m, self.n), (self.A.shape, self.m, self.n)
        assert self.q.shape == (self.n,) and self.b.shape == (self.m,)

    def kkt_residuals(self, x, s, z):
        """(stationarity, feasibility, s'z) of the ORIGINAL problem, as the reference's
        expectKktOptimal helper checks them (test/utils/test_helpers.h:32-48)."""
        st = sym_upper_matvec(self.P, x) + self.A.rmatvec(z) + self.q
        fe = self.A.matvec(x) + s - self.b
        return np.linalg.norm(st), np.linalg.norm(fe), float(s @ z)

    def cone_margins(self, v):
        """(min margin, sum of positive margins) as ConeSet::margins (cone_set.cpp:77-90)."""
        mn, pos = np.inf, 0.0
        off = self.zero
        if self.nonneg:
            mg = float(np.min(v[off:off + self.nonneg]))
            mn, pos = min(mn, mg), pos + max(mg, 0.0)
            off += self.nonneg
        for d in self.soc:
            mg = float(v[off] - np.linalg.norm(v[off + 1:off + d]))
            mn, pos = min(mn, mg), pos + max(mg, 0.0)
            off += d
        return (0.0 if not np.isfinite(mn) else mn), pos
