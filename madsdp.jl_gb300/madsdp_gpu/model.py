"""Problem data of a mixed PSD + nonnegative-orthant SDP.

This mirrors the constructor of ``LowRankOpt.Model(C, A, b, d_lin, C_lin,
sides)`` as MadSDP's tests and benchmark call it (test/runtests.jl:16-31,
test/runtests.jl:36-56, benchmark/maxcut.jl:28-40):

    min   sum_i <C_i, X_i> + d_lin' x
    s.t.  sum_i <A_ij, X_i> + (C_lin x)_j = b_j      j = 1..m
          X_i PSD (side n_i),  x >= 0 (ns scalars)

Its dual is  max b'y  s.t.  S_i = C_i - sum_j y_j A_ij PSD,
z = d_lin - C_lin' y >= 0 (src/step.jl:4-11, src/solver.jl:192-211).

Storage chosen for the device path:

* ``C[i]``: dense ``n_i x n_i`` float64 (symmetric).
* ``A[i]``: the constraint matrices of block ``i`` as a coordinate list
  of *full* symmetric entries (both triangles), sorted by constraint and
  then by column-major position: arrays ``con, row, col`` (int32) and
  ``val``.  A one-hot constraint ``e_k e_k'`` is one entry, a Hankel 0/1
  constraint ``sum_{a+b=k} E_ab`` is up to ``n`` entries, a dense
  constraint is ``n^2`` entries.
* ``b`` (m), ``d_lin`` (ns), ``C_lin`` (m x ns, column-major) dense float64.
"""

from __future__ import annotations

import numpy as np

__all__ = ["BlockConstraints", "Model"]


class BlockConstraints:
    """Coordinate list of the symmetric matrices ``A_ij`` of one block."""

    def __init__(self, n: int, m: int, con, row, col, val):
        con = np.asarray(con)
        row = np.asarray(row)
        col = np.asarray(col)
        val = np.asarray(val, dtype=np.float64)
        if not (con.shape == row.shape == col.shape == val.shape):
            raise ValueError("coordinate arrays must have the same length")
        keep = val != 0.0
        if not keep.all():
            con, row, col, val = con[keep], row[keep], col[keep], val[keep]
        if con.size and (con.min() < 0 or con.max() >= m):
            raise ValueError("constraint index out of range")
        if row.size and (min(row.min(), col.min()) < 0 or max(row.max(), col.max()) >= n):
            raise ValueError("entry index out of range")
        self.n = int(n)
        self.m = int(m)
        # (constraint, column, row) order; input already in that order (the
        # generators' and a column-major walk's) is kept without a sort
        key = (con.astype(np.int64) * n + col) * n + row
        if key.size < 2 or bool(np.all(key[1:] >= key[:-1])):
            order = slice(None)
        else:
            order = np.argsort(key, kind="stable")
        del key
        # int32 indices and contiguous values: the layout the C ABI reads,
        # so that a batch passes these arrays to it without copies
        self.con = np.ascontiguousarray(con[order], dtype=np.int32)
        self.row = np.ascontiguousarray(row[order], dtype=np.int32)
        self.col = np.ascontiguousarray(col[order], dtype=np.int32)
        self.val = np.ascontiguousarray(val[order])
        # constraint pointer (CSR over constraints)
        self.ptr = np.zeros(m + 1, dtype=np.int64)
        self.ptr[1:] = np.cumsum(np.bincount(self.con, minlength=m))

    @property
    def nnz(self) -> int:
        return int(self.val.size)

    @classmethod
    def from_dense_list(cls, n: int, mats) -> "BlockConstraints":
        """From a list of ``m`` symmetric ``n x n`` matrices (None = zero)."""
        m = len(mats)
        cons, rows, cols, vals = [], [], [], []
        for j, A in enumerate(mats):
            if A is None:
                continue
            A = np.asarray(A, dtype=np.float64)
            if A.shape != (n, n):
                raise ValueError("constraint matrix has the wrong shape")
            if not np.array_equal(A, A.T):
                raise ValueError("constraint matrices must be symmetric")
            r, c = np.nonzero(A)
            cons.append(np.full(r.size, j))
            rows.append(r)
            cols.append(c)
            vals.append(A[r, c])
        if cons:
            return cls(n, m, np.concatenate(cons), np.concatenate(rows),
                       np.concatenate(cols), np.concatenate(vals))
        return cls(n, m, [], [], [], [])

    def dense(self, j: int) -> np.ndarray:
        """Constraint ``j`` as a dense matrix."""
        A = np.zeros((self.n, self.n))
        s, e = self.ptr[j], self.ptr[j + 1]
        A[self.row[s:e], self.col[s:e]] = self.val[s:e]
        return A

    def is_onehot(self) -> bool:
        """Every constraint is ``v e_k e_k'`` with distinct ``k``."""
        counts = np.diff(self.ptr)
        return bool(np.all(counts <= 1) and np.all(self.row == self.col))


class Model:
    """An SDP in the form of ``LowRankOpt.Model`` (see module docstring)."""

    def __init__(self, C, A, b, d_lin=None, C_lin=None, sides=None):
        self.C = [np.ascontiguousarray(np.asarray(c, dtype=np.float64)) for c in C]
        self.sides = [int(c.shape[0]) for c in self.C] if sides is None else [int(s) for s in sides]
        self.b = np.asarray(b, dtype=np.float64).copy()
        self.m = int(self.b.size)
        self.d_lin = np.zeros(0) if d_lin is None else np.asarray(d_lin, dtype=np.float64).copy()
        self.ns = int(self.d_lin.size)
        if C_lin is None:
            C_lin = np.zeros((self.m, self.ns))
        # column-major, the layout of the C ABI
        self.C_lin = np.asfortranarray(np.asarray(C_lin, dtype=np.float64).reshape(self.m, self.ns))
        if len(A) != len(self.C):
            raise ValueError("one constraint list per PSD block is required")
        blocks = []
        for n, Ai in zip(self.sides, A):
            if isinstance(Ai, BlockConstraints):
                blocks.append(Ai)
            else:
                blocks.append(BlockConstraints.from_dense_list(n, Ai))
        self.A = blocks
        for i, (n, c) in enumerate(zip(self.sides, self.C)):
            if c.shape != (n, n):
                raise ValueError(f"C[{i}] has the wrong shape")
            if not np.array_equal(c, c.T):
                raise ValueError(f"C[{i}] must be symmetric")
            if self.A[i].m != self.m or self.A[i].n != n:
                raise ValueError(f"A[{i}] has the wrong dimensions")
        if len(self.C) == 0 and self.ns == 0:
            # src/solver.jl:103-105
            raise ValueError("MadSDP: model has no variables.")

    @property
    def nblocks(self) -> int:
        return len(self.C)

    def barrier_dim(self) -> int:
        """nu = sum n_i + n_scalar (src/solver.jl:180-181)."""
        return int(sum(self.sides)) + self.ns

    def copy(self) -> "Model":
        return Model([c.copy() for c in self.C], self.A, self.b.copy(), self.d_lin.copy(),
                     self.C_lin.copy(), list(self.sides))
