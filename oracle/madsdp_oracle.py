"""CPU oracle: a NumPy/SciPy restatement of MadSDP's interior-point methods.

TEST INFRASTRUCTURE ONLY.  This module is the checker for the GPU library:
only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it.  The product path never calls it.

It restates, function by function, the Julia reference (blegat/MadSDP.jl,
paths relative to that project) in float64:

* driver, initial points, Schur regularization, termination: src/solver.jl
* PrimalDual with Mehrotra / AdaptiveMu: src/primal_dual.jl
* NT / HKM directions: src/directions.jl
* residuals, right-hand side, directions, step lengths: src/step.jl
* block helpers (Cholesky with flush, inverse): src/blocks.jl
* DenseCholesky / MadNLPSchur: src/schur_solvers.jl, src/kkt.jl
* QRSchur (dense Householder QR instead of SPQR): src/qr_schur.jl
* DualCentering: src/dual_centering.jl
* component defaults: src/components.jl, options: src/options.jl

The arithmetic of the un-vendored dependency LowRankOpt (compat 0.2.5,
Project.toml:18; the patch version is unpinned, no Manifest is shipped) is
restated from its mathematical definition at MadSDP's call sites:

* ``schur_complement!(model, L, R, H)``: H_jk = sum_i <A_ij, L_i A_ik R_i>
  + sum_s C_lin[j,s] x_s/z_s C_lin[k,s] (src/solver.jl:30-31,117-118,304);
* ``add_jprod!`` / ``unsafe_jtprod``: A(X) and A*(y);
* ``eigen!``: an exact symmetric eigendecomposition (LAPACK syevd);
* ``lanczos_eigmin!``: the exact smallest eigenvalue of L^-1 D L^-T
  (LAPACK syevd on the formed matrix; LowRankOpt's Lanczos iteration count
  and tolerance are not visible, so the per-iteration step lengths of the
  reference are pinned only to the accuracy of its Lanczos).

Parity pin: the known answers of the reference test suite (objective values,
statuses, Newton-system identities, Cholesky flush, identity scale) are
checked in ``tests/test_oracle_known_answers.py``.
"""

from __future__ import annotations

import enum
import math
import time
from dataclasses import dataclass
from typing import Optional

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp

EPS = np.finfo(np.float64).eps


# --- statuses (MadNLP.Status values used by MadSDP, src/moi.jl:16-29) --------

class Status(enum.IntEnum):
    SOLVE_SUCCEEDED = 1
    SOLVED_TO_ACCEPTABLE_LEVEL = 2
    SEARCH_DIRECTION_BECOMES_TOO_SMALL = 3
    MAXIMUM_ITERATIONS_EXCEEDED = 5
    MAXIMUM_WALLTIME_EXCEEDED = 6
    INFEASIBLE_PROBLEM_DETECTED = 8
    ERROR_IN_STEP_COMPUTATION = 11
    USER_REQUESTED_STOP = 13
    INITIAL = 100
    REGULAR = 101


# --- components (src/components.jl) -------------------------------------------

@dataclass(frozen=True)
class NT:
    """Nesterov-Todd direction (src/components.jl:133-139)."""


@dataclass(frozen=True)
class HKM:
    """HKM direction (src/components.jl:141-153)."""


@dataclass(frozen=True)
class EigenStep:
    tau: float = 0.95  # src/components.jl:175-178


@dataclass(frozen=True)
class CholeskyBacktrack:
    shrink: float = 0.8  # src/components.jl:189-193
    boundary: float = 0.95


@dataclass(frozen=True)
class Mehrotra:
    sigma_exponent: float = 3.0  # src/components.jl:212-215


@dataclass(frozen=True)
class AdaptiveMu:
    initial_ratio: float = 0.25  # src/components.jl:231-235
    ratio: float = 0.5


@dataclass(frozen=True)
class PrimalDual:
    direction: object = NT()
    step: object = EigenStep()
    centering: object = Mehrotra()


@dataclass(frozen=True)
class DualCentering:
    beta: float = 0.2  # src/components.jl:100-108
    delta: float = 1.0
    A: Optional[float] = 2.0
    centering_max_iter: int = 50


class ScaledIdentity:
    """src/components.jl:251-260."""

    def __init__(self, scale: Optional[float] = None):
        if scale is not None:
            if not math.isfinite(scale) or scale <= 0:
                raise ValueError("The identity scale must be finite and positive.")
        self.scale = scale


@dataclass
class InitialPoint:
    X: list
    y: np.ndarray
    x: Optional[np.ndarray] = None


@dataclass(frozen=True)
class DualShift:
    initial_shift: float = 1.0  # src/components.jl:271-275
    max_shift: float = 1e10


@dataclass(frozen=True)
class DenseCholesky:
    pass


@dataclass(frozen=True)
class MadNLPSchur:
    """Bunch-Kaufman LDL' of the Schur complement (src/kkt.jl:15-25)."""


@dataclass(frozen=True)
class QRSchur:
    pass


@dataclass
class Options:
    """src/options.jl:3-15."""

    tol: float = 1e-7
    max_iter: int = 100
    max_wall_time: float = 3600.0
    mu_min: float = 1e-14
    regularize_schur: float = 1e-12
    max_schur_reg: int = 8
    datasparsity: int = 8


# --- constraint operators (LowRankOpt callbacks) --------------------------------

class _BlockOp:
    """A(X), A*(y) and the Schur complement of one PSD block."""

    def __init__(self, blk):
        n, m = blk.n, blk.m
        self.n, self.m = n, m
        self.con = np.asarray(blk.con, dtype=np.int64)
        self.row = np.asarray(blk.row, dtype=np.int64)
        self.col = np.asarray(blk.col, dtype=np.int64)
        self.val = np.asarray(blk.val)
        self.nnz = self.val.size
        self.sp = sp.csr_matrix((self.val, (self.con, self.row * n + self.col)), shape=(m, n * n))
        self.spT = self.sp.T.tocsr()
        self.P = sp.csr_matrix((np.ones(self.nnz), (self.con, np.arange(self.nnz))), shape=(m, self.nnz))
        self.ptr = np.asarray(blk.ptr)
        self.dense_threshold = 6000
        self._dense = None

    def jprod(self, X):
        return self.sp @ X.ravel()

    def jtprod(self, y):
        return (self.spT @ y).reshape(self.n, self.n)

    def dense_matrix(self, j):
        A = np.zeros((self.n, self.n))
        s, e = self.ptr[j], self.ptr[j + 1]
        A[self.row[s:e], self.col[s:e]] = self.val[s:e]
        return A

    def schur(self, L, R):
        """H_jk = <A_j, L A_k R>: entry pairs for few entries, batched dense
        products when the constraints are dense, else constraint by
        constraint (three summation orders of the same sum)."""
        if self.nnz <= self.dense_threshold:
            r, c, v = self.row, self.col, self.val
            # K[e, f] = v_e v_f L[r_e, r_f] R[c_f, c_e];  H = P K P'
            K = (v[:, None] * v[None, :]) * L[np.ix_(r, r)] * R[np.ix_(c, c)].T
            return np.asarray(self.P @ np.asarray(self.P @ K.T).T)
        if 2 * self.nnz >= self.m * self.n * self.n:
            return self.schur_dense(L, R)
        return self.schur_columns(L, R)

    def schur_dense(self, L, R):
        """All T_k = L A_k R by batched products, then H = [vec A_j]' [vec T_k]
        as one product: 4 m n^3 + 2 m^2 n^2 flops on dense A_k."""
        if self._dense is None:
            self._dense = self.sp.toarray().reshape(self.m, self.n, self.n)
        T = np.matmul(np.matmul(L, self._dense), R)
        return self._dense.reshape(self.m, -1) @ T.reshape(self.m, -1).T

    def schur_columns(self, L, R):
        """T_k = L A_k R from the entries of A_k, H[:, k] = A(T_k)."""
        H = np.zeros((self.m, self.m))
        for k in range(self.m):
            s, e = self.ptr[k], self.ptr[k + 1]
            if s == e:
                continue
            r, c, v = self.row[s:e], self.col[s:e], self.val[s:e]
            T = (L[:, r] * v) @ R[c, :]
            H[:, k] = self.sp @ T.ravel()
        return H


def _sym(A):
    """A = (A + A')/2 (src/blocks.jl:77-84)."""
    return (A + A.T) / 2


def _cholesky_factor(M):
    """Lower Cholesky factor of sym(M) with the flush of tiny entries, or None.

    src/blocks.jl:94-113: entries below eps^2 * max |L_ii| are set to zero.
    """
    A = _sym(M)
    if not np.all(np.isfinite(A)):
        return None
    Lm, info = sla.lapack.dpotrf(A, lower=1, clean=1)
    if info != 0:
        return None
    tol = EPS ** 2 * (np.max(np.abs(np.diag(Lm))) if Lm.shape[0] else 0.0)
    Lm = np.tril(Lm)
    Lm[np.abs(Lm) < tol] = 0.0
    return Lm


def _inverse_from_cholesky(Lm):
    """S^-1 from the Cholesky factor (LAPACK potri, src/blocks.jl:116-123)."""
    inv, info = sla.lapack.dpotri(Lm, lower=1)
    inv = np.tril(inv)
    return inv + np.tril(inv, -1).T


def _is_posdef(A):
    """LAPACK potrf on the lower triangle succeeds (src/blocks.jl:133-137)."""
    if not np.all(np.isfinite(A)):
        return False
    _, info = sla.lapack.dpotrf(A, lower=1, clean=0)
    return info == 0


def _max_scalar_step(x, dx):
    """Largest alpha with x + alpha dx >= 0 (src/step.jl:137-146)."""
    neg = dx < 0
    if not np.any(neg):
        return math.inf
    return float(np.min(-x[neg] / dx[neg]))


def eigmin_congruence(Lm, D):
    """Smallest eigenvalue of L^-1 D L^-T (Symmetric(D, :U), src/step.jl:150-163)."""
    Du = np.triu(D) + np.triu(D, 1).T
    T1 = sla.solve_triangular(Lm, Du, lower=True)
    Z = sla.solve_triangular(Lm, T1.T, lower=True)
    Z = _sym(Z)
    return float(np.linalg.eigvalsh(Z)[0]) if Z.shape[0] else math.inf


def _eigen_step(Lm, D, tau):
    """src/step.jl:178-183."""
    lam = eigmin_congruence(Lm, D)
    return 1.0 if lam > -math.sqrt(EPS) else min(1.0, -tau / lam)


# --- per-block state (src/blocks.jl:10-63, src/directions.jl:151-178) --------

class Block:
    def __init__(self, n):
        z = lambda: np.zeros((n, n))
        self.n = n
        self.X, self.S, self.Rd, self.Ls, self.Si = z(), z(), z(), z(), z()
        self.buf, self.buf2 = z(), z()
        # PrimalDualBlock
        self.delX, self.delS, self.Lx, self.corr = z(), z(), z(), z()
        # NT workspace
        self.W, self.G, self.Gi, self.Lx_nt, self.RNT = z(), z(), z(), z(), z()
        self.D = np.zeros(n)
        # DualCentering workspace
        self.Shat, self.Dc = z(), z()
        self.eigvals = np.zeros(n)


class Solver:
    """MadSDPSolver (src/solver.jl:7-160) restated."""

    def __init__(self, model, algorithm=None, direction=None, step=None, centering=None,
                 initial_point=None, schur=None, precision=None, **options):
        direction = NT() if direction is None else direction
        step = EigenStep() if step is None else step
        centering = Mehrotra() if centering is None else centering
        if algorithm is None:
            algorithm = PrimalDual(direction, step, centering)
        if initial_point is None:
            initial_point = DualShift() if isinstance(algorithm, DualCentering) else ScaledIdentity()
        schur = DenseCholesky() if schur is None else schur
        self.opt = Options(**options)
        self.model = model
        self.algorithm = algorithm
        self.initial_point = initial_point
        self.schur = schur
        self.nblocks = model.nblocks
        self.n_scalar = model.ns
        if self.nblocks == 0 and self.n_scalar == 0:
            raise ValueError("MadSDP: model has no variables.")
        # check_model (src/dual_centering.jl:68-76)
        if isinstance(algorithm, DualCentering):
            if self.n_scalar > 0:
                raise RuntimeError("MadSDP: `DualCentering` does not support scalar (LP) blocks yet.")
            if self.nblocks == 0:
                raise RuntimeError("MadSDP: `DualCentering` needs at least one PSD block.")
        # check_schur (src/qr_schur.jl:12-22)
        if isinstance(schur, QRSchur):
            if not (isinstance(algorithm, PrimalDual) and isinstance(algorithm.direction, NT)):
                raise ValueError("QRSchur requires PrimalDual with the NT direction.")
            if precision not in (None, np.float64):
                raise ValueError("QRSchur requires Float64 data.")
        self.ops = [_BlockOp(a) for a in model.A]
        self.blocks = [Block(n) for n in model.sides]
        m, ns = model.m, model.ns
        self.m = m
        self.y, self.dely, self.Rp = np.zeros(m), np.zeros(m), np.zeros(m)
        self.x, self.z = np.zeros(ns), np.zeros(ns)
        self.delx, self.delz = np.zeros(ns), np.zeros(ns)
        self.Rd_lin, self.zinv, self.corr_lin = np.zeros(ns), np.zeros(ns), np.zeros(ns)
        self.rd_nonzero = [True] * self.nblocks
        # cnorm: ||C_i||_inf as the max-abs entry (src/solver.jl:119-120)
        self.cnorm = [float(np.max(np.abs(c))) if c.size else 0.0 for c in model.C]
        self.H = np.zeros((m, m))
        self.F = None  # factorization of H
        self.mu = self.sigma = self.alpha = self.beta = 0.0
        self.inf_pr = self.inf_du = self.inf_compl = self.obj_val = 0.0
        self.iter = 0
        self.status = Status.INITIAL
        self.start_time = time.time()
        self.trajectory = []
        # DualCentering state (src/dual_centering.jl:12-41)
        self.dc_d, self.dc_g = np.zeros(m), np.zeros(m)
        self.dc_grad_zeta, self.dc_dy, self.dc_yhat = np.zeros(m), np.zeros(m), np.zeros(m)
        self.dc_nu, self.dc_A, self.dc_t, self.dc_lam = 0, 0.0, 0.0, 0.0
        self.n_predictor = self.n_newton = 0
        # QRSchur workspace
        self.qr_scale = np.ones(m)

    # --- model helpers -------------------------------------------------------
    def barrier_dim(self):
        return sum(b.n for b in self.blocks) + self.n_scalar

    def primal_objective(self):
        """src/solver.jl:164-174."""
        s = 0.0
        for c, b in zip(self.model.C, self.blocks):
            s += float(np.sum(c * b.X))
        if self.n_scalar > 0:
            s += float(self.model.d_lin @ self.x)
        return s

    def dual_objective(self):
        return float(self.model.b @ self.y)

    def total_complementarity(self):
        """src/solver.jl:183-190."""
        s = sum(float(np.sum(b.X * b.S)) for b in self.blocks)
        if self.n_scalar > 0:
            s += float(self.x @ self.z)
        return s

    def _slack(self, i, y):
        """S_i = sym(C_i - A_i*(y)) (src/solver.jl:192-198)."""
        return _sym(self.model.C[i] - self.ops[i].jtprod(y))

    def set_dual_slacks(self):
        """src/solver.jl:200-211."""
        for i, b in enumerate(self.blocks):
            b.S = self._slack(i, self.y)
        if self.n_scalar > 0:
            self.z = self.model.d_lin - self.model.C_lin.T @ self.y

    # --- initial points (src/solver.jl:213-284) ------------------------------
    def initial_point_(self, p):
        if isinstance(p, ScaledIdentity):
            bscale = float(np.max(np.abs(self.model.b))) if self.m else 0.0
            cscale = max(self.cnorm) if self.cnorm else 0.0
            if self.n_scalar > 0:
                cscale = max(cscale, float(np.max(np.abs(self.model.d_lin))))
            if p.scale is None:
                beta = max(10.0, math.sqrt(max(bscale, 1.0) * max(cscale, 1.0)) * math.sqrt(self.barrier_dim()))
            else:
                beta = float(p.scale)
            for b in self.blocks:
                b.X = beta * np.eye(b.n)
                b.S = beta * np.eye(b.n)
            self.y[:] = 0.0
            self.x[:] = beta
            self.z[:] = beta
        elif isinstance(p, InitialPoint):
            self.y = np.array(p.y, dtype=np.float64).copy()
            for b, X in zip(self.blocks, p.X):
                b.X = np.array(X, dtype=np.float64).copy()
            self.x = np.ones(self.n_scalar) if p.x is None else np.array(p.x, dtype=np.float64).copy()
            self.set_dual_slacks()
        elif isinstance(p, DualShift):
            for b in self.blocks:
                b.X = np.eye(b.n)
            self.x = np.ones(self.n_scalar)
            rho = 0.0
            while rho <= p.max_shift:
                self.y = np.full(self.m, -rho)
                self.set_dual_slacks()
                if self._dual_interior():
                    if rho != 0.0:
                        self.y = np.full(self.m, -2 * rho)
                        self.set_dual_slacks()
                    return
                rho = p.initial_shift if rho == 0.0 else 2 * rho
            raise RuntimeError(
                f"MadSDP: could not find a dual interior point `y = -ρ 1` with ρ ≤ {p.max_shift}; "
                "use `InitialPoint` to give one.")
        else:
            raise TypeError("unknown initial point")

    def _dual_interior(self):
        """src/solver.jl:254-258."""
        for b in self.blocks:
            Lm = _cholesky_factor(b.S)
            if Lm is None:
                return False
            b.Ls = Lm
        return bool(np.all(self.z > 0))

    # --- driver (src/solver.jl:286-396) ---------------------------------------
    def initialize(self):
        self.initial_point_(self.initial_point)
        self.iter = 0
        self.status = Status.REGULAR
        self.start_time = time.time()
        if isinstance(self.algorithm, DualCentering):
            self._dc_initialize()
        else:
            self.update_residuals()
            self._initialize_centering(self.algorithm.centering)

    def _initialize_centering(self, c):
        """src/primal_dual.jl:10-19."""
        mu = self.total_complementarity() / max(self.barrier_dim(), 1)
        self.mu = c.initial_ratio * mu if isinstance(c, AdaptiveMu) else mu

    def schur_scaling(self, b):
        """(L, R) of <A_j, L A_k R> (src/directions.jl:212,247; src/dual_centering.jl:66)."""
        if isinstance(self.algorithm, DualCentering):
            return b.Si, b.Si
        if isinstance(self.algorithm.direction, NT):
            return b.W, b.W
        return b.Si, b.X

    def schur_complement(self):
        """LowRankOpt.schur_complement!(model, L, R, H)."""
        H = np.zeros((self.m, self.m))
        for i, b in enumerate(self.blocks):
            L, R = self.schur_scaling(b)
            H += self.ops[i].schur(L, R)
        if self.n_scalar > 0:
            w = self.x * self.zinv
            H += (self.model.C_lin * w) @ self.model.C_lin.T
        return H

    def factorize(self, H):
        """DenseCholesky / MadNLPSchur factorize! (src/schur_solvers.jl:15-19,27-37)."""
        if isinstance(self.schur, MadNLPSchur):
            lu, piv, info = sla.lapack.dsytrf(np.tril(H) + np.tril(H, -1).T, lower=1)
            if info != 0:
                return False
            self.F = ("ldl", lu, piv)
            return True
        Lm, info = sla.lapack.dpotrf(H, lower=1, clean=1)
        if info != 0:
            return False
        self.F = ("chol", Lm)
        return True

    def schur_solve(self, rhs):
        """src/schur_solvers.jl:21 and src/kkt.jl:27-32."""
        if self.F[0] == "ldl":
            x, info = sla.lapack.dsytrs(self.F[1], self.F[2], rhs, lower=1)
            return x
        Lm = self.F[1]
        t = sla.solve_triangular(Lm, rhs, lower=True)
        return sla.solve_triangular(Lm, t, lower=True, trans="T")

    def factorize_schur(self):
        """Regularization retry loop (src/solver.jl:299-314)."""
        if isinstance(self.schur, QRSchur):
            return self._qr_factorize()
        reg = self.opt.regularize_schur
        for _ in range(self.opt.max_schur_reg):
            H = self.schur_complement()
            if reg > 0:
                H[np.diag_indices_from(H)] += reg
            self.H = H
            if self.factorize(H):
                return True
            reg = 1e-12 if reg == 0 else 10 * reg
        return False

    def update_infeasibilities(self):
        """src/solver.jl:318-334."""
        bn = float(np.max(np.abs(self.model.b))) if self.m else 0.0
        self.inf_pr = (float(np.max(np.abs(self.Rp))) if self.m else 0.0) / max(1.0, bn)
        rd = 0.0
        for b in self.blocks:
            if b.n:
                rd = max(rd, float(np.max(np.abs(b.Rd))))
        cn = max(self.cnorm) if self.cnorm else 0.0
        if self.n_scalar > 0:
            rd = max(rd, float(np.max(np.abs(self.Rd_lin))))
            cn = max(cn, float(np.max(np.abs(self.model.d_lin))))
        self.inf_du = rd / max(1.0, cn)

    def update_status(self, converged):
        """src/solver.jl:336-347."""
        if converged:
            self.status = Status.SOLVE_SUCCEEDED
        elif self.iter >= self.opt.max_iter:
            self.status = Status.MAXIMUM_ITERATIONS_EXCEEDED
        elif time.time() - self.start_time >= self.opt.max_wall_time:
            self.status = Status.MAXIMUM_WALLTIME_EXCEEDED

    def update_termination(self):
        if isinstance(self.algorithm, DualCentering):
            return self._dc_update_termination()
        # src/primal_dual.jl:123-134
        pobj = self.primal_objective()
        dobj = self.dual_objective()
        self.obj_val = pobj
        self.update_infeasibilities()
        self.inf_compl = abs(pobj - dobj) / max(1.0, abs(pobj) + abs(dobj))
        converged = max(self.inf_pr, self.inf_du, self.inf_compl) <= self.opt.tol
        self.update_status(converged)
        if self.status == Status.REGULAR and self.mu < self.opt.mu_min:
            self.status = Status.SEARCH_DIRECTION_BECOMES_TOO_SMALL
        self._record(pobj, dobj)

    def _record(self, pobj, dobj):
        self.trajectory.append(dict(iter=self.iter, pobj=pobj, dobj=dobj, inf_pr=self.inf_pr,
                                    inf_du=self.inf_du, gap=self.inf_compl, mu=self.mu,
                                    alpha=self.alpha, beta=self.beta))

    def iterate(self):
        if isinstance(self.algorithm, DualCentering):
            return self._dc_iterate()
        if isinstance(self.algorithm.centering, Mehrotra):
            return self._iterate_mehrotra(self.algorithm.centering)
        return self._iterate_adaptive(self.algorithm.centering)

    def solve(self, verbose=False):
        """src/solver.jl:385-396."""
        self.initialize()
        self.update_termination()
        while self.status == Status.REGULAR:
            self.iterate()
            if self.status != Status.REGULAR:
                break
            self.update_termination()
        return self

    # --- residuals, rhs, directions (src/step.jl) -----------------------------
    def update_residuals(self):
        """src/step.jl:12-47."""
        Rp = np.zeros(self.m)
        for i, b in enumerate(self.blocks):
            Rp += self.ops[i].jprod(b.X)
        if self.n_scalar > 0:
            Rp += self.model.C_lin @ self.x
        self.Rp = self.model.b - Rp
        for i, b in enumerate(self.blocks):
            ATy = self.ops[i].jtprod(self.y)
            b.Rd = self.model.C[i] - b.S - ATy
            threshold = 100 * EPS * max(1.0, self.cnorm[i])
            self.rd_nonzero[i] = (float(np.max(np.abs(b.Rd))) if b.n else 0.0) > threshold
        if self.n_scalar > 0:
            self.Rd_lin = self.model.d_lin - self.z - self.model.C_lin.T @ self.y

    def apply_E(self, b, M):
        """NT: W M W; HKM: sym(X M S^-1) (src/directions.jl:80-84,116-120)."""
        if isinstance(self.algorithm.direction, NT):
            return _sym(b.W @ M @ b.W)
        return _sym(b.X @ M @ b.Si)

    def rhs(self, mu, corrected):
        """src/step.jl:63-89."""
        h = self.Rp.copy()
        for i, b in enumerate(self.blocks):
            buf = b.X - mu * b.Si
            if self.rd_nonzero[i]:
                buf = buf + self.apply_E(b, b.Rd)
            if corrected:
                buf = buf - b.corr
            h += self.ops[i].jprod(buf)
        if self.n_scalar > 0:
            v = self.x - mu * self.zinv + self.x * self.zinv * self.Rd_lin
            if corrected:
                v = v - self.corr_lin
            h += self.model.C_lin @ v
        return h

    def directions(self, dely, mu, corrected):
        """src/step.jl:94-124."""
        for i, b in enumerate(self.blocks):
            ATdy = self.ops[i].jtprod(dely)
            b.delS = _sym(b.Rd - ATdy)
            b.delX = mu * b.Si - b.X + self.apply_E(b, ATdy)
            if self.rd_nonzero[i]:
                b.delX = b.delX - self.apply_E(b, b.Rd)
            if corrected:
                b.delX = b.delX + b.corr
            b.delX = _sym(b.delX)
        if self.n_scalar > 0:
            self.delz = self.Rd_lin - self.model.C_lin.T @ dely
            self.delx = mu * self.zinv - self.x - self.x * self.zinv * self.delz
            if corrected:
                self.delx = self.delx + self.corr_lin

    def correction(self):
        """src/step.jl:128-136 with src/directions.jl:90-100,123-127."""
        for b in self.blocks:
            if isinstance(self.algorithm.direction, NT):
                tmp = b.Gi @ b.delX
                RNT = tmp @ b.delS
                M = RNT @ b.G
                RNT = -(M + M.T) / (b.D[:, None] + b.D[None, :])
                b.RNT = RNT
                b.corr = _sym(b.G @ RNT @ b.G.T)
            else:
                b.corr = _sym(-(b.delX @ b.delS) @ b.Si)
        if self.n_scalar > 0:
            self.corr_lin = -self.delx * self.delz * self.zinv

    def solve_directions(self, mu, corrected):
        """src/primal_dual.jl:40-54 (or src/qr_schur.jl:90-160)."""
        if isinstance(self.schur, QRSchur):
            return self._qr_solve_directions(mu, corrected)
        h = self.rhs(mu, corrected)
        self.dely = self.schur_solve(h)
        self.directions(self.dely, mu, corrected)

    # --- step lengths (src/step.jl:148-228) ------------------------------------
    def step_lengths(self):
        s = self.algorithm.step
        if isinstance(s, EigenStep):
            a = bt = 1.0
            for b in self.blocks:
                a = min(a, _eigen_step(b.Lx, b.delX, s.tau))
                bt = min(bt, _eigen_step(b.Ls, b.delS, s.tau))
            if self.n_scalar > 0:
                a = min(a, s.tau * _max_scalar_step(self.x, self.delx))
                bt = min(bt, s.tau * _max_scalar_step(self.z, self.delz))
            return a, bt
        a = self._backtrack(s, [b.X for b in self.blocks], [b.delX for b in self.blocks], self.x, self.delx)
        bt = self._backtrack(s, [b.S for b in self.blocks], [b.delS for b in self.blocks], self.z, self.delz)
        return a, bt

    @staticmethod
    def _backtrack(s, Xs, dXs, x, dx):
        """src/step.jl:202-221."""
        a = 1.0
        for X, dX in zip(Xs, dXs):
            while not _is_posdef(X + a * dX):
                a *= s.shrink
                if a < EPS:
                    return 0.0
        if a != 1.0:
            a *= s.boundary
        if x.size:
            a = min(a, s.boundary * _max_scalar_step(x, dx))
        return a

    def affine_complementarity(self, a, bt):
        """src/step.jl:231-243."""
        s = 0.0
        for b in self.blocks:
            s += float(np.sum(b.X * b.S))
            s += bt * float(np.sum(b.X * b.delS))
            s += a * float(np.sum(b.delX * b.S))
            s += a * bt * float(np.sum(b.delX * b.delS))
        for k in range(self.n_scalar):
            s += (self.x[k] + a * self.delx[k]) * (self.z[k] + bt * self.delz[k])
        return s / max(self.barrier_dim(), 1)

    # --- PrimalDual (src/primal_dual.jl) ---------------------------------------
    def prepare_direction(self, b):
        """NT scaling (src/directions.jl:45-75)."""
        if not isinstance(self.algorithm.direction, NT):
            return True
        Lx = _cholesky_factor(b.X)
        if Lx is None:
            return False
        b.Lx_nt = Lx
        M = b.Ls.T @ Lx
        N = _sym(M.T @ M)
        lam, V = np.linalg.eigh(N)
        if not np.all(lam > 0):
            return False
        b.D = np.sqrt(lam)
        sc = np.sqrt(b.D)
        b.G = (Lx @ V) / sc[None, :]
        Gi = V.T * sc[:, None]
        b.Gi = sla.solve_triangular(Lx, Gi.T, lower=True, trans="T").T if b.n else Gi
        b.W = _sym(b.G @ b.G.T)
        return True

    def prepare(self):
        """src/primal_dual.jl:29-37."""
        for b in self.blocks:
            Ls = _cholesky_factor(b.S)
            if Ls is None:
                return False
            b.Ls = Ls
            b.Si = _inverse_from_cholesky(Ls)
            if not self.prepare_direction(b):
                return False
            if isinstance(self.algorithm.step, EigenStep):
                Lx = _cholesky_factor(b.X)
                if Lx is None:
                    return False
                b.Lx = Lx
        if self.n_scalar > 0:
            self.zinv = 1.0 / self.z
        return True

    def _start_iteration(self):
        if not self.prepare() or not self.factorize_schur():
            self.status = Status.ERROR_IN_STEP_COMPUTATION
            return False
        return True

    def take_step(self, a, bt):
        """src/primal_dual.jl:56-72."""
        self.alpha, self.beta = a, bt
        for b in self.blocks:
            b.X = _sym(b.X + a * b.delX)
            b.S = _sym(b.S + bt * b.delS)
        self.y = self.y + bt * self.dely
        if self.n_scalar > 0:
            self.x = self.x + a * self.delx
            self.z = self.z + bt * self.delz
        self.iter += 1
        self.update_residuals()

    def _iterate_mehrotra(self, c):
        """src/primal_dual.jl:85-101."""
        if not self._start_iteration():
            return
        mu = self.total_complementarity() / max(self.barrier_dim(), 1)
        self.mu = mu
        self.solve_directions(0.0, False)
        a_aff, b_aff = self.step_lengths()
        mu_aff = self.affine_complementarity(a_aff, b_aff)
        sigma = min(max((mu_aff / max(mu, EPS)) ** c.sigma_exponent, 1e-8), 1.0)
        self.sigma = sigma
        self.correction()
        self.solve_directions(sigma * mu, True)
        a, bt = self.step_lengths()
        self.take_step(a, bt)

    def _iterate_adaptive(self, c):
        """src/primal_dual.jl:104-121."""
        if not self._start_iteration():
            return
        self.solve_directions(self.mu, False)
        a, bt = self.step_lengths()
        self.take_step(a, bt)
        mu = c.ratio * self.total_complementarity() / max(self.barrier_dim(), 1)
        if min(a, bt) < 0.5:
            mu *= 1.5
        if a + bt > 1.6:
            mu *= 0.75
        if a + bt > 1.9:
            mu /= 1 + 0.1 * self.iter
        self.mu = mu

    # --- QRSchur (src/qr_schur.jl) ----------------------------------------------
    def _qr_factorize(self):
        """Columns svec(G' A_j G) (+ sqrt(x/z) C_lin), equilibration, QR (src/qr_schur.jl:24-88)."""
        rows = []
        for i, b in enumerate(self.blocks):
            n = b.n
            iu = np.triu_indices(n)  # column-major upper triangle == numpy's (row<=col) ordering by col
            order = np.lexsort((iu[0], iu[1]))
            r_idx, c_idx = iu[0][order], iu[1][order]
            w = np.where(r_idx == c_idx, 1.0, math.sqrt(2.0))
            Bi = np.zeros((n * (n + 1) // 2, self.m))
            op = self.ops[i]
            for j in range(self.m):
                if op.ptr[j] == op.ptr[j + 1]:
                    continue
                A = op.dense_matrix(j)
                T = b.G.T @ (A @ b.G)
                Bi[:, j] = T[r_idx, c_idx] * w
            rows.append(Bi)
        if self.n_scalar > 0:
            weight = np.sqrt(self.x / self.z)
            rows.append((self.model.C_lin * weight[None, :]).T)
        B = np.vstack(rows) if rows else np.zeros((0, self.m))
        for j in range(self.m):
            mag = float(np.linalg.norm(B[:, j]))
            if mag == 0.0 or not math.isfinite(mag):
                return False
            self.qr_scale[j] = 1.0 / mag
        B = B * self.qr_scale[None, :]
        if B.shape[0] < self.m:
            return False
        Q, R = np.linalg.qr(B, mode="reduced")
        self.qr_Q, self.qr_R = Q, R
        return bool(np.all(np.diag(R) != 0.0))

    def _qr_solve_directions(self, mu, corrected):
        """Projection solve (src/qr_schur.jl:90-160)."""
        parts = []
        for b in self.blocks:
            n = b.n
            T = -(b.G.T @ (b.Rd @ b.G))
            T[np.diag_indices(n)] += mu / b.D - b.D
            if corrected:
                T = T + b.RNT
            iu = np.triu_indices(n)
            order = np.lexsort((iu[0], iu[1]))
            r_idx, c_idx = iu[0][order], iu[1][order]
            parts.append(np.where(r_idx == c_idx, 1.0, math.sqrt(2.0)) * T[r_idx, c_idx])
        if self.n_scalar > 0:
            weight = np.sqrt(self.x / self.z)
            product = np.sqrt(self.x * self.z)
            v = mu / product - product - weight * self.Rd_lin
            if corrected:
                v = v + self.corr_lin / weight
            parts.append(v)
        base = np.concatenate(parts) if parts else np.zeros(0)
        Q, R = self.qr_Q, self.qr_R
        qb = Q.T @ base
        c = sla.solve_triangular(R, self.qr_scale * self.Rp, trans="T")
        t = c - qb
        self.dely = self.qr_scale * sla.solve_triangular(R, t)
        direction = base + Q @ t
        off = 0
        for i, b in enumerate(self.blocks):
            n = b.n
            k = n * (n + 1) // 2
            seg = direction[off:off + k]
            iu = np.triu_indices(n)
            order = np.lexsort((iu[0], iu[1]))
            r_idx, c_idx = iu[0][order], iu[1][order]
            Mt = np.zeros((n, n))
            vals = np.where(r_idx == c_idx, seg, seg / math.sqrt(2.0))
            Mt[r_idx, c_idx] = vals
            Mt[c_idx, r_idx] = vals
            b.delX = _sym(b.G @ Mt @ b.G.T)
            b.delS = _sym(b.Rd - self.ops[i].jtprod(self.dely))
            off += k
        if self.n_scalar > 0:
            self.delz = self.Rd_lin - self.model.C_lin.T @ self.dely
            self.delx = np.sqrt(self.x / self.z) * direction[off:off + self.n_scalar]

    # --- DualCentering (src/dual_centering.jl) ---------------------------------
    def _refresh_slacks(self):
        """src/dual_centering.jl:83-86."""
        self.set_dual_slacks()
        for b in self.blocks:
            Ls = _cholesky_factor(b.S)
            if Ls is None:
                return False
            b.Ls = Ls
            b.Si = _inverse_from_cholesky(Ls)
        return True

    def _compute_gradient(self):
        """src/dual_centering.jl:89-98."""
        g = np.zeros(self.m)
        for i, b in enumerate(self.blocks):
            g += self.ops[i].jprod(b.Si)
        self.dc_grad_zeta = g
        self.dc_g = g - self.dc_t * self.model.b

    def _newton_direction(self):
        """src/dual_centering.jl:102-110."""
        self._compute_gradient()
        if not self.factorize_schur():
            return False
        self.dc_d = self.schur_solve(self.dc_g.copy())
        self.dc_lam = math.sqrt(max(float(self.dc_g @ self.dc_d), 0.0))
        return True

    def _dc_initialize(self):
        """src/dual_centering.jl:112-143."""
        a = self.algorithm
        self.dc_nu = sum(b.n for b in self.blocks)
        if a.A is None:
            tau = 2 * a.beta / (1 - a.beta) ** 2
            self.dc_A = a.delta + (-tau - math.log1p(-tau))
        else:
            self.dc_A = float(a.A)
        self.n_predictor = self.n_newton = 0
        if not self._refresh_slacks():
            raise RuntimeError("MadSDP: the initial `y` does not give a dual slack `S ≻ 0`.")
        self.dc_t = 0.0
        if not self._newton_direction():
            raise RuntimeError("MadSDP: failed to factorize ∇²ζ at y₀.")
        bvec = self.model.b
        self.dc_dy = self.schur_solve(bvec.copy())
        bBb = max(float(bvec @ self.dc_dy), EPS)
        bBg = float(bvec @ self.dc_d)
        self.dc_t = max(bBg / bBb, a.beta / math.sqrt(bBb))
        for _ in range(a.centering_max_iter):
            if not self._newton_direction():
                raise RuntimeError("MadSDP: failed to factorize ∇²ζ during the initial centering.")
            if self.dc_lam <= a.beta / 2:
                break
            self.y = self.y - self.dc_d / (1 + self.dc_lam)
            self.iter += 1
            self.n_newton += 1
            if not self._refresh_slacks():
                raise RuntimeError("MadSDP: damped Newton left the interior during the initial centering.")
        self.mu = 1.0 / self.dc_t

    def _xi_value(self, alpha):
        """src/dual_centering.jl:146-160."""
        s = 0.0
        b2 = alpha / (1 - alpha)
        for b in self.blocks:
            for mu in b.eigvals:
                u = 1 - alpha * mu
                v = 1 + b2 * mu
                if not (u > 0 and v > 0):
                    return math.inf
                s -= math.log(u)
                s -= math.log(v)
        return s

    def _xi_alpha_max(self):
        """src/dual_centering.jl:163-177."""
        amax = 1.0
        for b in self.blocks:
            for mu in b.eigvals:
                if mu > 0:
                    amax = min(amax, 1.0 / mu)
                if mu < 0:
                    amax = min(amax, 1.0 / (1 - mu))
        return amax

    def _solve_alpha(self, A):
        """Bisection on xi(alpha) = A (src/dual_centering.jl:181-201)."""
        amax = self._xi_alpha_max()
        hi = amax * 0.99999
        xhi = self._xi_value(hi)
        if not math.isfinite(xhi) or xhi < A:
            return hi
        lo = 0.0
        for _ in range(80):
            mid = (lo + hi) / 2
            if self._xi_value(mid) < A:
                lo = mid
            else:
                hi = mid
            if hi - lo <= EPS * max(1.0, hi):
                break
        return (lo + hi) / 2

    def _predictor_step(self):
        """src/dual_centering.jl:232-264."""
        self.dc_yhat = self.y + self.dc_d
        self.dc_dy = self.dc_t * self.schur_solve(self.model.b.copy())
        for i, b in enumerate(self.blocks):
            b.Shat = self._slack(i, self.dc_yhat)
            b.Dc = _sym(self.ops[i].jtprod(self.dc_dy))
            Lh = _cholesky_factor(b.Shat)
            if Lh is None:
                return False
            T1 = sla.solve_triangular(Lh, b.Dc, lower=True)
            Z = _sym(sla.solve_triangular(Lh, T1.T, lower=True).T)
            b.eigvals = np.linalg.eigvalsh(Z)
        shat_n2 = 0.0
        for b in self.blocks:
            T1 = sla.solve_triangular(b.Ls, b.Shat, lower=True)
            Z = sla.solve_triangular(b.Ls, T1.T, lower=True).T
            shat_n2 += float(np.sum(Z * Z))
        alpha = self._solve_alpha(self.dc_A)
        self.alpha = self.beta = alpha
        for b in self.blocks:
            buf = (1 - alpha) * b.Shat + alpha * b.Dc
            b.X = _sym((b.Si @ buf) @ b.Si / self.dc_t)
        self.y = self.dc_yhat + alpha * self.dc_dy
        self.dc_t = self.dc_nu * self.dc_t / ((1 - alpha) * shat_n2)
        self.n_predictor += 1
        return True

    def _dc_iterate(self):
        """src/dual_centering.jl:266-289."""
        a = self.algorithm
        if not self._newton_direction():
            self.status = Status.ERROR_IN_STEP_COMPUTATION
            return
        if self.dc_lam > a.beta:
            self.y = self.y - self.dc_d / (1 + self.dc_lam)
            self.alpha = self.beta = 1.0 / (1 + self.dc_lam)
            self.n_newton += 1
        elif not self._predictor_step():
            self.status = Status.ERROR_IN_STEP_COMPUTATION
            return
        self.iter += 1
        if not self._refresh_slacks():
            self.status = Status.ERROR_IN_STEP_COMPUTATION
            return
        self.mu = 1.0 / self.dc_t

    def _dc_update_termination(self):
        """src/dual_centering.jl:293-303."""
        pobj = self.primal_objective()
        dobj = self.dual_objective()
        self.obj_val = pobj
        self.update_residuals()
        self.update_infeasibilities()
        self.inf_compl = self.dc_nu / max(self.dc_t, EPS) / max(1.0, abs(pobj) + abs(dobj))
        self.update_status(self.inf_compl <= self.opt.tol)
        self._record(pobj, dobj)


def madsdp(model, **kwargs):
    """src/solver.jl:404."""
    return Solver(model, **kwargs).solve()
