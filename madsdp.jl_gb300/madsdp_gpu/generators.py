"""Seeded synthetic instances with the shapes of the benchmark workloads.

The reference benchmarks random max-cut instances built with Julia's
``MersenneTwister``/``sprand`` (benchmark/maxcut.jl:17-40); that stream
cannot be reproduced without Julia, so these generators draw instances of
the same shape and distribution from ``numpy.random.default_rng(seed)``.

Workloads:

* ``maxcut``: min <-L/4, X> s.t. X_jj = 1, X PSD; one-hot constraints
  (benchmark/maxcut.jl:28-40).
* ``sos_hankel``: lower bound of a univariate polynomial by a Gram block of
  side d+1 and 2d+1 Hankel 0/1 constraints.
* ``dense_random``: dense symmetric constraint matrices on several PSD blocks
  plus nonnegative scalars, feasible by construction.
* the small problems of the reference test suite (test/runtests.jl,
  test/qr_schur.jl, test/dual_runtests.jl).
"""

from __future__ import annotations

import numpy as np

from .model import BlockConstraints, Model

__all__ = [
    "maxcut",
    "maxcut_from_weights",
    "sos_hankel",
    "sos_hankel_moment",
    "dense_random",
    "onehot_constraints",
    "hankel_constraints",
    "mixed_lp_example",
    "trivial_2x2",
    "trace_one",
    "qr_example",
    "weighted_4node_W",
    "cycle4_W",
]


def onehot_constraints(n: int) -> BlockConstraints:
    """A_j = e_j e_j' for j = 1..n (the diag(X) = 1 constraints of max-cut)."""
    idx = np.arange(n)
    return BlockConstraints(n, n, idx, idx, idx, np.ones(n))


def hankel_constraints(n: int) -> BlockConstraints:
    """A_k = sum_{a+b=k} E_ab for k = 0..2(n-1): 2n-1 constraints."""
    a, b = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a, b = a.ravel(), b.ravel()
    return BlockConstraints(n, 2 * n - 1, a + b, a, b, np.ones(a.size))


def maxcut_from_weights(W) -> Model:
    """min <-L/4, X> s.t. diag(X) = 1 for the weighted graph W."""
    W = np.asarray(W, dtype=np.float64)
    n = W.shape[0]
    L = np.diag(W.sum(axis=1)) - W
    return Model([-L / 4.0], [onehot_constraints(n)], np.ones(n))


def maxcut(n: int, p: float, weights: str = "unit", seed: int = 0) -> Model:
    """Erdos-Renyi max-cut relaxation; ``weights`` is 'unit' or 'pm1'."""
    rng = np.random.default_rng(seed)
    upper = np.triu(rng.random((n, n)) < p, 1)
    W = upper.astype(np.float64)
    if weights == "pm1":
        W *= rng.choice(np.array([-1.0, 1.0]), size=(n, n))
    elif weights != "unit":
        raise ValueError("weights must be 'unit' or 'pm1'")
    W = W + W.T
    return maxcut_from_weights(W)


def _sos_coefficients(d: int, rng) -> np.ndarray:
    """Coefficients p_0..p_2d of sum_{r=1..3} q_r(x)^2 + 0.1 sum_k x^(2k)."""
    p = np.zeros(2 * d + 1)
    for _ in range(3):
        q = rng.standard_normal(d + 1)
        p += np.convolve(q, q)
    p[0::2] += 0.1
    return p


def sos_hankel(d: int, seed: int = 0) -> Model:
    """max gamma s.t. p - gamma = v'Qv, Q PSD (v = [1, x, .., x^d]).

    The Gram matrix Q is the PSD block (side n = d+1) with the m = 2d+1
    Hankel constraints <A_k, Q> + [k = 0] gamma = p_k.  MadSDP's cones are
    the PSD cone and the nonnegative orthant only (src/solver.jl:17-20), so
    the free gamma is split as gamma+ - gamma- (ns = 2, objective
    min -gamma+ + gamma-).  The optimal value of the model is -gamma*.
    """
    rng = np.random.default_rng(seed)
    n = d + 1
    p = _sos_coefficients(d, rng)
    m = 2 * d + 1
    C_lin = np.zeros((m, 2))
    C_lin[0, 0], C_lin[0, 1] = 1.0, -1.0
    return Model([np.zeros((n, n))], [hankel_constraints(n)], p, np.array([-1.0, 1.0]), C_lin)


def sos_hankel_moment(d: int, seed: int = 0) -> Model:
    """The same bound with gamma eliminated: gamma = p_0 - Q_00.

    min Q_00 s.t. <A_k, Q> = p_k for k = 1..2d (m = 2d, no scalars); the
    optimal value is p_0 - gamma*.
    """
    rng = np.random.default_rng(seed)
    n = d + 1
    p = _sos_coefficients(d, rng)
    full = hankel_constraints(n)
    keep = full.con >= 1
    A = BlockConstraints(n, 2 * d, full.con[keep] - 1, full.row[keep], full.col[keep], full.val[keep])
    C = np.zeros((n, n))
    C[0, 0] = 1.0
    return Model([C], [A], p[1:])


def dense_random(sides, ns: int, m: int, seed: int = 0) -> Model:
    """Dense constraint matrices, feasible by construction.

    A_ij symmetric with N(0, 1/n_i) entries, C_lin with N(0, 1) entries;
    X0 = I, x0 = 1, y0 ~ N(0, 1), S0 = I, z0 = 1 give
    b = A(X0) + C_lin x0, C_i = A_i*(y0) + I, d_lin = C_lin' y0 + 1.
    """
    rng = np.random.default_rng(seed)
    y0 = rng.standard_normal(m)
    Cs, As = [], []
    b = np.zeros(m)
    for n in sides:
        Aj = rng.standard_normal((m, n, n)) / np.sqrt(n)
        Aj += Aj.transpose(0, 2, 1)
        Aj /= np.sqrt(2.0)
        b += np.einsum("jaa->j", Aj)
        Cs.append(np.einsum("j,jab->ab", y0, Aj) + np.eye(n))
        # entries in (constraint, column, row) order, the order the model
        # keeps (Aj is exactly symmetric, so Aj[j, c, r] is entry (r, c))
        jj = np.repeat(np.arange(m, dtype=np.int32), n * n)
        cc = np.tile(np.repeat(np.arange(n, dtype=np.int32), n), m)
        rr = np.tile(np.arange(n, dtype=np.int32), m * n)
        As.append(BlockConstraints(n, m, jj, rr, cc, Aj.ravel()))
        del Aj
    C_lin = rng.standard_normal((m, ns))
    b += C_lin.sum(axis=1)
    d_lin = C_lin.T @ y0 + 1.0
    Cs = [(c + c.T) / 2 for c in Cs]
    return Model(Cs, As, b, d_lin, C_lin)


def rank_one_random(sides, ns: int, m: int, seed: int = 0) -> Model:
    """Rank-one constraint matrices A_ij = s_ij v_ij v_ij' (LowRankOpt's
    low-rank format), v_ij with N(0, 1/n_i) entries and signs s_ij = +-1,
    feasible by construction as in dense_random: X0 = I, x0 = 1,
    y0 ~ N(0, 1), S0 = I, z0 = 1."""
    rng = np.random.default_rng(seed)
    y0 = rng.standard_normal(m)
    Cs, As = [], []
    b = np.zeros(m)
    for n in sides:
        Vm = rng.standard_normal((n, m)) / np.sqrt(n)
        sg = rng.choice([-1.0, 1.0], m)
        Aj = np.einsum("j,aj,bj->jab", sg, Vm, Vm)
        b += np.einsum("jaa->j", Aj)
        C = np.einsum("j,jab->ab", y0, Aj) + np.eye(n)
        Cs.append((C + C.T) / 2)
        jj, rr, cc = np.meshgrid(np.arange(m), np.arange(n), np.arange(n), indexing="ij")
        As.append(BlockConstraints(n, m, jj.ravel(), rr.ravel(), cc.ravel(), Aj.ravel()))
    C_lin = rng.standard_normal((m, ns))
    b += C_lin.sum(axis=1)
    d_lin = C_lin.T @ y0 + 1.0
    return Model(Cs, As, b, d_lin, C_lin)


# --- the small problems of the reference tests --------------------------------

def weighted_4node_W() -> np.ndarray:
    """Weighted 4-node graph of test/runtests.jl:73-78 (SDP value 18)."""
    return np.array([[0, 5, 7, 6], [5, 0, 0, 1], [7, 0, 0, 1], [6, 1, 1, 0]], dtype=np.float64)


def cycle4_W() -> np.ndarray:
    """4-cycle of test/runtests.jl:134-139 (SDP value 4)."""
    return np.array([[0, 1, 0, 1], [1, 0, 1, 0], [0, 1, 0, 1], [1, 0, 1, 0]], dtype=np.float64)


def trivial_2x2() -> Model:
    """min <diag(2,1), X> s.t. X_11 = 1 (test/runtests.jl:60-69): value 2."""
    return Model([np.diag([2.0, 1.0])], [[np.diag([1.0, 0.0])]], np.array([1.0]))


def trace_one() -> Model:
    """min <diag(3,2), X> s.t. tr X = 1 (test/runtests.jl:96-107): value 2."""
    return Model([np.diag([3.0, 2.0])], [[np.eye(2)]], np.array([1.0]))


def mixed_lp_example() -> Model:
    """min t + 2x1 + x2, t + x1 = 1, t + x2 = 1 (test/runtests.jl:113-129)."""
    return Model([np.ones((1, 1))], [[np.ones((1, 1)), np.ones((1, 1))]], np.array([1.0, 1.0]),
                 np.array([2.0, 1.0]), np.eye(2))


def qr_example(scalars: int = 0) -> Model:
    """3x3 block with diagonal constraints (test/qr_schur.jl:8-14)."""
    C = np.array([[3, 0.1, 0], [0.1, 2, 0.2], [0, 0.2, 1]], dtype=np.float64)
    A = [np.diag((np.arange(3) == k).astype(np.float64)) for k in range(3)]
    d = np.ones(scalars)
    L = np.arange(1, 3 * scalars + 1, dtype=np.float64).reshape(scalars, 3).T
    return Model([C], [A], np.ones(3), d, L)
