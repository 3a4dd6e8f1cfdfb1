"""Newton-system identities of the oracle (test/qr_schur.jl:16-66)."""
import numpy as np
import pytest

from oracle import madsdp_oracle as o
from madsdp_gpu import generators as g

X_DIAG = np.diag([2.0, 3.0, 4.0])
S_DIAG = np.diag([4.0, 2.0, 3.0])
X_FULL = np.array([[2.0, 0.3, 0.1], [0.3, 3.0, 0.4], [0.1, 0.4, 4.0]])
S_FULL = np.array([[4.0, -0.2, 0.1], [-0.2, 2.0, 0.3], [0.1, 0.3, 3.0]])


def check_identities(s, model, mu, corrected, atol=1e-10):
    b = s.blocks[0]
    op = s.ops[0]
    lhs = op.jprod(b.delX) + model.C_lin @ s.delx
    assert np.allclose(lhs, s.Rp, atol=atol)
    dual = op.jtprod(s.dely)
    assert np.allclose(b.delS + dual, b.Rd, atol=atol)
    center = mu * np.linalg.inv(b.S) - b.X
    if corrected:
        center = center + b.corr
    assert np.allclose(b.delX + b.W @ b.delS @ b.W, center, atol=atol)


@pytest.mark.parametrize("scalars", [0, 2])
@pytest.mark.parametrize("diagonal", [True, False])
def test_newton_identities_dense_vs_qr(scalars, diagonal):
    model = g.qr_example(scalars)
    solvers = [o.Solver(model, schur=sc, initial_point=o.ScaledIdentity()) for sc in (o.DenseCholesky(), o.QRSchur())]
    for s in solvers:
        s.initialize()
        s.blocks[0].X = (X_DIAG if diagonal else X_FULL).copy()
        s.blocks[0].S = (S_DIAG if diagonal else S_FULL).copy()
        s.update_residuals()
        assert s.prepare()
        assert s.factorize_schur()
    for corrected in (False, True):
        mu = 0.3 if corrected else 0.0
        for s in solvers:
            if corrected:
                s.correction()
            s.solve_directions(mu, corrected)
            check_identities(s, model, mu, corrected)
        a, c = solvers
        assert np.allclose(a.dely, c.dely, atol=1e-10)
        assert np.allclose(a.delx, c.delx, atol=1e-10)
        assert np.allclose(a.delz, c.delz, atol=1e-10)
        assert np.allclose(a.blocks[0].delX, c.blocks[0].delX, atol=1e-10)


@pytest.mark.parametrize("sides,m", [([6], 20), ([12], 60), ([9, 5], 40), ([16], 100)])
def test_dense_schur_summation_orders_agree(sides, m):
    """The oracle's three summation orders of H_jk = <A_j, L A_k R> (entry
    pairs, constraint by constraint, batched dense products) agree on
    dense constraints, for symmetric L = R (NT) and L != R (HKM)."""
    from oracle.madsdp_oracle import _BlockOp
    model = g.dense_random(sides, 0, m, seed=7)
    rng = np.random.default_rng(1)
    for blk in model.A:
        op = _BlockOp(blk)
        n = op.n
        M1, M2 = rng.standard_normal((n, n)), rng.standard_normal((n, n))
        W = M1 @ M1.T + n * np.eye(n)
        X, Si = M2 @ M2.T + n * np.eye(n), W / n
        for L, R in ((W, W), (Si, X)):
            ref = op.schur_columns(L, R)
            scale = np.abs(ref).max()
            assert np.abs(op.schur_dense(L, R) - ref).max() <= 1e-13 * scale
            if op.nnz <= op.dense_threshold:  # the entry-pair order (nnz^2 memory)
                assert np.abs(op.schur(L, R) - ref).max() <= 1e-13 * scale
