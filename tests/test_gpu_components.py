"""Component-granular entry points against the oracle's components on the
same iterate: _prepare! (NT scaling W, D, S^-1), the Schur complement
assembly (tensor-core products for dense blocks, entry pairs for coordinate
lists, plus the scalar block), the EigenStep lambda_min, and a Schur-solver
component (schur_workspace / factorize! / schur_solve!) in FP64 and mixed
precision."""
import numpy as np
import pytest

import madsdp_gpu as M
from madsdp_gpu import generators as g
from oracle import madsdp_oracle as o

pytestmark = pytest.mark.gpu


def oracle_after(model, iterations=2):
    s = o.Solver(model)
    s.initialize()
    s.update_termination()
    for _ in range(iterations):
        s.iterate()
        s.update_termination()
    return s


@pytest.mark.parametrize("model", [g.dense_random([30, 12], 6, 60, seed=3), g.maxcut(40, 0.2, seed=2),
                                   g.rank_one_random([30, 20], 4, 50, seed=9)],
                         ids=["dense_scalars", "maxcut", "rank_one"])
def test_prepare_and_assembly_match_oracle(gpu_ctx, model):
    ref = oracle_after(model)
    inst = M.InstanceSolver(model)
    inst.set_iterate([b.X for b in ref.blocks], [b.S for b in ref.blocks], ref.y, ref.x, ref.z)
    assert inst.prepare()
    assert ref.prepare()
    for i, b in enumerate(ref.blocks):
        W = inst.block_matrix(i, "W")
        assert np.abs(W - b.W).max() <= 1e-10 * np.abs(b.W).max()
        assert np.allclose(inst.block_matrix(i, "D"), b.D, rtol=1e-10, atol=0)
        Si = inst.block_matrix(i, "Sinv")
        assert np.abs(Si - b.Si).max() <= 1e-10 * np.abs(b.Si).max()
    H = inst.schur_assemble()
    Href = np.tril(ref.schur_complement())
    assert np.abs(H - Href).max() <= 1e-12 * np.abs(Href).max()
    inst.close()


def test_split_precision_assembly(gpu_ctx):
    """The split-precision assembly of a mixed-precision NT solver is an
    FP32-class approximation of the FP64 one."""
    model = g.dense_random([40], 5, 80, seed=8)
    ref = oracle_after(model)
    inst = M.InstanceSolver(model, precision="mixed")
    inst.set_iterate([b.X for b in ref.blocks], [b.S for b in ref.blocks], ref.y, ref.x, ref.z)
    assert inst.prepare()
    H64 = inst.schur_assemble("fp64")
    H32 = inst.schur_assemble("mixed")
    scale = np.abs(H64).max()
    assert np.abs(H32 - H64).max() <= 1e-5 * scale
    assert np.abs(H32 - H64).max() > 0.0
    inst.close()


@pytest.mark.parametrize("n", [20, 150, 300])
def test_step_eig_matches_oracle(gpu_ctx, n):
    rng = np.random.default_rng(n)
    model = g.maxcut(n, 4.0 / n, seed=1)
    inst = M.InstanceSolver(model)
    B = rng.standard_normal((n, n))
    Lm = np.linalg.cholesky(B @ B.T / n + np.eye(n))
    D = rng.standard_normal((n, n))
    D = (D + D.T) / 2
    lam = inst.step_eig(0, Lm, D)
    ref = o.eigmin_congruence(Lm, D)
    assert abs(lam - ref) <= 1e-9 * max(1.0, abs(ref))
    inst.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("m,cond", [(300, 1e3), (1000, 1e4), (500, 1e10)])
def test_schur_workspace_solves(gpu_ctx, precision, m, cond):
    rng = np.random.default_rng(m)
    Q, _ = np.linalg.qr(rng.standard_normal((m, m)))
    H = (Q * np.exp(np.linspace(0, np.log(cond), m))) @ Q.T
    H = (H + H.T) / 2
    ws = M.SchurWorkspace(m, precision=precision)
    Hl = np.tril(H) + np.triu(np.full((m, m), 5.0), 1)  # only the lower triangle is read
    assert ws.factorize(Hl)
    rhs = rng.standard_normal(m)
    x = ws.solve(rhs)
    xr = np.linalg.solve(H, rhs)
    # backward error of a solve with a float64 Cholesky factor
    assert np.abs(H @ x - rhs).max() <= 1e-12 * (np.abs(H).max() * np.abs(x).max() * m ** 0.5)
    assert np.abs(x - xr).max() <= 1e-15 * cond * m * np.abs(xr).max()
    if precision == "mixed" and cond <= 1e4:
        assert not ws.fp64_active  # refinement converged from the FP32-class factor
    x2 = ws.solve(rhs)  # a second solve of the same factorization
    assert np.array_equal(x, x2)
    ws.close()


def test_schur_workspace_reports_indefinite(gpu_ctx):
    H = np.eye(64)
    H[10, 10] = -1.0
    ws = M.SchurWorkspace(64)
    assert not ws.factorize(H)
    ws.close()
