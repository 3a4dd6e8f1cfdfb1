"""Whole-GPU solver of one large problem (msdp_solver) against the oracle:
known answers, every PrimalDual component, coordinate-list (one-hot,
Hankel) and dense constraint assembly, scalar blocks, initial points and
per-iteration trajectories.  Tolerances as in the batch parity tests."""
import json
import os

import numpy as np
import pytest

import madsdp_gpu as M
from madsdp_gpu import generators as g
from oracle import madsdp_oracle as o
from problems import build, compare_trajectories

pytestmark = pytest.mark.gpu
KA = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


def comps(spec, mod):
    return {k: getattr(mod, v)() for k, v in (spec or {}).items()}


def inst(model, **kw):
    return M.MadSDPSolver(model, engine="instance", **kw).solve()


def assert_matches_oracle(s, ref, traj=True, iters=1):
    assert s.status == M.Status.SOLVE_SUCCEEDED, s.stats
    assert int(ref.status) == int(M.Status.SOLVE_SUCCEEDED)
    assert abs(s.iter - ref.iter) <= iters
    scale = max(1.0, abs(ref.primal_objective()) + abs(ref.dual_objective()))
    assert abs(s.primal_objective() - ref.primal_objective()) <= 1e-7 * scale
    assert abs(s.dual_objective() - ref.dual_objective()) <= 1e-7 * scale
    assert max(s.inf_pr, s.inf_du, s.inf_compl) <= 1e-7
    if traj:
        compare_trajectories(s.trajectory(), ref.trajectory)


@pytest.mark.parametrize("case", [c for c in KA["cases"] if "objective" in c], ids=lambda c: c["name"])
def test_known_objective(gpu_ctx, case):
    s = inst(build(case["model"]), **comps(case.get("components"), M), **case["options"])
    assert s.engine == "instance"
    assert abs(s.primal_objective() - case["objective"]) <= case["atol"]
    ref = o.Solver(build(case["model"]), **comps(case.get("components"), o), **case["options"]).solve()
    assert_matches_oracle(s, ref, traj=False)


@pytest.mark.parametrize("direction", ["NT", "HKM"])
@pytest.mark.parametrize("step", ["EigenStep", "CholeskyBacktrack"])
@pytest.mark.parametrize("centering", ["Mehrotra", "AdaptiveMu"])
def test_component_matrix(gpu_ctx, direction, step, centering):
    model = g.maxcut(30, 0.2, seed=7)
    kw = dict(direction=getattr(M, direction)(), step=getattr(M, step)(), centering=getattr(M, centering)())
    okw = dict(direction=getattr(o, direction)(), step=getattr(o, step)(), centering=getattr(o, centering)())
    s = inst(model, **kw)
    ref = o.Solver(model, **okw).solve()
    assert_matches_oracle(s, ref)


def test_maxcut_config1_trajectory(gpu_ctx):
    """MaxCut n = 100, p = 0.1: one-hot constraints, Schur = W o W."""
    model = g.maxcut(100, 0.1, seed=0)
    assert_matches_oracle(inst(model), o.Solver(model).solve())


def test_maxcut_pm1_weights_large(gpu_ctx):
    """MaxCut n = 400 with +-1 weights (the distribution of the n = 2000 case)."""
    model = g.maxcut(400, 0.02, weights="pm1", seed=3)
    assert_matches_oracle(inst(model), o.Solver(model).solve())


@pytest.mark.parametrize("n,refined", [(100, True), (400, False), (700, True)])
def test_nt_eigendecomposition_refined(gpu_ctx, n, refined):
    """The NT eigendecomposition N = V diag(lam) V' by the FP32 eigensolver
    refined to FP64 accuracy with tensor-core products (orders where that is
    faster than the FP64 eigensolver) or by the FP64 eigensolver: the same
    trajectory as the oracle either way, and the counters show which ran."""
    model = g.maxcut(n, 4.0 / n, weights="pm1", seed=n)
    s = M.InstanceSolver(model)
    s.solve()
    c = s.counters()
    st = s.stats()
    s.close()
    if refined:
        assert c["eig_refined"] >= st["iter"] and c["eig_dense"] == 0, c
        assert c["eig_refinement_steps"] <= 6 * c["eig_refined"], c
    else:
        assert c["eig_refined"] == 0 and c["eig_dense"] >= st["iter"], c
    assert_matches_oracle(inst(model), o.Solver(model).solve())


def test_lanczos_step_lengths_hkm(gpu_ctx):
    """Blocks of 257 and more take lambda_min by Lanczos; HKM exercises both
    the primal (Lx) and dual (Ls) congruences."""
    model = g.maxcut(300, 0.03, seed=8)
    assert_matches_oracle(inst(model, direction=M.HKM()), o.Solver(model, direction=o.HKM()).solve())


@pytest.mark.parametrize("direction", ["NT", "HKM"])
def test_dense_mixed_cones(gpu_ctx, direction):
    """Dense A with two PSD blocks and scalars: the GEMM assembly path."""
    model = g.dense_random([14, 9], 6, 40, seed=5)
    s = inst(model, direction=getattr(M, direction)())
    ref = o.Solver(model, direction=getattr(o, direction)()).solve()
    assert_matches_oracle(s, ref)


def test_sos_hankel_pairs(gpu_ctx):
    model = g.sos_hankel(40, seed=9)
    assert_matches_oracle(inst(model), o.Solver(model).solve())


def test_mixed_lp_and_solution(gpu_ctx):
    model = g.mixed_lp_example()
    s = inst(model)
    ref = o.Solver(model).solve()
    assert_matches_oracle(s, ref, traj=False)
    X, y, x, z = s.solution()
    np.testing.assert_allclose(X[0], ref.blocks[0].X, atol=1e-6)
    np.testing.assert_allclose(y, ref.y, atol=1e-6)
    np.testing.assert_allclose(x, ref.x, atol=1e-6)


def test_initial_points(gpu_ctx):
    model = g.maxcut(40, 0.2, seed=2)
    L = -4.0 * model.C[0]
    ip = dict(X=[np.eye(40)], y=-(1.0 + np.abs(L).sum(axis=0)))
    s = inst(model, initial_point=M.InitialPoint(**ip))
    ref = o.Solver(model, initial_point=o.InitialPoint(**ip)).solve()
    assert_matches_oracle(s, ref)
    s = inst(model, initial_point=M.DualShift())
    ref = o.Solver(model, initial_point=o.DualShift()).solve()
    assert_matches_oracle(s, ref)
    s = inst(model, initial_point=M.ScaledIdentity(50.0))
    ref = o.Solver(model, initial_point=o.ScaledIdentity(50.0)).solve()
    assert_matches_oracle(s, ref)


@pytest.mark.parametrize("model_name", ["maxcut400", "dense"])
def test_fp64_tensor_emulation_matches_oracle(gpu_ctx, model_name):
    """precision="fp64_tensor": the dense double-precision products run as
    fixed-point FP64 emulation on tensor cores; the trajectory still matches
    the FP64 oracle at the FP64 tolerances."""
    model = g.maxcut(400, 0.02, weights="pm1", seed=3) if model_name == "maxcut400" else \
        g.dense_random([14, 9], 6, 40, seed=5)
    s = M.MadSDPSolver(model, precision="fp64_tensor").solve()
    assert s.engine == "instance"
    assert_matches_oracle(s, o.Solver(model).solve())


def test_auto_engine_and_unsupported(gpu_ctx):
    assert M.MadSDPSolver(g.maxcut(200, 0.05, seed=1)).engine == "instance"
    assert M.MadSDPSolver(g.maxcut(30, 0.2, seed=1)).engine == "batch"
    with pytest.raises(NotImplementedError):
        M.InstanceSolver(g.maxcut(30, 0.2, seed=1), schur=M.QRSchur())
    with pytest.raises(NotImplementedError):
        M.InstanceSolver(g.maxcut(30, 0.2, seed=1), precision="mixed", direction=M.HKM())
    with pytest.raises(NotImplementedError):
        M.Batch([g.maxcut(30, 0.2, seed=1)], precision="fp64_tensor")
    with pytest.raises(NotImplementedError):
        M.InstanceSolver(g.maxcut(30, 0.2, seed=1), precision="mixed", schur=M.MadNLPSchur())
    # a large problem with a component the whole-GPU engine does not take
    # runs in one thread block, and says so
    with pytest.warns(UserWarning, match="one thread block"):
        s = M.MadSDPSolver(g.maxcut(100, 0.1, seed=1), schur=M.QRSchur())
    assert s.engine == "batch"
    s.close()
    assert M.MadSDPSolver(g.maxcut(100, 0.1, seed=1), schur=M.MadNLPSchur()).engine == "instance"


@pytest.mark.parametrize("direction,model", [("NT", g.maxcut(120, 0.05, seed=8)),
                                             ("HKM", g.dense_random([40, 20], 30, 350, seed=9))])
def test_madnlp_schur_on_the_whole_gpu(gpu_ctx, direction, model):
    """MadNLPSchur (Bunch-Kaufman LDL' of the Schur matrix, src/kkt.jl:7-32,
    src/schur_solvers.jl:23-39) on the whole-GPU engine: the same trajectory
    as the oracle with the same component."""
    s = inst(model, direction=getattr(M, direction)(), schur=M.MadNLPSchur())
    assert s.engine == "instance"
    ref = o.Solver(model, direction=getattr(o, direction)(), schur=o.MadNLPSchur()).solve()
    assert_matches_oracle(s, ref)


# ---------------------------------------------------------------- full sizes
def test_config2_maxcut_n2000_matches_oracle(gpu_ctx):
    """MaxCut n = 2000, p = 0.005, weights +-1 (configuration 2) at full
    size: same iteration count, objectives and per-iteration trajectory as
    the oracle."""
    model = g.maxcut(2000, 0.005, weights="pm1", seed=4)
    s = inst(model)
    ref = o.Solver(model).solve()
    assert_matches_oracle(s, ref)


@pytest.fixture(scope="module")
def config3():
    model = g.dense_random([200, 100, 50, 50], 500, 2000, seed=4)
    return model, o.Solver(model).solve()


def test_config3_dense_mixed_cones_full_size(gpu_ctx, config3):
    """Blocks [200, 100, 50, 50] + 500 scalars, m = 2000, dense A
    (configuration 3) at full size: NT matches the oracle (iterations,
    objectives, per-iteration trajectory; the oracle assembles the dense
    Schur matrix by batched dense products, about a minute on the host
    cores).  Size-independent checks besides: NT and HKM both reach 1e-7,
    their objectives agree, and the solution is in the cones."""
    model, ref = config3
    nt = inst(model)
    assert_matches_oracle(nt, ref)
    hkm = inst(model, direction=M.HKM())
    for s in (nt, hkm):
        assert s.status == M.Status.SOLVE_SUCCEEDED, s.stats
        assert max(s.inf_pr, s.inf_du, s.inf_compl) <= 1e-7
    scale = max(1.0, abs(nt.primal_objective()) + abs(nt.dual_objective()))
    assert abs(nt.primal_objective() - hkm.primal_objective()) <= 1e-6 * scale
    assert abs(nt.dual_objective() - hkm.dual_objective()) <= 1e-6 * scale
    X, y, x, z = nt.solution()
    for Xi in X:
        assert np.linalg.eigvalsh((Xi + Xi.T) / 2)[0] > -1e-8
    assert np.all(x > -1e-10) and np.all(z > -1e-10)


# ---------------------------------------------------------------- mixed precision
# Split-precision Schur assembly on the tensor cores, FP32-class factor and
# FP64 iterative refinement against the matrix-free Schur operator, FP64
# after a stall: same status, objectives to 1e-7 of the oracle's scale and
# the iteration count within one.
@pytest.mark.parametrize("model", [g.dense_random([40, 20], 30, 150, seed=2), g.maxcut(120, 0.05, seed=3),
                                   g.dense_random([60], 0, 400, seed=6)], ids=["dense_scalars", "maxcut", "dense"])
def test_mixed_instance_matches_oracle(gpu_ctx, model):
    s = inst(model, precision="mixed")
    ref = o.Solver(model).solve()
    assert_matches_oracle(s, ref, traj=False)
    st = s.stats
    assert st["iter_fp32"] + st["iter_fp64"] == st["iter"]


def test_mixed_config3_full_size(gpu_ctx, config3):
    """Configuration 3 (NT) in mixed precision: the split-precision
    assembly and FP32-class factor carry most iterations, and the result
    equals the FP64 oracle's."""
    model, ref = config3
    s = inst(model, precision="mixed")
    assert_matches_oracle(s, ref, traj=False)
    assert s.stats["iter_fp32"] >= 1


# ---------------------------------------------------------------- rank-one constraints
# LowRankOpt's low-rank format (README.md:137-152 of the reference): every
# A_j = s_j v_j v_j' is detected at upload and applied through V = [v_1 ...
# v_m] (H = s s' o (V'WV) o (V'WV) for NT, A(X)_j = s_j v_j'Xv_j,
# A*(y) = V diag(s y) V').
@pytest.mark.parametrize("direction", ["NT", "HKM"])
def test_rank_one_constraints_match_oracle(gpu_ctx, direction):
    model = g.rank_one_random([40, 25], 8, 60, seed=5)
    s = inst(model, direction=getattr(M, direction)())
    ref = o.Solver(model, direction=getattr(o, direction)()).solve()
    assert_matches_oracle(s, ref)


def test_rank_one_constraints_mixed(gpu_ctx):
    model = g.rank_one_random([60], 0, 120, seed=6)
    s = inst(model, precision="mixed")
    assert_matches_oracle(s, o.Solver(model).solve(), traj=False)
