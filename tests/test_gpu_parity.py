"""GPU (libmadsdp_gpu.so, sm_103a) against the oracle and the reference's
known answers.  Tolerances: objectives as in the reference tests; per
iteration, pobj/dobj relative difference <= 1e-6 while the gap is above
1e-5; final objectives within 1e-7 * max(1, |p| + |d|) of the oracle."""
import json
import math
import os

import numpy as np
import pytest

import madsdp_gpu as M
from madsdp_gpu import generators as g
from oracle import madsdp_oracle as o
from problems import build, compare_trajectories, laplacian

pytestmark = pytest.mark.gpu
KA = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


def comps(spec, mod):
    return {k: getattr(mod, v)() for k, v in (spec or {}).items()}


def gpu_solve(model, **kw):
    return M.MadSDPSolver(model, engine="batch", **kw).solve()


@pytest.mark.parametrize("case", [c for c in KA["cases"] if "objective" in c], ids=lambda c: c["name"])
def test_known_objective(gpu_ctx, case):
    s = gpu_solve(build(case["model"]), **comps(case.get("components"), M), **case["options"])
    assert s.status == M.Status.SOLVE_SUCCEEDED
    assert abs(s.primal_objective() - case["objective"]) <= case["atol"]
    ref = o.Solver(build(case["model"]), **comps(case.get("components"), o), **case["options"]).solve()
    scale = max(1.0, abs(ref.primal_objective()) + abs(ref.dual_objective()))
    assert abs(s.primal_objective() - ref.primal_objective()) <= 1e-7 * scale
    assert abs(s.iter - ref.iter) <= 1
    if "X11" in case:
        X, y, x, z = s.solution()
        assert abs(X[0][0, 0] - case["X11"]) <= case["X11_atol"]
        assert np.all(x < case["x_below"])


@pytest.mark.parametrize("direction", ["NT", "HKM"])
@pytest.mark.parametrize("step", ["EigenStep", "CholeskyBacktrack"])
@pytest.mark.parametrize("centering", ["Mehrotra", "AdaptiveMu"])
def test_component_matrix(gpu_ctx, direction, step, centering):
    cm = KA["component_matrix"]
    for model, expected in cm["problems"]:
        kw = dict(direction=getattr(M, direction)(), step=getattr(M, step)(),
                  centering=getattr(M, centering)(), max_iter=cm["max_iter"])
        s = gpu_solve(build(model), **kw)
        assert s.status == M.Status.SOLVE_SUCCEEDED, (model, s.stats)
        assert abs(s.primal_objective() - expected) <= cm["atol"]


@pytest.mark.parametrize("schur", ["DenseCholesky", "MadNLPSchur"])
def test_mc_psd_start(gpu_ctx, schur):
    case = KA["mc_psd_start"]
    L = laplacian(g.weighted_4node_W())
    ip = M.InitialPoint([np.eye(4)], -(1 + np.abs(L / 4).sum(axis=0)))
    s = gpu_solve(build("maxcut_weighted4"), direction=M.HKM(), step=M.CholeskyBacktrack(),
                  centering=M.AdaptiveMu(), initial_point=ip, schur=getattr(M, schur)())
    assert s.status == M.Status.SOLVE_SUCCEEDED
    assert abs(s.primal_objective() - case["objective"]) <= case["atol"]
    assert s.inf_du < case["inf_du_below"]


def test_initial_point_with_scalars(gpu_ctx):
    ip = M.InitialPoint([np.ones((1, 1))], np.array([-1.0, -1.0]), np.array([0.5, 0.5]))
    s = gpu_solve(build("mixed_lp"), direction=M.HKM(), initial_point=ip)
    assert s.status == M.Status.SOLVE_SUCCEEDED
    assert abs(s.primal_objective() - 1.0) <= 1e-5


def test_identity_scale(gpu_ctx):
    for scale in (1, 0.2, 10.0):
        s = M.MadSDPSolver(g.qr_example(2), initial_point=M.ScaledIdentity(scale))
        s.initialize()
        X, y, x, z = s.solution()
        assert np.array_equal(X[0], scale * np.eye(3))
        assert np.all(x == scale) and np.all(z == scale) and np.all(y == 0)
    model = g.qr_example(2)
    model.b *= 1000
    s = M.MadSDPSolver(model)
    s.initialize()
    X, y, x, z = s.solution()
    assert np.allclose(X[0], math.sqrt(15000.0) * np.eye(3))


def test_dual_shift_failure_raises(gpu_ctx):
    model = g.maxcut_from_weights(np.ones((2, 2)) - np.eye(2))
    with pytest.raises(RuntimeError):
        M.MadSDPSolver(model, direction=M.HKM(), initial_point=M.DualShift(1.0, 0.1)).solve()


X_FULL = np.array([[2.0, 0.3, 0.1], [0.3, 3.0, 0.4], [0.1, 0.4, 4.0]])
S_FULL = np.array([[4.0, -0.2, 0.1], [-0.2, 2.0, 0.3], [0.1, 0.3, 3.0]])


@pytest.mark.parametrize("schur", ["DenseCholesky", "QRSchur"])
@pytest.mark.parametrize("scalars", [0, 2])
@pytest.mark.parametrize("diagonal", [True, False])
def test_newton_identities(gpu_ctx, scalars, diagonal, schur):
    """test/qr_schur.jl:16-66 through the component entry points."""
    model = g.qr_example(scalars)
    X0 = np.diag([2.0, 3.0, 4.0]) if diagonal else X_FULL
    S0 = np.diag([4.0, 2.0, 3.0]) if diagonal else S_FULL
    bt = M.Batch([model], initial_point=M.ScaledIdentity(), schur=getattr(M, schur)())
    bt.initialize()
    bt.set_iterate(0, X=[X0], S=[S0])
    bt.update_residuals()
    assert bt.prepare()[0]
    ref = o.Solver(model, initial_point=o.ScaledIdentity())
    ref.initialize()
    ref.blocks[0].X, ref.blocks[0].S = X0.copy(), S0.copy()
    ref.update_residuals()
    assert ref.prepare() and ref.factorize_schur()
    A = [model.A[0].dense(j) for j in range(model.m)]
    for corrected in (False, True):
        mu = 0.3 if corrected else 0.0
        if corrected:
            bt.correction()
            ref.correction()
        bt.solve_directions(mu, corrected)
        ref.solve_directions(mu, corrected)
        dX, dS, dy, dx, dz = bt.directions(0)
        Rp, Rd, Rdl = bt.residuals(0)
        W = bt.block_matrix(0, 0, "W")
        lhs = np.array([np.sum(A[j] * dX[0]) for j in range(model.m)]) + model.C_lin @ dx
        assert np.allclose(lhs, Rp, atol=1e-10)
        assert np.allclose(dS[0] + sum(A[j] * dy[j] for j in range(model.m)), Rd[0], atol=1e-10)
        center = mu * np.linalg.inv(S0) - X0
        if corrected:
            center = center + bt.block_matrix(0, 0, "corr")
        assert np.allclose(dX[0] + W @ dS[0] @ W, center, atol=1e-10)
        assert np.allclose(dy, ref.dely, atol=1e-10)
        assert np.allclose(dX[0], ref.blocks[0].delX, atol=1e-10)
        assert np.allclose(dx, ref.delx, atol=1e-10)
        assert np.allclose(W, ref.blocks[0].W, atol=1e-10)


def test_trajectory_maxcut_config1(gpu_ctx):
    """MaxCut n = 100, p = 0.1, NT + EigenStep + Mehrotra + DenseCholesky, FP64."""
    model = g.maxcut(100, 0.1, seed=0)
    ref = o.Solver(model).solve()
    s = gpu_solve(model)
    assert s.status == M.Status.SOLVE_SUCCEEDED
    assert abs(s.iter - ref.iter) <= 1
    scale = max(1.0, abs(ref.primal_objective()) + abs(ref.dual_objective()))
    assert abs(s.primal_objective() - ref.primal_objective()) <= 1e-7 * scale
    assert abs(s.dual_objective() - ref.dual_objective()) <= 1e-7 * scale
    assert max(s.inf_pr, s.inf_du, s.inf_compl) <= 1e-7
    compare_trajectories(s.trajectory(), ref.trajectory)


def sos_batch(n=12, seed=0, dmin=5, dmax=24):
    rng = np.random.default_rng(seed)
    ds = rng.integers(dmin, dmax + 1, size=n)
    return [g.sos_hankel(int(d), seed=1000 + i) for i, d in enumerate(ds)]


@pytest.mark.parametrize("direction", ["NT", "HKM"])
def test_sos_batch_fp64(gpu_ctx, direction):
    models = sos_batch()
    bt = M.Batch(models, direction=getattr(M, direction)())
    bt.solve()
    stats = bt.all_stats()
    for i, (m, st) in enumerate(zip(models, stats)):
        ref = o.Solver(m, direction=getattr(o, direction)()).solve()
        assert st["status"] == M.Status.SOLVE_SUCCEEDED, (i, st)
        scale = max(1.0, abs(ref.primal_objective()) + abs(ref.dual_objective()))
        assert abs(st["pobj"] - ref.primal_objective()) <= 1e-7 * scale, (i, st["pobj"], ref.primal_objective())
        assert abs(st["iter"] - ref.iter) <= 1
        compare_trajectories(bt.trajectory(i), ref.trajectory)


def test_sos_batch_fft_assembly(gpu_ctx):
    """Gram blocks of 32 and more assemble the Hankel Schur matrix in float64
    through an FFT along one index; trajectories still match the oracle."""
    models = sos_batch(n=6, seed=7, dmin=31, dmax=90)
    bt = M.Batch(models)
    bt.solve()
    for i, (m, st) in enumerate(zip(models, bt.all_stats())):
        ref = o.Solver(m).solve()
        assert st["status"] == M.Status.SOLVE_SUCCEEDED, (i, st)
        scale = max(1.0, abs(ref.primal_objective()) + abs(ref.dual_objective()))
        assert abs(st["pobj"] - ref.primal_objective()) <= 1e-7 * scale
        assert abs(st["iter"] - ref.iter) <= 1
        compare_trajectories(bt.trajectory(i), ref.trajectory)


def test_sos_batch_mixed(gpu_ctx):
    """Mixed precision reaches the same tolerance; its error against the
    FP64 oracle is within the tolerance of the objective gap."""
    models = sos_batch(seed=1)
    bt = M.Batch(models, precision="mixed")
    bt.solve()
    for i, (m, st) in enumerate(zip(models, bt.all_stats())):
        ref = o.Solver(m).solve()
        assert st["status"] == M.Status.SOLVE_SUCCEEDED, (i, st)
        assert max(st["inf_pr"], st["inf_du"], st["gap"]) <= 1e-7
        scale = max(1.0, abs(ref.primal_objective()) + abs(ref.dual_objective()))
        assert abs(st["pobj"] - ref.primal_objective()) <= 1e-7 * scale
        assert st["iter_fp32"] >= 1


def test_mixed_late_fp32_steps_stay_interior(gpu_ctx):
    """Near convergence, with cond(S) close to 1/eps_f32, a step length from
    FP32 factors can overshoot the PSD boundary; such steps are checked in
    float64 before they are taken (max-cut requests of the served stream
    that ended in ERROR_IN_STEP_COMPUTATION without the check)."""
    from madsdp_gpu.serving import poisson_stream
    st = poisson_stream(200.0, 1.0, seed=21, sos_d=(5, 127), maxcut_n=(20, 100), dense_n=(8, 32), dense_m=200)
    mc = [m for _, k, m in st if k == "maxcut"]
    assert len(mc) >= 34
    bt = M.Batch(mc, precision="mixed")
    bt.solve()
    for i, s in enumerate(bt.all_stats()):
        assert s["status"] == M.Status.SOLVE_SUCCEEDED, (i, s)
        assert max(s["inf_pr"], s["inf_du"], s["gap"]) <= 1e-7


def test_mixed_blocks_beyond_shared_memory(gpu_ctx):
    """Blocks whose FP64 Jacobi operands exceed shared memory (n > 67) polish
    the FP32 eigenvectors through global scratch."""
    models = [g.sos_hankel(79, seed=31), g.maxcut(100, 0.04, seed=32), g.sos_hankel(120, seed=33)]
    bt = M.Batch(models, precision="mixed")
    bt.solve()
    for m, st in zip(models, bt.all_stats()):
        ref = o.Solver(m).solve()
        assert st["status"] == M.Status.SOLVE_SUCCEEDED, st
        assert max(st["inf_pr"], st["inf_du"], st["gap"]) <= 1e-7
        scale = max(1.0, abs(ref.primal_objective()) + abs(ref.dual_objective()))
        assert abs(st["pobj"] - ref.primal_objective()) <= 1e-7 * scale


def test_batch_uneven_results_independent_of_mix(gpu_ctx):
    """A problem's result is the same alone and inside an uneven batch."""
    models = [g.sos_hankel(7, seed=5), g.maxcut(30, 0.2, seed=3), g.sos_hankel(20, seed=6),
              g.dense_random([6, 4], 3, 10, seed=2)]
    together = M.Batch(models)
    together.solve()
    st_all = together.all_stats()
    for i, m in enumerate(models):
        alone = M.Batch([m])
        alone.solve()
        a = alone.all_stats()[0]
        assert a["status"] == st_all[i]["status"] == M.Status.SOLVE_SUCCEEDED
        assert a["iter"] == st_all[i]["iter"]
        assert a["pobj"] == st_all[i]["pobj"] and a["dobj"] == st_all[i]["dobj"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("direction", ["NT", "HKM"])
def test_dense_constraints_column_assembly(gpu_ctx, direction, precision):
    """Dense A_j (every entry nonzero) takes the column assembly
    T_k = L A_k R, H_jk = A_j(T_k) instead of entry pairs."""
    models = [g.dense_random([10], 0, 30, seed=11), g.dense_random([8, 5], 3, 25, seed=12)]
    bt = M.Batch(models, direction=getattr(M, direction)(), precision=precision)
    bt.solve()
    for m, st in zip(models, bt.all_stats()):
        ref = o.Solver(m, direction=getattr(o, direction)()).solve()
        assert st["status"] == M.Status.SOLVE_SUCCEEDED, st
        scale = max(1.0, abs(ref.primal_objective()) + abs(ref.dual_objective()))
        assert abs(st["pobj"] - ref.primal_objective()) <= 1e-7 * scale
        if precision == "fp64":
            assert abs(st["iter"] - ref.iter) <= 1


# ------------------------------------------------------------------ DualCentering
@pytest.mark.parametrize("case", KA["dual_centering"], ids=lambda c: c["model"])
def test_dual_centering_known_answers(gpu_ctx, case):
    s = gpu_solve(build(case["model"]), algorithm=M.DualCentering(), tol=case["tol"], max_iter=case["max_iter"])
    assert s.status == M.Status.SOLVE_SUCCEEDED, s.stats
    assert abs(s.dual_objective() - case["dual_objective"]) <= case["atol"]
    if "primal_objective" in case:
        assert abs(s.primal_objective() - case["primal_objective"]) <= case["atol"]
    if "inf_du_below" in case:
        assert s.inf_du < case["inf_du_below"]
    ref = o.Solver(build(case["model"]), algorithm=o.DualCentering(), tol=case["tol"], max_iter=case["max_iter"]).solve()
    assert abs(s.iter - ref.iter) <= 1
    scale = max(1.0, abs(ref.dual_objective()))
    assert abs(s.dual_objective() - ref.dual_objective()) <= 1e-7 * scale
    st = s.stats
    assert st["n_newton"] == ref.n_newton and st["n_predictor"] == ref.n_predictor


def test_dual_centering_theoretical_A(gpu_ctx):
    # test/dual_runtests.jl:76-101 (second half, with the MadNLPSchur solver)
    L = laplacian(g.weighted_4node_W())
    y0 = -(1 + np.abs(L / 4).sum(axis=0))
    s = gpu_solve(build("maxcut_weighted4"), algorithm=M.DualCentering(A=None),
                  initial_point=M.InitialPoint([np.eye(4)], y0), schur=M.MadNLPSchur(), tol=1e-6, max_iter=300)
    assert s.status == M.Status.SOLVE_SUCCEEDED
    assert abs(s.dual_objective() + 18.0) <= 1e-3


def test_dual_centering_errors(gpu_ctx):
    # test/dual_runtests.jl:103-131
    model = g.maxcut_from_weights(np.ones((2, 2)) - np.eye(2))
    with pytest.raises(RuntimeError):
        gpu_solve(model, algorithm=M.DualCentering(),
                  initial_point=M.InitialPoint([np.eye(2)], np.array([1.0, 1.0])))
    with pytest.raises(RuntimeError):
        gpu_solve(model, algorithm=M.DualCentering(), initial_point=M.DualShift(1.0, 0.1))
    with pytest.raises(RuntimeError):
        M.MadSDPSolver(build("mixed_lp"), algorithm=M.DualCentering())


def test_dual_centering_trajectory(gpu_ctx):
    model = g.maxcut(20, 0.3, seed=8)
    ref = o.Solver(model, algorithm=o.DualCentering()).solve()
    s = gpu_solve(model, algorithm=M.DualCentering())
    assert s.status == M.Status.SOLVE_SUCCEEDED
    assert abs(s.iter - ref.iter) <= 1
    compare_trajectories(s.trajectory(), ref.trajectory)
    st = s.stats
    assert st["n_newton"] > 0 and st["n_predictor"] > 0


# ------------------------------------------------------------------ QRSchur
def test_qr_solves_psd_and_lp(gpu_ctx):
    """test/qr_schur.jl:68-91."""
    from madsdp_gpu.model import Model
    lp = Model([], [], np.array([1.0]), np.array([1.0, 2.0]), np.array([[1.0, 1.0]]))
    for model in (g.qr_example(0), g.qr_example(2), lp):
        s = gpu_solve(model, schur=M.QRSchur(), initial_point=M.ScaledIdentity(), step=M.CholeskyBacktrack())
        assert s.status == M.Status.SOLVE_SUCCEEDED
        assert max(s.inf_pr, s.inf_du, s.inf_compl) <= 1e-7
        ref = o.Solver(model, schur=o.QRSchur(), initial_point=o.ScaledIdentity(), step=o.CholeskyBacktrack()).solve()
        scale = max(1.0, abs(ref.primal_objective()) + abs(ref.dual_objective()))
        assert abs(s.primal_objective() - ref.primal_objective()) <= 1e-7 * scale
        assert abs(s.iter - ref.iter) <= 1


def test_qr_matches_dense_cholesky_on_sos(gpu_ctx):
    model = g.sos_hankel(8, seed=21)
    a = gpu_solve(model, schur=M.QRSchur())
    b = gpu_solve(model)
    assert a.status == b.status == M.Status.SOLVE_SUCCEEDED
    assert abs(a.primal_objective() - b.primal_objective()) <= 1e-7 * max(1.0, abs(b.primal_objective()))


def test_qr_unsupported_and_rank_deficient(gpu_ctx):
    """test/qr_schur.jl:93-139."""
    from madsdp_gpu.model import Model
    with pytest.raises(ValueError):
        M.MadSDPSolver(g.qr_example(), schur=M.QRSchur(), direction=M.HKM())
    with pytest.raises(ValueError):
        M.MadSDPSolver(g.qr_example(), schur=M.QRSchur(), algorithm=M.DualCentering())
    with pytest.raises(ValueError):
        M.MadSDPSolver(g.qr_example(), schur=M.QRSchur(), precision="mixed")
    zero = Model([np.ones((1, 1))], [[np.zeros((1, 1))]], np.array([0.0]))
    assert gpu_solve(zero, schur=M.QRSchur()).status == M.Status.ERROR_IN_STEP_COMPUTATION
    for d, mats in ((1, [np.ones((1, 1)), np.ones((1, 1))]),
                    (2, [np.diag([1.0, 0.0]), np.diag([1.0, 0.0])])):
        model = Model([np.eye(d)], [mats], np.ones(2))
        assert gpu_solve(model, schur=M.QRSchur()).status == M.Status.ERROR_IN_STEP_COMPUTATION


# ------------------------------------------------------------------ MadNLPSchur (Bunch-Kaufman)
@pytest.mark.parametrize("model_name", ["maxcut_weighted4", "mixed_lp", "qr_example2"])
def test_madnlp_schur_matches_oracle(gpu_ctx, model_name):
    model = build(model_name)
    s = gpu_solve(model, schur=M.MadNLPSchur())
    ref = o.Solver(build(model_name), schur=o.MadNLPSchur()).solve()
    assert s.status == ref.status == M.Status.SOLVE_SUCCEEDED
    scale = max(1.0, abs(ref.primal_objective()) + abs(ref.dual_objective()))
    assert abs(s.primal_objective() - ref.primal_objective()) <= 1e-7 * scale
    assert abs(s.iter - ref.iter) <= 1


def test_madnlp_schur_batch_sos(gpu_ctx):
    models = sos_batch(n=6, seed=3)
    a = M.Batch(models, schur=M.MadNLPSchur())
    a.solve()
    b = M.Batch(models)
    b.solve()
    for sa, sb in zip(a.all_stats(), b.all_stats()):
        assert sa["status"] == sb["status"] == M.Status.SOLVE_SUCCEEDED
        assert abs(sa["pobj"] - sb["pobj"]) <= 1e-7 * max(1.0, abs(sb["pobj"]) + abs(sb["dobj"]))
