"""The oracle against the known answers of the reference test suite."""
import json
import math
import os

import numpy as np
import pytest

from oracle import madsdp_oracle as o
from problems import build, laplacian
from madsdp_gpu import generators as g

KA = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


def comps(spec, mod):
    out = {}
    for k, v in (spec or {}).items():
        out[k] = getattr(mod, v)()
    return out


@pytest.mark.parametrize("case", [c for c in KA["cases"] if "objective" in c], ids=lambda c: c["name"])
def test_known_objective(case):
    s = o.Solver(build(case["model"]), **comps(case.get("components"), o), **case["options"]).solve()
    assert s.status == o.Status.SOLVE_SUCCEEDED
    assert abs(s.primal_objective() - case["objective"]) <= case["atol"]
    if "X11" in case:
        assert abs(s.blocks[0].X[0, 0] - case["X11"]) <= case["X11_atol"]
        assert np.all(s.x < case["x_below"])


@pytest.mark.parametrize("direction", ["NT", "HKM"])
@pytest.mark.parametrize("step", ["EigenStep", "CholeskyBacktrack"])
@pytest.mark.parametrize("centering", ["Mehrotra", "AdaptiveMu"])
def test_component_matrix(direction, step, centering):
    cm = KA["component_matrix"]
    for model, expected in cm["problems"]:
        s = o.Solver(build(model), direction=getattr(o, direction)(), step=getattr(o, step)(),
                     centering=getattr(o, centering)(), max_iter=cm["max_iter"]).solve()
        assert s.status == o.Status.SOLVE_SUCCEEDED
        assert abs(s.primal_objective() - expected) <= cm["atol"]


@pytest.mark.parametrize("schur", ["DenseCholesky", "MadNLPSchur"])
def test_mc_psd_start(schur):
    case = KA["mc_psd_start"]
    W = g.weighted_4node_W()
    L = laplacian(W)
    ip = o.InitialPoint([np.eye(4)], -(1 + np.abs(L / 4).sum(axis=0)))
    s = o.Solver(build("maxcut_weighted4"), direction=o.HKM(), step=o.CholeskyBacktrack(),
                 centering=o.AdaptiveMu(), initial_point=ip, schur=getattr(o, schur)()).solve()
    assert s.status == o.Status.SOLVE_SUCCEEDED
    assert abs(s.primal_objective() - case["objective"]) <= case["atol"]
    assert s.inf_du < case["inf_du_below"]


def test_initial_point_with_scalars():
    case = KA["initial_point_scalars"]
    ip = o.InitialPoint([np.ones((1, 1))], np.array([-1.0, -1.0]), np.array([0.5, 0.5]))
    s = o.Solver(build("mixed_lp"), direction=o.HKM(), initial_point=ip).solve()
    assert s.status == o.Status.SOLVE_SUCCEEDED
    assert abs(s.primal_objective() - case["objective"]) <= case["atol"]


@pytest.mark.parametrize("case", KA["dual_centering"], ids=lambda c: c["model"])
def test_dual_centering(case):
    s = o.Solver(build(case["model"]), algorithm=o.DualCentering(), tol=case["tol"],
                 max_iter=case["max_iter"]).solve()
    assert s.status == o.Status.SOLVE_SUCCEEDED
    assert abs(s.dual_objective() - case["dual_objective"]) <= case["atol"]
    if "primal_objective" in case:
        assert abs(s.primal_objective() - case["primal_objective"]) <= case["atol"]
    if "inf_du_below" in case:
        assert s.inf_du < case["inf_du_below"]


def test_dual_centering_theoretical_A_and_bunch_kaufman():
    # test/dual_runtests.jl:76-101, second half
    W = g.weighted_4node_W()
    L = laplacian(W)
    y0 = -(1 + np.abs(L / 4).sum(axis=0))
    s = o.Solver(build("maxcut_weighted4"), algorithm=o.DualCentering(A=None),
                 initial_point=o.InitialPoint([np.eye(4)], y0), schur=o.MadNLPSchur(),
                 tol=1e-6, max_iter=300).solve()
    assert s.status == o.Status.SOLVE_SUCCEEDED
    assert abs(s.dual_objective() + 18.0) <= 1e-3


def test_dual_centering_errors():
    # test/dual_runtests.jl:103-131
    model = g.maxcut_from_weights(np.ones((2, 2)) - np.eye(2))
    with pytest.raises(RuntimeError):
        o.Solver(model, algorithm=o.DualCentering(),
                 initial_point=o.InitialPoint([np.eye(2)], np.array([1.0, 1.0]))).solve()
    with pytest.raises(RuntimeError):
        o.Solver(model, algorithm=o.DualCentering(), initial_point=o.DualShift(1.0, 0.1)).solve()
    with pytest.raises(RuntimeError):
        o.Solver(build("mixed_lp"), algorithm=o.DualCentering())


def test_qr_schur_solves():
    # test/qr_schur.jl:68-91
    from madsdp_gpu.model import Model
    lp = Model([], [], np.array([1.0]), np.array([1.0, 2.0]), np.array([[1.0, 1.0]]))
    for model in (build("qr_example"), build("qr_example2"), lp):
        s = o.Solver(model, schur=o.QRSchur(), initial_point=o.ScaledIdentity(),
                     step=o.CholeskyBacktrack()).solve()
        assert s.status == o.Status.SOLVE_SUCCEEDED
        assert max(s.inf_pr, s.inf_du, s.inf_compl) <= s.opt.tol


def test_qr_unsupported_and_rank_deficient():
    # test/qr_schur.jl:93-139
    from madsdp_gpu.model import Model
    with pytest.raises(ValueError):
        o.Solver(build("qr_example"), schur=o.QRSchur(), direction=o.HKM())
    with pytest.raises(ValueError):
        o.Solver(build("qr_example"), schur=o.QRSchur(), algorithm=o.DualCentering())
    zero = Model([np.ones((1, 1))], [[np.zeros((1, 1))]], np.array([0.0]))
    s = o.Solver(zero, schur=o.QRSchur()).solve()
    assert s.status == o.Status.ERROR_IN_STEP_COMPUTATION
    for d, mats in ((1, [np.ones((1, 1)), np.ones((1, 1))]),
                    (2, [np.diag([1.0, 0.0]), np.diag([1.0, 0.0])])):
        model = Model([np.eye(d)], [mats], np.ones(2))
        s = o.Solver(model, schur=o.QRSchur()).solve()
        assert s.status == o.Status.ERROR_IN_STEP_COMPUTATION


def test_identity_scale():
    # test/identity_scale.jl:17-42
    for scale in (1, 0.2, 10.0):
        s = o.Solver(g.qr_example(2), initial_point=o.ScaledIdentity(scale))
        s.initialize()
        assert np.array_equal(s.blocks[0].X, scale * np.eye(3))
        assert np.array_equal(s.blocks[0].S, scale * np.eye(3))
        assert np.all(s.x == scale) and np.all(s.z == scale) and np.all(s.y == 0)
    for scale in (0, -1.0, math.inf, math.nan):
        with pytest.raises(ValueError):
            o.ScaledIdentity(scale)
    model = g.qr_example(2)
    model.b *= 1000
    s = o.Solver(model)
    s.initialize()
    expected = math.sqrt(KA["identity_scale"]["value_squared"])
    assert np.allclose(s.blocks[0].X, expected * np.eye(3))
    assert np.allclose(s.x, expected) and np.allclose(s.z, expected)


def test_cholesky_flush():
    # test/blocks.jl:9-35
    M = np.array([[4.0, 1.0], [3.0, 2.0]])
    L = o._cholesky_factor(M)
    assert L is not None
    assert np.allclose(L @ L.T, (M + M.T) / 2)
    assert L[0, 1] == 0.0
    assert np.array_equal(M, [[4.0, 1.0], [3.0, 2.0]])
    for N in (np.array([[1.0, 2.0], [2.0, 1.0]]), np.zeros((2, 2))):
        assert o._cholesky_factor(N) is None
    eps = np.finfo(np.float64).eps
    F = np.array([[1, 0, 0], [np.finfo(np.float64).tiny, 1, 0], [eps, 1, 1]])
    L = o._cholesky_factor(F @ F.T)
    assert L[1, 0] == 0.0
    assert L[2, 0] == eps
    assert np.allclose(L @ L.T, F @ F.T)


def test_small_mu_does_not_certify_optimality():
    # test/termination.jl:15-40
    from madsdp_gpu.model import Model

    def scalar_solver():
        return o.Solver(Model([np.ones((1, 1))], [[np.ones((1, 1))]], np.array([1.0])))
    for x, sv, y in ((2.0, 0.0, 1.0), (1.0, 0.0, 0.0), (1.0, 1.0, 0.0)):
        s = scalar_solver()
        s.initialize()
        s.blocks[0].X[0, 0], s.blocks[0].S[0, 0], s.y[0] = x, sv, y
        s.mu = 0.0
        s.update_residuals()
        s.update_termination()
        assert s.status == o.Status.SEARCH_DIRECTION_BECOMES_TOO_SMALL
        assert max(s.inf_pr, s.inf_du, s.inf_compl) > s.opt.tol
    s = scalar_solver()
    s.initialize()
    s.blocks[0].X[0, 0], s.blocks[0].S[0, 0], s.y[0] = 1.0, 0.0, 1.0
    s.mu = 0.0
    s.update_residuals()
    s.update_termination()
    assert s.status == o.Status.SOLVE_SUCCEEDED
    assert max(s.inf_pr, s.inf_du, s.inf_compl) == 0
