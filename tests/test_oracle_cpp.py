"""The compiled CPU restatement (oracle/cpu_ipm.cpp) against the NumPy
oracle and the reference's known answers; runs on CPU.

The compiled port times the CPU baseline, so it has to take the same
iterates as the checker: same status and iteration count, objectives equal
to rounding, on every default-component case."""
import json
import os

import numpy as np
import pytest

from madsdp_gpu import generators as g
from oracle import cpu_ipm
from oracle import madsdp_oracle as o
from problems import build

KA = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


def agree(model, rtol=1e-9, iter_tol=0, **options):
    """Same status and iterates to rounding (default); with rtol = 1e-7 and
    iter_tol = 1 the GPU-vs-oracle contract, for runs long and ill-conditioned
    enough that rounding differences grow to the termination tolerance."""
    c = cpu_ipm.solve(model, **options)
    r = o.Solver(model, **options).solve()
    scale = max(1.0, abs(r.primal_objective()) + abs(r.dual_objective()))
    assert c["status"] == int(r.status)
    assert abs(c["iter"] - r.iter) <= iter_tol
    assert abs(c["pobj"] - r.primal_objective()) <= rtol * scale
    assert abs(c["dobj"] - r.dual_objective()) <= rtol * scale
    if iter_tol == 0:
        for key, ref in (("inf_pr", r.inf_pr), ("inf_du", r.inf_du), ("gap", r.inf_compl)):
            assert abs(c[key] - ref) <= 1e-9 + 1e-3 * ref, key
    return c


@pytest.mark.parametrize("case", [c for c in KA["cases"] if "objective" in c and not c.get("components")],
                         ids=lambda c: c["name"])
def test_known_objective(case):
    opts = {k: v for k, v in case["options"].items() if k in ("tol", "max_iter")}
    c = agree(build(case["model"]), **opts)
    assert c["status"] == 1
    assert abs(c["pobj"] - case["objective"]) <= case["atol"]


@pytest.mark.parametrize("name", ["trivial_2x2", "trace_one", "mixed_lp", "maxcut_weighted4", "maxcut_cycle4",
                                  "maxcut_K4", "qr_example", "qr_example2"])
def test_reference_fixtures(name):
    agree(build(name))


@pytest.mark.parametrize("d", [5, 9, 17, 31])
def test_sos_hankel(d):
    agree(g.sos_hankel(d, seed=d))


@pytest.mark.parametrize("n,p", [(12, 0.3), (30, 0.2)])
def test_maxcut(n, p):
    agree(g.maxcut(n, p, seed=n))


def test_dense_mixed_cones():
    # dense constraints: the per-constraint summation order of the assembly
    agree(g.dense_random([8, 5, 3], 4, 25, seed=3))


def test_dense_one_block_served_mix_shape():
    from madsdp_gpu.serving import _dense_request
    agree(_dense_request(np.random.default_rng(7), 16, 16, 60, 11))


COMBOS = [(d, st, c) for d in ("NT", "HKM") for st in ("EigenStep", "CholeskyBacktrack")
          for c in ("Mehrotra", "AdaptiveMu")]


@pytest.mark.parametrize("direction,step,centering", COMBOS)
def test_component_matrix(direction, step, centering):
    """The reference's component matrix (test/runtests.jl:157-184) and an
    SOS and a max-cut instance with every combination."""
    comps = dict(direction=getattr(o, direction)(), step=getattr(o, step)(), centering=getattr(o, centering)())
    cm = KA["component_matrix"]
    for model, expected in cm["problems"]:
        c = agree(build(model), max_iter=cm["max_iter"], **comps)
        assert c["status"] == 1 and abs(c["pobj"] - expected) <= cm["atol"]
    # SOS under AdaptiveMu: 33 iterations, cond(X) and cond(S) reach 4.5e12
    # (1e9-1e10 under Mehrotra), ending at the tolerance edge
    loose = dict(rtol=1e-7, iter_tol=1) if centering == "AdaptiveMu" else {}
    agree(g.sos_hankel(11, seed=2), **loose, **comps)
    agree(g.maxcut(16, 0.3, seed=5), **comps)


def test_component_parameters():
    """Non-default constants reach the compiled restatement."""
    agree(g.sos_hankel(8, seed=3), step=o.EigenStep(tau=0.9), centering=o.Mehrotra(sigma_exponent=2.0))
    agree(g.sos_hankel(8, seed=3), rtol=1e-7, iter_tol=1, step=o.CholeskyBacktrack(shrink=0.5, boundary=0.9),
          centering=o.AdaptiveMu(initial_ratio=0.5, ratio=0.3))


def test_unsupported_component_rejected():
    with pytest.raises(ValueError):
        cpu_ipm.solve(build("trivial_2x2"), direction="XYZ")


def test_max_iter_status():
    c = agree(g.sos_hankel(9, seed=1), max_iter=3)
    assert c["status"] == int(o.Status.MAXIMUM_ITERATIONS_EXCEEDED) and c["iter"] == 3


def test_solve_many_matches_solve():
    models = [g.sos_hankel(d, seed=d) for d in (5, 6, 7, 8, 9, 10)] + [build("mixed_lp")]
    many = cpu_ipm.solve_many(models, threads=3)
    for m, s in zip(models, many):
        one = cpu_ipm.solve(m)
        assert s["status"] == one["status"] and s["iter"] == one["iter"] and s["pobj"] == one["pobj"]
    part = cpu_ipm.solve_many(cpu_ipm.Prepared(models), threads=2, start=2, count=3)
    assert [s["pobj"] for s in part] == [s["pobj"] for s in many[2:5]]


def test_invalid_index_rejected():
    m = build("trivial_2x2")
    m.A[0].row[0] = 7  # outside the 2 x 2 block
    with pytest.raises(ValueError):
        cpu_ipm.solve(m)


@pytest.mark.parametrize("kind", ["random", "repeated", "diagonal", "zero", "one", "tridiagonal", "graded"])
def test_symeig(kind):
    rng = np.random.default_rng(5)
    n = 24
    if kind == "random":
        A = rng.standard_normal((n, n))
        A = A + A.T
    elif kind == "repeated":
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        A = Q @ np.diag(np.repeat([1.0, -2.0, 3.0], n // 3)) @ Q.T
    elif kind == "diagonal":
        A = np.diag(rng.standard_normal(n))
    elif kind == "zero":
        A = np.zeros((n, n))
    elif kind == "one":
        A = np.array([[2.5]])
    elif kind == "tridiagonal":
        A = np.diag(np.full(n, 2.0)) - np.diag(np.ones(n - 1), 1) - np.diag(np.ones(n - 1), -1)
    else:
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        A = Q @ np.diag(np.logspace(-12, 3, n)) @ Q.T
    A = (A + A.T) / 2
    w, V = cpu_ipm.symeig(A)
    k = A.shape[0]
    scale = max(1.0, np.abs(A).max())
    assert np.all(np.diff(w) >= 0)
    assert np.max(np.abs(w - np.linalg.eigvalsh(A))) <= 1e-12 * scale * k
    assert np.max(np.abs(V.T @ V - np.eye(k))) <= 1e-12 * k
    assert np.max(np.abs(V @ np.diag(w) @ V.T - A)) <= 1e-12 * scale * k


def test_defaults_equal_the_gpu_library_defaults():
    """The compiled restatement starts from the same components and options
    as the GPU library (both mirror src/components.jl and src/options.jl)."""
    import ctypes as C

    from madsdp_gpu import _lib as G
    gpu, cpu = G.load(), cpu_ipm.load()
    for struct, gfun, cfun in ((G.Components, gpu.msdp_default_components, cpu.msdp_cpu_default_components),
                               (G.Options, gpu.msdp_default_options, cpu.msdp_cpu_default_options)):
        a, b = struct(), struct()
        gfun(C.byref(a))
        cfun(C.byref(b))
        for name, _ in struct._fields_:
            va, vb = getattr(a, name), getattr(b, name)
            assert va == vb or (va != va and vb != vb), (struct.__name__, name, va, vb)
