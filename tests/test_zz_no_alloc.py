"""msdp_solve_static: the entry point for callers that may not allocate
device memory (a runtime or plugin host that owns all GPU memory through its
own pool, or a loop that must not risk an allocation).  It must give the
same result as the allocating entry point (msdp_batch_create +
msdp_batch_solve) within the tolerance of the other parity tests, on two
calls in a row (the static scratch array is reused and re-zeroed).

It is also checked directly against the oracle, on entries that arrive in
any order, for the property it exists for (a repeat call allocates no device
memory) and for its argument checks.

Collected last on purpose; it also passes alone in a fresh process."""
import copy
import ctypes as C

import numpy as np
import pytest

import madsdp_gpu as M
from madsdp_gpu import _lib, generators as g
from madsdp_gpu.solver import _Marshalled, _components, _options, _ptr

pytestmark = pytest.mark.gpu


def static_status(model):
    lib = _lib.load()
    mm = _Marshalled(model)
    st = _lib.Stats()
    return lib.msdp_solve_static(C.byref(mm.desc), None, None, None, None, None, None, None, C.byref(st))


def static_solve(model):
    lib = _lib.load()
    mm = _Marshalled(model)
    comp = _components(M.PrimalDual(), M.ScaledIdentity(), M.DenseCholesky(), "fp64")
    opts = _options(M.Options())
    X = [np.zeros((n, n), order="F") for n in model.sides]
    Xp = (C.POINTER(C.c_double) * max(len(X), 1))(*[_ptr(a) for a in X])
    y, x, z = np.zeros(model.m), np.zeros(model.ns), np.zeros(model.ns)
    st = _lib.Stats()
    rc = lib.msdp_solve_static(C.byref(mm.desc), C.byref(comp), C.byref(opts), None, Xp, _ptr(y),
                               _ptr(x) if model.ns else None, _ptr(z) if model.ns else None, C.byref(st))
    assert rc == 0, _lib.ERRORS.get(rc, rc)
    return st, [np.ascontiguousarray(a) for a in X], y, x, z


@pytest.mark.parametrize("model", [g.sos_hankel(9, seed=11), g.maxcut(24, 0.3, seed=5), g.mixed_lp_example(),
                                   g.dense_random([5, 3], 2, 8, seed=4)], ids=["sos", "maxcut", "mixed_lp", "dense"])
def test_static_matches_batch_entry_point(gpu_ctx, model):
    ref = M.Batch([model])
    ref.solve()
    rs = ref.all_stats()[0]
    rX, ry, rx, rz = ref.solution(0)
    assert rs["status"] == M.Status.SOLVE_SUCCEEDED
    scale = max(1.0, abs(rs["pobj"]) + abs(rs["dobj"]))
    for call in range(2):
        st, X, y, x, z = static_solve(model)
        assert st.status == M.Status.SOLVE_SUCCEEDED, call
        assert abs(st.iter - rs["iter"]) <= 1
        assert abs(st.pobj - rs["pobj"]) <= 1e-7 * scale
        assert abs(st.dobj - rs["dobj"]) <= 1e-7 * scale
        assert max(st.inf_pr, st.inf_du, st.gap) <= 1e-7
        for a, b in zip(X, rX):
            assert np.allclose(a, b, atol=1e-6 * max(1.0, np.abs(b).max()))


def test_static_rejects_oversize(gpu_ctx):
    big = g.maxcut(300, 0.02, seed=1)   # 300^2 workspaces exceed the static array
    lib = _lib.load()
    mm = _Marshalled(big)
    st = _lib.Stats()
    rc = lib.msdp_solve_static(C.byref(mm.desc), None, None, None, None, None, None, None, C.byref(st))
    assert rc == -6


def test_static_matches_oracle(gpu_ctx):
    from oracle import madsdp_oracle as o
    model = g.sos_hankel(11, seed=3)
    ref = o.Solver(model).solve()
    st, X, y, x, z = static_solve(model)
    assert st.status == M.Status.SOLVE_SUCCEEDED
    scale = max(1.0, abs(ref.primal_objective()) + abs(ref.dual_objective()))
    assert abs(st.iter - ref.iter) <= 1
    assert abs(st.pobj - ref.primal_objective()) <= 1e-7 * scale
    assert abs(st.dobj - ref.dual_objective()) <= 1e-7 * scale


def test_static_entry_order_does_not_matter(gpu_ctx):
    """The entries of a constraint list may arrive in any order: the device
    staging orders them, so the result equals the batch path's."""
    model = g.dense_random([5, 3], 2, 8, seed=4)
    ref = M.Batch([model])
    ref.solve()
    rs = ref.all_stats()[0]
    shuffled = copy.deepcopy(model)
    rng = np.random.default_rng(0)
    for blk in shuffled.A:
        perm = rng.permutation(blk.nnz)
        blk.con, blk.row, blk.col = blk.con[perm].copy(), blk.row[perm].copy(), blk.col[perm].copy()
        blk.val = blk.val[perm].copy()
    st, X, y, x, z = static_solve(shuffled)
    scale = max(1.0, abs(rs["pobj"]) + abs(rs["dobj"]))
    assert st.status == M.Status.SOLVE_SUCCEEDED
    assert abs(st.pobj - rs["pobj"]) <= 1e-7 * scale
    assert abs(st.dobj - rs["dobj"]) <= 1e-7 * scale


def test_static_repeat_call_allocates_nothing(gpu_ctx):
    import torch
    model = g.maxcut(20, 0.3, seed=8)
    static_solve(model)            # first call: per-device set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    static_solve(model)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_static_rejects_out_of_range_entries(gpu_ctx):
    model = copy.deepcopy(g.maxcut(10, 0.3, seed=2))
    blk = model.A[0]
    blk.con = blk.con.copy()
    blk.con[0] = model.m            # constraint index past m
    assert static_status(model) == -1
