"""Continuous-batching server (msdp_server_*): a request's result does not
depend on what else is on the GPU, on when it was admitted, or on how many
iterations each wave runs."""

import numpy as np
import pytest

import madsdp_gpu as M
from madsdp_gpu import generators as g
from madsdp_gpu.serving import Server, poisson_stream, serve_stream

pytestmark = pytest.mark.gpu


def mixed_requests():
    return [g.sos_hankel(9, seed=11), g.maxcut(24, 0.2, seed=4), g.dense_random([7], 0, 12, seed=3),
            g.sos_hankel(30, seed=12), g.dense_random([6, 4], 3, 10, seed=2), g.maxcut(40, 0.1, seed=5),
            g.sos_hankel(5, seed=13), g.dense_random([12], 0, 40, seed=8)]


def alone(model, **kw):
    bt = M.Batch([model], **kw)
    bt.solve()
    X, y, x, z = bt.solution(0)
    return bt.all_stats()[0], X, y


def assert_same(r, st, X, y):
    assert r["status"] == st["status"]
    assert r["iter"] == st["iter"]
    scale = max(1.0, abs(st["pobj"]) + abs(st["dobj"]))
    assert abs(r["pobj"] - st["pobj"]) <= 1e-12 * scale
    assert abs(r["dobj"] - st["dobj"]) <= 1e-12 * scale
    for a, b in zip(r["X"], X):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-10 * max(1.0, np.abs(b).max()))
    np.testing.assert_allclose(r["y"], y, rtol=0, atol=1e-10 * max(1.0, np.abs(y).max()))


def test_server_matches_solving_alone(gpu_ctx):
    """Requests arrive two per wave while earlier ones are mid-solve."""
    models = mixed_requests()
    srv = Server(memory_budget_bytes=64 << 20, max_slots=16)
    ids = []
    for k in range(0, len(models), 2):
        ids += [srv.submit(models[k]), srv.submit(models[k + 1])]
        srv.step(3)
    srv.drain(3)
    assert srv.counts()[2] == len(models)
    assert sorted(srv.finished()) == sorted(ids) and srv.finished() == []
    for rid, m in zip(ids, models):
        r = srv.result(rid)
        assert r is not None and r["latency_s"] > 0
        st, X, y = alone(m)
        assert st["status"] == M.Status.SOLVE_SUCCEEDED
        assert_same(r, st, X, y)
    srv.close()


@pytest.mark.parametrize("iterations,budget_s", [(1, 0.0), (7, 0.0), (1000, 0.002)])
def test_server_wave_length_does_not_change_results(gpu_ctx, iterations, budget_s):
    models = mixed_requests()[:4]
    srv = Server(memory_budget_bytes=32 << 20, max_slots=8)
    ids = [srv.submit(m) for m in models]
    srv.drain(iterations, budget_s=budget_s)
    for rid, m in zip(ids, models):
        st, X, y = alone(m)
        assert_same(srv.result(rid), st, X, y)


def test_server_admits_by_memory(gpu_ctx):
    """With room for two SOS(63) regions, five requests run at most two at a
    time, in arrival order, and all finish with the same answers."""
    models = [g.sos_hankel(63, seed=20 + i) for i in range(5)]
    srv = Server(memory_budget_bytes=3 << 20, max_slots=8)
    ids = [srv.submit(m) for m in models]
    assert srv.result(ids[0]) is None
    srv.step(2)
    pending, active, _ = srv.counts()
    assert 1 <= active <= 2 and pending == 5 - active
    seen_max = active
    for _ in range(1000):
        p, a, _ = srv.counts()
        if p == 0 and a == 0:
            break
        srv.step(2)
        seen_max = max(seen_max, srv.counts()[1])
    assert seen_max <= 2
    for rid, m in zip(ids, models):
        st, X, y = alone(m)
        assert_same(srv.result(rid), st, X, y)


def test_server_rejects_oversize_and_bad_options(gpu_ctx):
    srv = Server(memory_budget_bytes=1 << 20, max_slots=2)
    with pytest.raises(ValueError, match="TOO_LARGE"):
        srv.submit(g.sos_hankel(63, seed=1))
    srv.close()
    with pytest.raises(RuntimeError):
        Server(memory_budget_bytes=0)


def test_server_mixed_precision(gpu_ctx):
    models = [g.sos_hankel(int(d), seed=40 + i) for i, d in enumerate([6, 18, 33, 47])]
    srv = Server(memory_budget_bytes=64 << 20, max_slots=8, precision="mixed")
    ids = [srv.submit(m) for m in models]
    srv.drain(2)
    for rid, m in zip(ids, models):
        r = srv.result(rid)
        st, X, y = alone(m, precision="mixed")
        assert r["iter_fp32"] == st["iter_fp32"] and r["iter_fp32"] >= 1
        assert_same(r, st, X, y)


def test_serve_poisson_stream(gpu_ctx):
    stream = poisson_stream(rate=400.0, duration=0.1, seed=3, sos_d=(5, 20), maxcut_n=(20, 30), dense_n=(6, 10))
    srv = Server(memory_budget_bytes=256 << 20, max_slots=64)
    out = serve_stream(srv, stream, iterations=1000, time_limit=120.0, budget_s=0.005)
    assert out["completed"] == out["requests"] == len(stream) > 0
    assert out["succeeded"] == out["completed"]
    assert out["p99_latency_ms"] >= out["p50_latency_ms"] > 0


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-7), ("mixed", 1e-7)])
def test_served_mix_matches_oracle(gpu_ctx, precision, rtol):
    """Every request of a served Poisson stream with the compact mix
    (SOS d <= 127, max-cut n <= 100, dense n <= 32 with m <= 200) converges
    and agrees with the compiled oracle: objectives within
    rtol * max(1, |p| + |d|) (the FP64 and mixed tolerances of the batch
    parity tests)."""
    import os

    import bench
    from oracle import cpu_ipm
    stream = poisson_stream(40.0, 1.5, seed=23, **bench.SERVE_MIXES["compact"])
    models = [m for _, _, m in stream]
    ref = cpu_ipm.solve_many(models, threads=os.cpu_count() or 1)
    srv = Server(memory_budget_bytes=2 << 30, max_slots=256, precision=precision)
    ids = [srv.submit(m) for m in models]
    srv.drain(50)
    kinds = [k for _, k, _ in stream]
    for rid, kind, r in zip(ids, kinds, ref):
        s = srv.result(rid)
        assert r["status"] == 1
        assert s["status"] == M.Status.SOLVE_SUCCEEDED, (rid, kind, s["status"])
        scale = max(1.0, abs(r["pobj"]) + abs(r["dobj"]))
        assert abs(s["pobj"] - r["pobj"]) <= rtol * scale, (rid, kind, s["pobj"], r["pobj"])
    srv.close()


def test_whole_gpu_requests_same_alone_and_in_the_mix(gpu_ctx):
    """Requests above one thread block (a max-cut with n = 300, a dense
    block of 120 with m = 600) are served by the whole-GPU slot type while
    small ones run in batched waves, all at once and overlapping on the GPU;
    every result equals solving the request alone (small: a one-problem
    batch; large: the whole-GPU solver)."""
    small = mixed_requests()[:4]
    large = [g.maxcut(300, 4.0 / 300, seed=21), g.dense_random([120], 0, 600, seed=22)]
    srv = Server(memory_budget_bytes=64 << 20, max_slots=16, whole_gpu_slots=2)
    ids = [srv.submit(m) for m in small[:2]] + [srv.submit(m) for m in large] + [srv.submit(m) for m in small[2:]]
    models = small[:2] + large + small[2:]
    srv.drain(3, budget_s=0.002)
    assert srv.counts()[:2] == (0, 0)
    assert sorted(srv.finished()) == sorted(ids)
    for rid, m in zip(ids, models):
        r = srv.result(rid)
        assert r is not None
        if m in large:
            s = M.InstanceSolver(m).solve()
            st = s.stats()
            X, y, _, _ = s.solution()
            s.close()
        else:
            st, X, y = alone(m)
        assert st["status"] == M.Status.SOLVE_SUCCEEDED
        assert_same(r, st, X, y)
    srv.close()


def test_served_stated_mix_subsample_matches_oracle(gpu_ctx):
    """The serving workload's stated mix (SOS d <= 127, max-cut n in
    [50, 800], dense n in [32, 256] with m in [100, 3000]) through the server
    with whole-GPU slots for the large requests, in mixed precision: the
    requests of a seeded stream that the compiled oracle solves in seconds
    (max-cut n <= 400, dense m n^2 <= 2e7) are served together; each
    converges and agrees with the oracle to 1e-7 * max(1, |p| + |d|)."""
    import os

    import bench
    from madsdp_gpu.serving import serve_whole_gpu
    from oracle import cpu_ipm
    stream = poisson_stream(200.0, 0.5, seed=29, **bench.SERVE_MIXES["stated"])

    def cheap(kind, m):
        if kind == "maxcut":
            return m.sides[0] <= 400
        if kind == "dense":
            return m.m * m.sides[0] ** 2 <= 2e7
        return True

    keep = [(k, m) for _, k, m in stream if cheap(k, m)][:24]
    kinds = [k for k, _ in keep]
    models = [m for _, m in keep]
    large = [serve_whole_gpu(m) for m in models]
    assert any(l and k == "maxcut" for k, l in zip(kinds, large))
    assert any(l and k == "dense" for k, l in zip(kinds, large))
    ref = cpu_ipm.solve_many(models, threads=os.cpu_count() or 1)
    srv = Server(memory_budget_bytes=2 << 30, max_slots=256, precision="mixed", whole_gpu_slots=2)
    ids = [srv.submit(m) for m in models]
    srv.drain(50, budget_s=0.005)
    for rid, kind, r in zip(ids, kinds, ref):
        s = srv.result(rid)
        assert r["status"] == 1
        assert s["status"] == M.Status.SOLVE_SUCCEEDED, (rid, kind, s["status"])
        scale = max(1.0, abs(r["pobj"]) + abs(r["dobj"]))
        assert abs(s["pobj"] - r["pobj"]) <= 1e-7 * scale, (rid, kind, s["pobj"], r["pobj"])
    srv.close()
