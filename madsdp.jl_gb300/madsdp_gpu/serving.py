"""Continuous-batching serving over the C ABI (msdp_server_*).

``Server`` admits requests into a fixed device-memory budget and advances
every active request a few iterations per launch; ``serve_stream`` replays a
timed request stream in real time and reports latency percentiles and
throughput.  ``poisson_stream`` draws the mixed request stream of the
serving workload (SOS, max-cut and dense SDPs) from a seed.
"""

from __future__ import annotations

import ctypes as C
import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib, generators as g
from .components import DenseCholesky, EigenStep, Mehrotra, NT, Options, PrimalDual, ScaledIdentity, Status
from .model import Model
from .solver import Context, _Marshalled, _components, _options, _ptr, _stats_dict, default_context

__all__ = ["Server", "poisson_stream", "serve_stream"]


class Server:
    """A continuous-batching solve server on one GPU (msdp_server)."""

    def __init__(self, memory_budget_bytes: int = 1 << 30, max_slots: int = 1024, direction=None,
                 step=None, centering=None, initial_point=None, schur=None, precision: str = "fp64",
                 context: Optional[Context] = None, **options):
        self.ctx = context or default_context()
        self.lib = self.ctx.lib
        alg = PrimalDual(direction or NT(), step or EigenStep(), centering or Mehrotra())
        comp = _components(alg, initial_point or ScaledIdentity(), schur or DenseCholesky(), precision)
        self.opt = Options(**options)
        opts = _options(self.opt)
        h = C.c_void_p()
        rc = self.lib.msdp_server_create(self.ctx.h, C.byref(comp), C.byref(opts), int(memory_budget_bytes),
                                         int(max_slots), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"msdp_server_create failed: {_lib.ERRORS.get(rc, rc)}")
        self.h = h
        self.models: Dict[int, Model] = {}
        self.ctx.adopt(self)

    def close(self):
        if getattr(self, "h", None):
            self.lib.msdp_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, model: Model) -> int:
        mm = _Marshalled(model)
        rid = C.c_int64()
        rc = self.lib.msdp_server_submit(self.h, C.byref(mm.desc), C.byref(rid))
        if rc != 0:
            raise ValueError(f"msdp_server_submit: {_lib.ERRORS.get(rc, rc)}")
        self.models[rid.value] = model
        return rid.value

    def step(self, iterations: int = 2, budget_s: float = 0.0) -> Tuple[int, int]:
        """budget_s = 0: one synchronous wave (admit, initialize newcomers,
        `iterations` iterations per active request).  budget_s > 0: collect
        finished waves and start a wave over the idle requests on a free
        stream without waiting (waves overlap on the GPU); each request of
        a wave runs until the wave has lasted budget_s and every request
        of it has iterated once."""
        act, done = C.c_int32(), C.c_int32()
        if budget_s > 0:
            rc = self.lib.msdp_server_step_budget(self.h, int(iterations), float(budget_s), C.byref(act),
                                                  C.byref(done))
        else:
            rc = self.lib.msdp_server_step(self.h, int(iterations), C.byref(act), C.byref(done))
        if rc != 0:
            raise RuntimeError(f"msdp_server_step: {_lib.ERRORS.get(rc, rc)}")
        return act.value, done.value

    def counts(self) -> Tuple[int, int, int]:
        p, a, c = C.c_int32(), C.c_int32(), C.c_int64()
        self.lib.msdp_server_counts(self.h, C.byref(p), C.byref(a), C.byref(c))
        return p.value, a.value, c.value

    @property
    def launch_count(self) -> int:
        return int(self.lib.msdp_server_launch_count(self.h))

    def result(self, rid: int) -> Optional[dict]:
        """The finished request's stats and solution, or None if still running."""
        model = self.models[rid]
        X = [np.zeros((n, n), order="F") for n in model.sides]
        Xp = (C.POINTER(C.c_double) * max(len(X), 1))(*[_ptr(a) for a in X])
        y, x, z = np.zeros(model.m), np.zeros(model.ns), np.zeros(model.ns)
        st = _lib.Stats()
        lat = C.c_double()
        rc = self.lib.msdp_server_result(self.h, int(rid), C.byref(st), Xp, _ptr(y), _ptr(x), _ptr(z), C.byref(lat))
        if rc == 1:
            return None
        if rc != 0:
            raise ValueError(f"msdp_server_result: {_lib.ERRORS.get(rc, rc)}")
        del self.models[rid]
        out = _stats_dict(st)
        out.update(X=[np.ascontiguousarray(a) for a in X], y=y, x=x, z=z, latency_s=lat.value)
        return out

    def finished(self, capacity: int = 4096) -> List[int]:
        """Ids of requests finished since the last call, each reported once."""
        out: List[int] = []
        buf = (C.c_int64 * capacity)()
        cnt = C.c_int32()
        while True:
            rc = self.lib.msdp_server_finished(self.h, buf, capacity, C.byref(cnt))
            if rc != 0:
                raise RuntimeError(f"msdp_server_finished: {_lib.ERRORS.get(rc, rc)}")
            out.extend(buf[: cnt.value])
            if cnt.value < capacity:
                return out

    def drain(self, iterations: int = 2, max_steps: int = 1000000, budget_s: float = 0.0) -> None:
        """Step until nothing is pending or active (with budget_s > 0 the
        waves run asynchronously and this polls them)."""
        for _ in range(max_steps):
            p, a, _ = self.counts()
            if p == 0 and a == 0:
                return
            self.step(iterations, budget_s)
            if budget_s > 0:
                time.sleep(1e-4)
        raise RuntimeError("server did not drain")


def _dense_request(rng, nmin: int, nmax: int, mmax: int, seed: int) -> Model:
    n = int(rng.integers(nmin, nmax + 1))
    m = int(rng.integers(min(10, n * (n + 1) // 2), min(mmax, n * (n + 1) // 2) + 1))
    return g.dense_random([n], 0, m, seed=seed)


def poisson_stream(rate: float, duration: float, seed: int = 0, sos_d=(5, 63), maxcut_n=(20, 64),
                   dense_n=(8, 24), dense_m=60) -> List[Tuple[float, str, Model]]:
    """(arrival time, kind, model) for Poisson arrivals at `rate` per second.

    The mix is 50% SOS lower bounds (Gram side d+1, d ~ U(sos_d)), 30% max-cut
    (n ~ U(maxcut_n), edge probability 4/n) and 20% random dense SDPs (one
    block n ~ U(dense_n), m <= min(dense_m, n(n+1)/2), no scalars; m is capped
    because larger m makes the constraint map rank-deficient).
    """
    rng = np.random.default_rng(seed)
    t, out, k = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        u = rng.random()
        s = seed * 1000003 + k
        if u < 0.5:
            out.append((t, "sos", g.sos_hankel(int(rng.integers(sos_d[0], sos_d[1] + 1)), seed=s)))
        elif u < 0.8:
            n = int(rng.integers(maxcut_n[0], maxcut_n[1] + 1))
            out.append((t, "maxcut", g.maxcut(n, min(1.0, 4.0 / n), seed=s)))
        else:
            out.append((t, "dense", _dense_request(rng, dense_n[0], dense_n[1], dense_m, s)))
        k += 1
    return out


def serve_stream(server: Server, stream: Sequence[Tuple[float, str, Model]], iterations: int = 2,
                 time_limit: float = 600.0, budget_s: float = 0.0) -> dict:
    """Replay `stream` in real time: requests are submitted when their arrival
    time has passed, the server steps continuously (waves of `iterations`
    iterations, time-sliced by `budget_s` when positive).  Latency = finish
    time - arrival time (host clock)."""
    t0 = time.perf_counter()
    nxt, ids = 0, {}
    lat, kinds, statuses = [], [], []
    while True:
        now = time.perf_counter() - t0
        while nxt < len(stream) and stream[nxt][0] <= now:
            ids[server.submit(stream[nxt][2])] = (stream[nxt][0], stream[nxt][1])
            nxt += 1
        p, a, _ = server.counts()
        if p or a:
            server.step(iterations, budget_s)
        elif nxt < len(stream):
            time.sleep(min(0.002, max(0.0, stream[nxt][0] - now)))
        t_after = time.perf_counter() - t0
        fin = server.finished()
        if not fin and (p or a) and budget_s > 0:
            time.sleep(2e-4)  # waves are running; poll again shortly
        for rid in fin:
            r = server.result(rid)
            arr, kind = ids.pop(rid)
            lat.append(t_after - arr)
            kinds.append(kind)
            statuses.append(r["status"])
        if nxt >= len(stream) and not ids:
            break
        if t_after > time_limit:
            raise RuntimeError("serving did not finish within the time limit")
    wall = time.perf_counter() - t0
    lat = np.array(lat)
    by_kind = {}
    for k, st, l in zip(kinds, statuses, lat):
        d = by_kind.setdefault(k, {"n": 0, "succeeded": 0, "lat": []})
        d["n"] += 1
        d["succeeded"] += int(st == Status.SOLVE_SUCCEEDED)
        d["lat"].append(l)
    per_kind = {k: {"requests": d["n"], "succeeded": d["succeeded"],
                    "p50_latency_ms": float(np.percentile(d["lat"], 50) * 1e3),
                    "p99_latency_ms": float(np.percentile(d["lat"], 99) * 1e3)} for k, d in by_kind.items()}
    return {
        "requests": len(stream), "completed": len(lat), "wall_s": wall,
        "solves_per_s": len(lat) / wall,
        "p50_latency_ms": float(np.percentile(lat, 50) * 1e3) if len(lat) else None,
        "p99_latency_ms": float(np.percentile(lat, 99) * 1e3) if len(lat) else None,
        "succeeded": int(sum(1 for s in statuses if s == Status.SOLVE_SUCCEEDED)),
        "launches": server.launch_count,
        "per_kind": per_kind,
        "statuses": {str(k): int(v) for k, v in zip(*np.unique([int(x) for x in statuses], return_counts=True))}
        if statuses else {},
    }
