"""Continuous-batching serving over the C ABI (msdp_server_*).

``Server`` admits requests into a fixed device-memory budget and advances
every active request a few iterations per launch; ``serve_stream`` replays a
timed request stream in real time and reports latency percentiles and
throughput.  ``poisson_stream`` draws the mixed request stream of the
serving workload (SOS, max-cut and dense SDPs) from a seed.
"""

from __future__ import annotations

import ctypes as C
import threading
import time
from collections import deque
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib, generators as g
from .components import DenseCholesky, EigenStep, Mehrotra, NT, Options, PrimalDual, ScaledIdentity, Status
from .model import Model
from .solver import (Context, InstanceSolver, _Marshalled, _components, _options, _ptr, _stats_dict,
                     default_context)

__all__ = ["Server", "poisson_stream", "serve_stream", "instance_bytes_estimate", "serve_whole_gpu"]

LARGE_ID0 = 1 << 40  # request ids of whole-GPU requests start here


def serve_whole_gpu(model: Model, batch_max_side: int = 128) -> bool:
    """Whether a served request takes a whole-GPU slot.  For throughput the
    rule is wider than MadSDPSolver's single-problem rule (blocks above 64):
    a request whose blocks are at most `batch_max_side` and whose m is at
    most 300 runs in the batched waves, one thread block among hundreds
    resident at once, which serves many such requests at a time where a
    whole-GPU solve of one of them leaves most of the GPU idle."""
    return max(model.sides, default=0) > batch_max_side or model.m > 300


def instance_bytes_estimate(model: Model) -> int:
    """Device bytes of the whole-GPU solver for `model` (its allocations at
    creation: block matrices, tensor-core operand slices, Schur matrices,
    and for dense constraint blocks the constraint data, its slices and the
    assembly's operands)."""
    m = model.m
    nmax = max(model.sides, default=1)
    b = 8 * (19 * sum(n * n for n in model.sides) + 2 * m * m + max(nmax * nmax, m * m) + 8 * m)
    b += 28 * (nmax + 128) * (nmax + 32)
    if nmax > 128:
        b += 8 * nmax * (min(nmax, 320) + 1)
    for n, A in zip(model.sides, model.A):
        if A.nnz >= m * n * n // 2:
            b += (24 + 14 + 14 + 7) * m * n * n + 128 * n * n
    return int(b)


class _WholeGPURequests:
    """Requests too large for one thread block, each solved on the whole GPU
    (InstanceSolver) by one of `slots` worker threads.  Every worker owns a
    context (its own stream), so these solves overlap on the device with
    each other and with the batched waves; they are started in arrival order
    while the estimated device bytes of the running solves fit
    `memory_budget_bytes` (one runs regardless when none is running)."""

    def __init__(self, slots: int, memory_budget_bytes: int, device: int, kwargs: dict):
        self.kwargs = kwargs
        self.budget = int(memory_budget_bytes)
        self.cv = threading.Condition()
        self.queue = deque()           # (rid, model, estimate)
        self.running: Dict[int, int] = {}
        self.results: Dict[int, dict] = {}
        self.done: List[int] = []
        self.used = 0
        self.stop = False
        self.error: Optional[BaseException] = None
        self.threads = [threading.Thread(target=self._work, args=(device,), daemon=True) for _ in range(slots)]
        for t in self.threads:
            t.start()

    def submit(self, rid: int, model: Model):
        with self.cv:
            self.queue.append((rid, model, instance_bytes_estimate(model)))
            self.cv.notify_all()

    def _next(self):
        # called with the lock held: the head of the queue when it fits
        if self.queue and (not self.running or self.used + self.queue[0][2] <= self.budget):
            rid, model, est = self.queue.popleft()
            self.running[rid] = est
            self.used += est
            return rid, model
        return None

    def _work(self, device: int):
        ctx = Context(device)
        while True:
            with self.cv:
                job = None
                while not self.stop and job is None:
                    job = self._next()
                    if job is None:
                        self.cv.wait(0.05)
                if self.stop:
                    return
            rid, model = job
            try:
                s = InstanceSolver(model, context=ctx, **self.kwargs)
                s.solve()
                st = s.stats()
                X, y, x, z = s.solution()
                s.close()
                res = dict(st)
                res.update(X=X, y=y, x=x, z=z, finish=time.perf_counter())
            except BaseException as e:  # surfaced by the owning server
                res = None
                with self.cv:
                    self.error = e
            with self.cv:
                self.used -= self.running.pop(rid)
                if res is not None:
                    self.results[rid] = res
                    self.done.append(rid)
                self.cv.notify_all()

    def counts(self) -> Tuple[int, int]:
        with self.cv:
            if self.error is not None:
                raise RuntimeError(f"whole-GPU request failed: {self.error!r}")
            return len(self.queue), len(self.running)

    def finished(self) -> List[int]:
        with self.cv:
            out, self.done = self.done, []
            return out

    def close(self):
        with self.cv:
            self.stop = True
            self.cv.notify_all()
        for t in self.threads:
            t.join()


class Server:
    """A continuous-batching solve server on one GPU (msdp_server).

    `whole_gpu_slots` > 0 adds a slot type for requests too large for the
    batched waves (`serve_whole_gpu`: a block above `batch_max_side` or more
    than 300 constraints): they are solved by that many concurrent
    whole-GPU solvers, admitted by `whole_gpu_memory_bytes`, beside the
    batched waves.  They run in `whole_gpu_precision` (FP64 by default: on
    the whole GPU the FP64 products are tensor-core products already, and
    the split-precision Schur solve with refinement measured slower; None
    takes `precision`)."""

    def __init__(self, memory_budget_bytes: int = 1 << 30, max_slots: int = 1024, direction=None,
                 step=None, centering=None, initial_point=None, schur=None, precision: str = "fp64",
                 context: Optional[Context] = None, whole_gpu_slots: int = 0,
                 whole_gpu_memory_bytes: int = 16 << 30, batch_max_side: int = 128,
                 whole_gpu_precision: Optional[str] = "fp64", **options):
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
        self.large = None
        self.batch_max_side = int(batch_max_side)
        self._next_large = LARGE_ID0
        if whole_gpu_slots > 0:
            kw = dict(direction=alg.direction, step=alg.step, centering=alg.centering,
                      initial_point=initial_point or ScaledIdentity(), schur=schur or DenseCholesky(),
                      precision=whole_gpu_precision or precision, **options)
            self.large = _WholeGPURequests(whole_gpu_slots, whole_gpu_memory_bytes, self.ctx.device, kw)
        self.ctx.adopt(self)

    def close(self):
        if getattr(self, "large", None) is not None:
            self.large.close()
            self.large = None
        if getattr(self, "h", None):
            self.lib.msdp_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, model: Model) -> int:
        if self.large is not None and serve_whole_gpu(model, self.batch_max_side):
            rid = self._next_large
            self._next_large += 1
            self.models[rid] = model
            self.large.submit(rid, model)
            return rid
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
        if self.large is not None:
            p, a, _ = self._batched_counts()
            if p == 0 and a == 0:
                time.sleep(5e-4)  # only whole-GPU requests are running (in their threads)
                return 0, 0
        act, done = C.c_int32(), C.c_int32()
        if budget_s > 0:
            rc = self.lib.msdp_server_step_budget(self.h, int(iterations), float(budget_s), C.byref(act),
                                                  C.byref(done))
        else:
            rc = self.lib.msdp_server_step(self.h, int(iterations), C.byref(act), C.byref(done))
        if rc != 0:
            raise RuntimeError(f"msdp_server_step: {_lib.ERRORS.get(rc, rc)}")
        return act.value, done.value

    def _batched_counts(self) -> Tuple[int, int, int]:
        p, a, c = C.c_int32(), C.c_int32(), C.c_int64()
        self.lib.msdp_server_counts(self.h, C.byref(p), C.byref(a), C.byref(c))
        return p.value, a.value, c.value

    def counts(self) -> Tuple[int, int, int]:
        """(pending, active, completed) over both slot types."""
        p, a, c = self._batched_counts()
        if self.large is not None:
            lp, la = self.large.counts()
            p, a = p + lp, a + la
            c += len(self.large.results)
        return p, a, c

    @property
    def launch_count(self) -> int:
        return int(self.lib.msdp_server_launch_count(self.h))

    def result(self, rid: int) -> Optional[dict]:
        """The finished request's stats and solution, or None if still running."""
        if rid >= LARGE_ID0:
            with self.large.cv:
                r = self.large.results.pop(rid, None)
            if r is None:
                return None
            del self.models[rid]
            return r
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
        out: List[int] = [] if self.large is None else self.large.finished()
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


def _dense_request(rng, nmin: int, nmax: int, mmax: int, seed: int, mmin: int = 10) -> Model:
    n = int(rng.integers(nmin, nmax + 1))
    cap = n * (n + 1) // 2
    m = int(rng.integers(min(mmin, cap), min(mmax, cap) + 1))
    return g.dense_random([n], 0, m, seed=seed)


def poisson_stream(rate: float, duration: float, seed: int = 0, sos_d=(5, 63), maxcut_n=(20, 64),
                   dense_n=(8, 24), dense_m=60, dense_m_min: int = 10,
                   dense_pool: Optional[int] = None) -> List[Tuple[float, str, Model]]:
    """(arrival time, kind, model) for Poisson arrivals at `rate` per second.

    The mix is 50% SOS lower bounds (Gram side d+1, d ~ U(sos_d)), 30% max-cut
    (n ~ U(maxcut_n), edge probability 4/n) and 20% random dense SDPs (one
    block n ~ U(dense_n), m ~ U(dense_m_min, dense_m) capped at n(n+1)/2, no
    scalars; the cap keeps the constraint map of full rank).

    dense_pool = K draws the dense requests from K models generated up front
    with that distribution (each arrival picks one at random): a dense
    request with n = 256 and m = 3000 holds about 1.5 GB of constraint data,
    so a stream of hundreds of distinct ones does not fit host memory.
    """
    rng = np.random.default_rng(seed)
    pool = None
    if dense_pool:
        prng = np.random.default_rng(seed + 7919)
        pool = [_dense_request(prng, dense_n[0], dense_n[1], dense_m, seed * 1000003 + 999000 + k, dense_m_min)
                for k in range(dense_pool)]
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
            if pool is not None:
                out.append((t, "dense", pool[int(rng.integers(len(pool)))]))
            else:
                out.append((t, "dense", _dense_request(rng, dense_n[0], dense_n[1], dense_m, s, dense_m_min)))
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
