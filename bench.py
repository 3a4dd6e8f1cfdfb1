#!/usr/bin/env python
"""Benchmark: SDP solves/sec + p50/p99 latency at 1e-7 gap on GB300.

Workload (one "step" = one batched solve of every instance to termination):
4096 univariate SOS lower-bound SDPs, one Gram block of side d+1 with
d ~ U{5..63} and m = 2d+1 Hankel 0/1 constraints (free gamma split into
two nonnegative scalars), solved by PrimalDual + NT + EigenStep + Mehrotra +
DenseCholesky in mixed precision (FP32 phase, FP64 finish) by one persistent
launch.  The same batch in plain FP64 is timed for the mixed/FP64 ratio.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  Under torchrun every rank solves its own
4096 instances (weak scaling, no collective on the data path).
"""

from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "madsdp.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

# request mixes of the served stream (Poisson arrivals): the serving
# workload's stated mix (max-cut n up to 800 and dense requests with m up to
# 3000 run in the server's whole-GPU slots), and a compact mix that one
# thread block per request serves
SERVE_MIXES = {
    "stated": {"sos_d": (5, 127), "maxcut_n": (50, 800), "dense_n": (32, 256), "dense_m": 3000, "dense_m_min": 100},
    "compact": {"sos_d": (5, 127), "maxcut_n": (20, 100), "dense_n": (8, 32), "dense_m": 200, "dense_m_min": 10},
}

METRIC = "SDP solves/sec + p50/p99 latency at 1e-7 gap: mixed/batched vs FP64 GPU vs CPU"
UNIT = "solves/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------- workload
def workload(n: int, seed: int, dmin: int = 5, dmax: int = 63):
    import numpy as np
    from madsdp_gpu import generators as g
    rng = np.random.default_rng(seed)
    ds = rng.integers(dmin, dmax + 1, size=n)
    return [g.sos_hankel(int(d), seed=seed * 100003 + i) for i, d in enumerate(ds)], [int(d) for d in ds]


def flops_per_iteration(n: int, m: int, nnz: int) -> float:
    """Algorithmic flops of one NT + Mehrotra + EigenStep iteration of one
    block (LAPACK conventions, eig = 4 n^3): 28 n^3 for the scaling, E(.),
    correction and step lengths, nnz^2 for the sparse Schur assembly
    (Hankel: n^4 entry pairs), m^3/3 for the Schur Cholesky and 4 m^2 for
    the two solves."""
    return 28.0 * n ** 3 + 2.0 * nnz * nnz / 2.0 + m ** 3 / 3.0 + 4.0 * m * m


# ----------------------------------------------------------------- CPU baseline
def _timed_port(prep, start, seconds, cores):
    """Solve the prepared instances from `start` on (cyclically) with the
    compiled CPU restatement on `cores` threads, starting new solves for
    `seconds` and letting the ones in flight finish.  Returns (solves/s,
    results as (index, status, pobj, iter, solve ms), next index)."""
    from oracle import cpu_ipm
    n = len(prep)
    nxt, results = start % n, []
    t0 = time.perf_counter()
    while True:
        left = seconds - (time.perf_counter() - t0)
        if left <= 0:
            break
        out = cpu_ipm.solve_many(prep, cores, left, start=nxt, count=n - nxt)
        for k, s in enumerate(out):
            if s is not None:
                if s["status"] < 0:
                    raise RuntimeError(f"the CPU restatement rejected instance {nxt + k}")
                results.append((nxt + k, s["status"], s["pobj"], s["iter"], s["solve_ns"] / 1e6))
        done = sum(s is not None for s in out)
        nxt = (nxt + done) % n
        if done < len(out):
            break
    return len(results) / (time.perf_counter() - t0), results, nxt


def cpu_port_prepare(models):
    """Build the compiled CPU restatement, marshal the instances and run one
    small solve (all untimed)."""
    from oracle import cpu_ipm
    cpu_ipm.build()
    prep = cpu_ipm.Prepared(models)
    cpu_ipm.solve_many(prep, 1, 0.0, start=0, count=1)
    return prep


def fifo_latencies(arrivals, service, workers):
    """Latency (finish - arrival) of each request served first-in first-out
    by `workers` identical workers; arrivals in nondecreasing order."""
    import heapq
    free = [0.0] * workers
    out = []
    for a, t in zip(arrivals, service):
        start = max(a, heapq.heappop(free))
        heapq.heappush(free, start + t)
        out.append(start + t - a)
    return out


def cpu_serve_replay(stream, cores, seconds):
    """The served stream on the host cores.  Every request is solved by the
    compiled restatement with all cores busy, in arrival order, new solves
    starting for `seconds` (the requests solved are a prefix of the
    stream).  The measured solve times are then scheduled first-in
    first-out on `cores` workers from the arrival times.  That latency is
    the one of an ideal CPU server without dispatch overhead (a lower
    bound); `capacity_solves_per_s` is the solves per second of all cores
    on this mix."""
    import numpy as np
    from oracle import cpu_ipm
    prep = cpu_port_prepare([m for _, _, m in stream])
    t0 = time.perf_counter()
    res = cpu_ipm.solve_many(prep, cores, seconds)
    wall = time.perf_counter() - t0
    k = 0
    while k < len(res) and res[k] is not None:
        k += 1
    if not k:
        return {"requests": 0, "of": len(stream), "note": f"no request solved within {seconds:.0f} s"}
    lat = fifo_latencies([a for a, _, _ in stream[:k]], [r["solve_ns"] / 1e9 for r in res[:k]], cores)
    per_kind = {}
    for (arrival, kind, _), t in zip(stream[:k], lat):
        per_kind.setdefault(kind, []).append(t)
    last = max(a + t for (a, _, _), t in zip(stream[:k], lat))
    return {
        "requests": k, "of": len(stream), "cores": cores,
        "converged": int(sum(res[i]["status"] == 1 for i in range(k))),
        "capacity_solves_per_s": k / wall,
        "solves_per_s": k / max(last - stream[0][0], 1e-9),
        "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
        "per_kind": {kd: {"count": len(v), "p50_latency_s": float(np.percentile(v, 50)),
                          "p99_latency_s": float(np.percentile(v, 99))} for kd, v in sorted(per_kind.items())},
        "method": "compiled C++ restatement solves each request (all cores busy); FIFO schedule of the measured "
                  "solve times on one worker per core from the arrival times (ideal CPU server, no overhead)",
    }


def cpu_batch_sample(args):
    """The batched workload on the host cores: all cores for `cpu_seconds`
    over the instances in order, then one thread for a quarter of that on
    the instances after them."""
    cores = os.cpu_count() or 1
    prep = cpu_port_prepare(workload(args.instances, args.seed)[0])
    v, res, nxt = _timed_port(prep, 0, args.cpu_seconds, cores)
    v1, res1, _ = _timed_port(prep, nxt, max(2.0, args.cpu_seconds / 4), 1)
    return {"value": v, "results": res, "count": len(res), "cores": cores, "one_thread": v1,
            "one_thread_count": len(res1)}


def cpu_batch_block(cpu, args, gpu_stats):
    """(cpu_baseline object of the line, largest relative objective
    difference between the GPU stats and the CPU solves of the same
    instances); (None, None) without a CPU sample."""
    import numpy as np
    if cpu is None:
        return None, None
    block = {"value": cpu["value"], "unit": UNIT, "cores": cpu["cores"], "kind": "port",
             "sample": f"{CPU_PORT}: {cpu['count']} solves of the {args.instances} instances in order "
                       f"(from the first, cyclically), {args.cpu_seconds:.0f} s, {cpu['cores']} threads",
             "one_thread_solves_per_s": cpu["one_thread"],
             "one_thread_sample": f"the next {cpu['one_thread_count']} instances on one thread, "
                                  f"{max(2.0, args.cpu_seconds / 4):.0f} s"}
    cpu_ms = np.array([r[4] for r in cpu["results"]])
    if cpu_ms.size:
        block["p50_latency_ms"] = float(np.percentile(cpu_ms, 50))
        block["p99_latency_ms"] = float(np.percentile(cpu_ms, 99))
    errs = []
    for i, status, pobj, it, _ in cpu["results"]:
        s = gpu_stats[i]
        errs.append(abs(pobj - s["pobj"]) / max(1.0, abs(s["pobj"]) + abs(s["dobj"])))
    return block, (max(errs) if errs else None)


CPU_PORT = "compiled C++ restatement of the oracle (oracle/cpu_ipm.cpp: FP64, NT+EigenStep+Mehrotra+DenseCholesky, " \
           "own dense kernels, no BLAS; its Hankel Schur assembly is the entry-pair sum, about n^4 per iteration, " \
           "while the GPU's FP64 path assembles by FFT along one index, O(n^3 log n): part of the ratio is that " \
           "algorithmic difference)"


# ----------------------------------------------------------------- single large instances
INSTANCE_WORKLOADS = {
    # MaxCut, ER n = 100, p = 0.1, unit weights (the reference's benchmark/maxcut.jl shape)
    "maxcut_n100": dict(kind="maxcut", n=100, p=0.1, weights="unit"),
    # MaxCut at scale, ER n = 2000, p = 0.005, weights +-1
    "maxcut_n2000": dict(kind="maxcut", n=2000, p=0.005, weights="pm1"),
    # dense constraints, PSD blocks [200, 100, 50, 50] + 500 scalars, m = 2000
    "dense_mixed_cones": dict(kind="dense", sides=[200, 100, 50, 50], ns=500, m=2000),
}


def instance_model(spec, seed):
    from madsdp_gpu import generators as g
    if spec["kind"] == "maxcut":
        return g.maxcut(spec["n"], spec["p"], weights=spec["weights"], seed=seed)
    return g.dense_random(spec["sides"], spec["ns"], spec["m"], seed=seed)


def instance_flops_per_iteration(model) -> float:
    """28 n^3 per block (NT scaling, E(.), correction, step lengths), the
    Schur assembly (one-hot n^2; Hankel/sparse nnz^2; dense
    4 n^3 m + m^2 n(n+1)/2), m^3/3 + 4 m^2 for the Schur factor and solves
    and m^2 ns for the scalar block."""
    m = model.m
    f = m ** 3 / 3.0 + 4.0 * m * m + float(m) * m * model.ns
    for n, A in zip(model.sides, model.A):
        f += 28.0 * n ** 3
        if A.nnz >= m * n * n // 2:
            f += 4.0 * n ** 3 * m + float(m) * m * n * (n + 1) / 2.0
        else:
            f += float(A.nnz) ** 2
    return f


def assembly_flops_per_iteration(model) -> float:
    """FP64-equivalent flops of the tensor-core Schur assembly of dense
    blocks (NT): P = [A_1; ...; A_m] G and B_j = (A_j G)' G (2 m n^3 each),
    then H += svec(B)' svec(B) over the lower triangle (m^2 n(n+1)/2), plus
    the scalar block C_lin diag(x/z) C_lin' (m^2 ns)."""
    m = model.m
    f = float(m) * m * model.ns
    for n, A in zip(model.sides, model.A):
        if A.nnz >= m * n * n // 2:
            f += 4.0 * m * n ** 3 + float(m) * m * n * (n + 1) / 2.0
    return f


def _oracle_iterations(spec, seed, q):
    sys.path[:0] = [ROOT, PKG]
    from oracle import madsdp_oracle as o
    model = instance_model(spec, seed)
    s = o.Solver(model)
    t = time.perf_counter()
    s.initialize()
    s.update_termination()
    q.put(("init", time.perf_counter() - t))
    while s.status == o.Status.REGULAR:
        t = time.perf_counter()
        s.iterate()
        if s.status != o.Status.REGULAR:
            break
        s.update_termination()
        q.put(("iter", time.perf_counter() - t))
    q.put(("done", s.iter))


def cpu_instance_sample(spec, seed, seconds):
    """Iterations of the oracle on the same instance (all BLAS threads) for
    about `seconds`; returns (seconds per iteration or None, iterations, init s)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    proc = ctx.Process(target=_oracle_iterations, args=(spec, seed, q))
    proc.start()
    t0 = time.perf_counter()
    iters, init = [], None
    while time.perf_counter() - t0 < seconds + 600:
        try:
            kind, v = q.get(timeout=1.0)
        except Exception:
            if not proc.is_alive():
                break
            if init is not None and time.perf_counter() - t0 > seconds:
                break
            continue
        if kind == "init":
            init = v
            t0 = time.perf_counter()
        elif kind == "iter":
            iters.append(v)
            if time.perf_counter() - t0 > seconds:
                break
        else:
            break
    proc.terminate()
    proc.join(5)
    return (statistics.mean(iters) if iters else None), len(iters), init


# instances whose solve the compiled restatement (own dense kernels, no
# BLAS) finishes in about a second: timed with it, larger ones with the
# NumPy oracle on all BLAS threads
PORT_MAX_FLOPS_PER_SOLVE = 5e9


def port_fits(model) -> bool:
    return 20 * instance_flops_per_iteration(model) <= PORT_MAX_FLOPS_PER_SOLVE


def cpu_port_instance(model, seconds):
    """Full solves of one instance by the compiled restatement on one
    thread, repeated for about `seconds` (at least one); returns (solves/s,
    solves, iterations of a solve)."""
    from oracle import cpu_ipm
    cpu_ipm.build()
    cpu_ipm.solve(model)  # load, untimed
    done, t0 = 0, time.perf_counter()
    while True:
        st = cpu_ipm.solve(model)
        if st["status"] < 0:
            raise RuntimeError("the CPU restatement rejected the instance")
        done += 1
        if time.perf_counter() - t0 >= seconds:
            break
    return done / (time.perf_counter() - t0), done, st["iter"]


def port_block(v, done, iters):
    return {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{CPU_PORT}: {done} full solves of the same instance on one thread ({iters} iterations)"}


def run_instance_reference(args):
    """The oracle on the same large instance, all BLAS threads: a bounded
    number of iterations, solve time = init + mean iteration x iterations to
    1e-7 (the iteration count of the oracle's own run when it finishes, else
    of the GPU run recorded by the same workload)."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    spec = INSTANCE_WORKLOADS[args.workload]
    cores = os.cpu_count() or 1
    line = {"impl": "reference", "metric": METRIC, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": args.workload, **{k: v for k, v in spec.items() if k != "kind"},
                                            "seed": args.seed}}
    model = instance_model(spec, args.seed)
    if port_fits(model):
        v, done, it = cpu_port_instance(model, args.cpu_seconds)
        line.update(value=v, cpu_baseline=port_block(v, done, it))
        line["e2e"] = {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
        print(json.dumps(line), flush=True)
        return
    per_it, nit, init = cpu_instance_sample(spec, args.seed, args.cpu_seconds)
    iters = {"maxcut_n100": 11, "maxcut_n2000": 16, "dense_mixed_cones": 18}[args.workload]
    if per_it is None:
        line.update(value=None, cpu_baseline={"value": None, "unit": UNIT, "cores": cores, "kind": "port",
                                              "sample": f"no oracle iteration finished within {args.cpu_seconds:.0f} s"})
    else:
        v = 1.0 / ((init or 0.0) + per_it * iters)
        line.update(value=v, cpu_baseline={"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                           "sample": f"oracle on the same instance: {nit} iterations timed, "
                                                     f"init + mean iteration x {iters}"})
    line["e2e"] = {"value": line["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    print(json.dumps(line), flush=True)


def run_instance(args):
    """One large problem per step on the whole GPU (msdp_solver)."""
    import numpy as np
    spec = INSTANCE_WORKLOADS[args.workload]
    cpu = port = None
    if not args.no_cpu:
        small = instance_model(spec, args.seed)
        if port_fits(small):
            port = cpu_port_instance(small, args.cpu_seconds)
        else:
            cpu = cpu_instance_sample(spec, args.seed, args.cpu_seconds)
        del small
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import madsdp_gpu as M
    model = instance_model(spec, args.seed)
    ctx = M.Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream_handle, device=torch.device("cuda", 0))
    # the engine MadSDPSolver(model) picks: one thread block (a one-problem
    # batch) for small problems, the whole-GPU solver for large ones
    engine = "instance" if (args.precision == "fp64_tensor" or M.solver._use_instance_engine(model)) else "batch"
    if engine == "instance":
        solver = M.InstanceSolver(model, context=ctx, precision=args.precision)
        run = solver.solve
    else:
        solver = M.Batch([model], context=ctx, precision="mixed" if args.precision == "mixed" else "fp64")
        run = solver.solve
    for _ in range(args.warmup):
        run()
    sampler = ClockSampler(0)
    sampler.start()
    ms, launches = [], solver.launch_count
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        run()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    clocks = sampler.stop()
    launches = solver.launch_count - launches
    counters = None
    if engine == "instance":
        st = solver.stats()
        phases = {k: round(v, 4) for k, v in solver.profile().items()}
        counters = solver.counters()
    else:
        st = solver.stats(0)
        phases = None
    device_bytes = solver.device_bytes
    solver.close()
    # end to end: upload, solve, download through the public API
    t = time.perf_counter()
    e2 = M.MadSDPSolver(model, engine=engine, context=ctx, precision=args.precision)
    e2.solve()
    X, y, x, z = e2.solution()
    e2e_s = time.perf_counter() - t
    h2d = sum(8 * n * n for n in model.sides) + sum(16 * A.nnz + 12 * A.nnz for A in model.A) + 8 * (
        model.m + model.ns + model.m * model.ns)
    d2h = sum(8 * n * n for n in model.sides) + 8 * (model.m + 2 * model.ns)
    e2.close()
    t_solve = statistics.mean(ms) / 1000.0
    flops = instance_flops_per_iteration(model) * st["iter"]
    fp64_peak, _ = measured_fp_rates()  # GFLOP/s
    # the tensor-core Schur assembly against the bf16 peak: slice products
    # (28 for FP64-accurate, 6 for split precision) x FP64-equivalent flops
    tc_assembly = None
    if engine == "instance" and phases and phases.get("schur_assembly"):
        af = assembly_flops_per_iteration(model) * st["iter"]
        if af > 0:
            hbm, bf16, peak_kind = measured_peaks()
            n32, n64 = st.get("iter_fp32", 0), st.get("iter_fp64", 0)
            pairs = (28.0 * n64 + 6.0 * n32) / max(1, n32 + n64)
            tensor_tflops = af * pairs / phases["schur_assembly"] / 1e12
            tc_assembly = {"fp64_equiv_tflops": af / phases["schur_assembly"] / 1e12,
                           "tensor_tflops": tensor_tflops, "bf16_peak_tflops": bf16,
                           "frac_of_bf16_peak": tensor_tflops / bf16, "peak_kind": f"{peak_kind} bf16 dense (burst)",
                           "slice_products_per_flop": pairs,
                           "note": "assembly phase device time (includes the slicing passes and the scalar block)"}
    cpu_block = port_block(*port) if port is not None else None
    if cpu is not None:
        per_it, nit, init = cpu
        if per_it is not None:
            est = (init or 0.0) + per_it * st["iter"]
            cpu_block = {"value": 1.0 / est, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                         "sample": f"oracle (NumPy/SciPy FP64, all BLAS threads) on the same instance: "
                                   f"{nit} iterations timed, solve time = init + mean iteration x {st['iter']} GPU iterations"}
        else:
            cpu_block = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                         "sample": f"oracle did not finish one iteration within {args.cpu_seconds:.0f} s"}
    line = {
        "metric": METRIC, "value": 1.0 / t_solve, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(ms), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {"fp64": "f64", "fp64_tensor": "f64 (tensor-core emulated products)",
                  "mixed": "f32+f64"}[args.precision],
        "data": "synthetic",
        "config": {"workload": args.workload, "precision": args.precision, **{k: v for k, v in spec.items() if k != "kind"}, "seed": args.seed,
                   "m": model.m, "components": "PrimalDual(NT, EigenStep, Mehrotra) + DenseCholesky, ScaledIdentity",
                   "engine": ("whole-GPU instance solver: tensor-core split-bf16 products and Schur assembly (tcgen05), "
                              "blocked Cholesky with tensor-core updates and own triangular solves, own assembly/"
                              "residual kernels; cuSOLVER eigensolver and S^-1, cuBLAS triangular solves of the "
                              "step lengths" if engine == "instance"
                              else "one thread block (persistent batch kernel, one problem)"),
                   "iterations_fp32_schur": st.get("iter_fp32"), "iterations_fp64_schur": st.get("iter_fp64"),
                   "tensor_core_assembly": tc_assembly,
                   "status": str(st["status"]), "iterations": st["iter"], "pobj": st["pobj"], "gap": st["gap"],
                   "inf_pr": st["inf_pr"], "inf_du": st["inf_du"], "phase_seconds_last_solve": phases,
                   "work_counters_last_solve": counters,
                   "l2": f"{device_bytes / 2**20:.0f} MiB resident"},
        "gpu_launches": launches // max(1, args.steps),
        "e2e": {"value": 1.0 / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "fp64", "achieved": flops / t_solve / 1e9, "peak": fp64_peak, "unit": "GFLOP/s",
                     "frac": flops / t_solve / 1e9 / fp64_peak, "traffic": None,
                     "peak_kind": "measured FP64 FMA throughput (profiles/gb300_primitives.txt)",
                     "note": "algorithmic flops of the iterations (model above) / solve time"},
        "cpu_baseline": cpu_block,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], 0.0, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names[1:], parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_fp_rates():
    """(FP64, FP32) CUDA-core rates in GFLOP/s measured on GB300
    (profiles/gb300_primitives.txt: FMA throughput of independent chains)."""
    fp64, fp32 = 1000.0, 67000.0
    p = os.path.join(ROOT, "profiles", "gb300_primitives.txt")
    if os.path.exists(p):
        for line in open(p):
            if "TFLOP/s" in line and line.startswith(("fp64 fma throughput", "fp32 fma throughput")):
                try:
                    v = float(line.split("~")[1].split("TFLOP/s")[0]) * 1e3
                except (IndexError, ValueError):
                    continue
                if line.startswith("fp64"):
                    fp64 = v
                else:
                    fp32 = v
    return fp64, fp32


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of the IPM kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ipm_kernel_sos_batch.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch"):
            try:
                return float(line.split("=")[1].split()[0])
            except (IndexError, ValueError):
                return None
    return None


# ----------------------------------------------------------------- arms
def run_reference(args):
    """The compiled CPU restatement on all host cores (one solve per thread)
    over the workload's instances, in order; each step starts solves for
    about `cpu_seconds / (warmup + steps)` seconds and lets the ones in
    flight finish."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.instances
    models = workload(n, args.seed)[0]
    cores = os.cpu_count() or 1
    per_step = max(2.0, args.cpu_seconds / max(1, args.steps + args.warmup))
    prep = cpu_port_prepare(models)
    vals, nxt, solve_ms = [], 0, []
    for k in range(args.warmup + args.steps):
        rate, res, nxt = _timed_port(prep, nxt, per_step, cores)
        if k >= args.warmup:
            vals.append(rate)
            solve_ms += [r[4] for r in res]
    value = statistics.mean(vals)
    solve_ms.sort()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "sos_hankel_batch", "instances": n, "d_range": [5, 63], "m": "2d+1",
                   "components": "PrimalDual(NT, EigenStep, Mehrotra) + DenseCholesky"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{CPU_PORT} on the workload's instances in order, {per_step:.0f} s per step, "
                                   f"{cores} threads",
                         "p50_latency_ms": solve_ms[len(solve_ms) // 2] if solve_ms else None,
                         "p99_latency_ms": solve_ms[min(len(solve_ms) - 1, int(0.99 * len(solve_ms)))]
                         if solve_ms else None},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import numpy as np

    # CPU baseline first, on the host cores before any CUDA work
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_batch_sample(args)

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import __graft_entry__
    __graft_entry__.build()
    import madsdp_gpu as M

    # every rank draws the same world x instances problems and takes its
    # cost-balanced share (weak scaling: `instances` per GPU on average)
    from madsdp_gpu.distributed import shard_by_cost, solve_cost
    all_models, all_ds = workload(args.instances * world, args.seed)
    mine = shard_by_cost([solve_cost(mm) for mm in all_models], world)[rank] if world > 1 else list(range(len(all_models)))
    models, ds = [all_models[i] for i in mine], [all_ds[i] for i in mine]
    ctx = M.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream_handle, device=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    def timed_solves(batch, steps, warmup):
        for _ in range(warmup):
            batch.launch_solve()
            batch.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
               torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        barrier()
        torch.cuda.synchronize()
        batch.synchronize()
        l0 = batch.launch_count
        for e0, e1, e2 in ev:
            e0.record(stream)
            batch.launch_initialize()
            e1.record(stream)
            batch.iterate(0, sync=False)
            e2.record(stream)
        batch.synchronize()
        torch.cuda.synchronize()
        barrier()
        step_ms = [a.elapsed_time(c) for a, _, c in ev]
        kern_ms = [b.elapsed_time(c) for _, b, c in ev]
        return step_ms, kern_ms, batch.launch_count - l0

    # ---- FP64 GPU path (comparison)
    b64 = M.Batch(models, precision="fp64", context=ctx)
    f64_steps = max(1, min(args.steps, args.fp64_steps))
    s64, k64, _ = timed_solves(b64, f64_steps, 1)
    st64 = b64.all_stats()
    b64.close()

    # ---- mixed path (headline)
    bm = M.Batch(models, precision="mixed", context=ctx)
    sampler = ClockSampler(local)
    sampler.start()
    step_ms, kern_ms, launches = timed_solves(bm, args.steps, args.warmup)
    clocks = sampler.stop()
    stm = bm.all_stats()
    device_bytes = bm.device_bytes
    bm.close()

    from madsdp_gpu.distributed import max_over_ranks
    total_ms = max_over_ranks(sum(step_ms))
    value = args.instances * world * args.steps / (total_ms / 1000.0)
    fp64_value = len(models) / (statistics.mean(s64) / 1000.0)

    # ---- end to end through the public API with host buffers: upload,
    # solve, every instance's statistics and solution (X, y, x, z) back
    e2e_times = []
    h2d = d2h = 0
    for k in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        be = M.Batch(models, precision="mixed", context=ctx)
        be.launch_solve()
        st = be.all_stats()
        sols = be.all_solutions()
        h2d = be.upload_bytes
        d2h = len(st) * 120 + 8 * sum(sum(x.size for x in X) + y.size + xx.size + z.size for X, y, xx, z in sols)
        be.close()
        e2e_times.append(time.perf_counter() - t0)
    e2e_value = len(models) / statistics.mean(e2e_times[1:] if len(e2e_times) > 1 else e2e_times)

    # ---- served Poisson stream (continuous batching, real time)
    serving = None
    if args.serve_seconds > 0:
        from madsdp_gpu.serving import Server, poisson_stream, serve_stream
        mix = SERVE_MIXES[args.serve_mix]
        pool = args.serve_dense_pool if args.serve_mix == "stated" else None
        stream = poisson_stream(args.serve_rate, args.serve_seconds, seed=args.seed + 17 + rank, dense_pool=pool,
                                **mix)
        srv = Server(memory_budget_bytes=8 << 30, max_slots=4096, precision="mixed", context=ctx,
                     whole_gpu_slots=args.serve_whole_gpu_slots, whole_gpu_memory_bytes=64 << 30)
        serving = serve_stream(srv, stream, iterations=args.serve_iterations, time_limit=1800.0,
                               budget_s=args.serve_budget_ms / 1e3)
        srv.close()
        serving.update({"rate_per_s": args.serve_rate, "duration_s": args.serve_seconds,
                        "iterations_per_wave": args.serve_iterations, "wave_budget_ms": args.serve_budget_ms,
                        "memory_budget_bytes": 8 << 30, "whole_gpu_slots": args.serve_whole_gpu_slots,
                        "whole_gpu_memory_bytes": 64 << 30, "mix_name": args.serve_mix,
                        "precision": "mixed in the batched waves, FP64 in the whole-GPU slots (the faster of the "
                                     "two there: config 2 2.02 s FP64 against 2.29 s mixed)",
                        "dense_requests": ("drawn from %d dense models generated before the stream (each up to "
                                           "1.5 GB of constraint data); every request is solved in full" % pool)
                        if pool else "one model per request",
                        "mix": "50%% SOS d~U%s, 30%% max-cut n~U%s p=4/n, 20%% dense one block n~U%s "
                               "m~U(%d, %d) capped at n(n+1)/2; requests with a block above 128 or m above 300 run "
                               "in whole-GPU slots (serve_whole_gpu)" % (mix["sos_d"], mix["maxcut_n"], mix["dense_n"],
                                                      mix["dense_m_min"], mix["dense_m"]),
                        "latency": "host clock, arrival to result available"})
        if rank == 0 and world == 1 and not args.no_cpu:
            if args.serve_mix == "compact":
                serving["cpu_replay"] = cpu_serve_replay(stream, os.cpu_count() or 1, args.cpu_seconds)
            else:
                serving["cpu_replay"] = {"note": "not run for this mix: the compiled restatement (no BLAS) needs "
                                                 "minutes per dense request with m in the thousands, so a bounded "
                                                 "sample would not finish its solves in flight"}

    if rank != 0:
        return
    conv = [s["status"] == M.Status.SOLVE_SUCCEEDED and max(s["inf_pr"], s["inf_du"], s["gap"]) <= 1e-7 for s in stm]
    conv64 = [s["status"] == M.Status.SOLVE_SUCCEEDED for s in st64]
    lat = np.array([s["solve_ns"] for s in stm]) / 1e6
    rel = [abs(a["pobj"] - b["pobj"]) / max(1.0, abs(b["pobj"]) + abs(b["dobj"])) for a, b in zip(stm, st64)]
    iters = np.array([s["iter"] for s in stm])
    flops = 0.0
    for mdl, s in zip(models, stm):
        n = mdl.sides[0]
        flops += s["iter"] * flops_per_iteration(n, mdl.m, mdl.A[0].nnz)
    kern_s = statistics.mean(kern_ms) / 1000.0
    hbm, bf16, peak_kind = measured_peaks()
    fp64_rate, fp32_rate = measured_fp_rates()
    achieved = flops / kern_s / 1e12
    traffic = profiled_traffic()
    cpu_block, oracle_err = cpu_batch_block(cpu, args, stm)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {
            "workload": "sos_hankel_batch (4th workload: batched SOS SDPs)", "instances_per_gpu": args.instances,
            "instances_this_rank": len(models),
            "d_range": [5, 63], "m": "2d+1", "ns": 2, "seed": args.seed,
            "components": "PrimalDual(NT, EigenStep, Mehrotra) + DenseCholesky, ScaledIdentity",
            "precision": "mixed: FP32 block algebra and Schur factor, each direction refined twice against the "
                         "float64 primal defect; FP64 iterations after an FP32 failure, a short step or a rejected "
                         "direction",
            "parallelism": f"one persistent launch, one CTA per instance; {world} GPU(s) x own instances",
            "l2": f"inputs and workspaces ({device_bytes / 2**20:.0f} MiB resident) larger than L2",
            "converged_1e-7": f"{sum(conv)}/{len(conv)}", "fp64_converged": f"{sum(conv64)}/{len(conv64)}",
            "p50_latency_ms": float(np.percentile(lat, 50)), "p99_latency_ms": float(np.percentile(lat, 99)),
            "iterations_mean": float(iters.mean()),
            "fp32_iterations_mean": float(np.mean([s["iter_fp32"] for s in stm])),
            "fp64_gpu_solves_per_s": fp64_value, "mixed_over_fp64": value / world / fp64_value,
            "mixed_vs_fp64_max_rel_obj_diff": max(rel), "mixed_vs_oracle_max_rel_obj_diff": oracle_err,
            "served_stream": serving,
        },
        "gpu_launches": launches,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
                     "frac": achieved / bf16, "traffic": traffic,
                     "peak_kind": f"{peak_kind} bf16 dense (burst)",
                     "note": "algorithmic flops of the iteration (28n^3 + nnz^2 + m^3/3 + 4m^2 per instance-"
                             "iteration) / iterate-kernel time; the kernel runs on CUDA cores (FP32/FP64), not tcgen05",
                     "limiter": "FP64 pipe (1.25 TFLOP/s nominal on GB300): 26% of active cycles on average, "
                                "saturated on the busiest SMs (profiles/ipm_kernel_sos_batch.txt)",
                     "fp64_pipe_frac": achieved * 1e3 / fp64_rate, "fp32_pipe_frac": achieved * 1e3 / fp32_rate,
                     "pipe_peaks_gflops": {"fp64": fp64_rate, "fp32": fp32_rate,
                                           "source": "measured FMA throughput, profiles/gb300_primitives.txt"}},
        "cpu_baseline": cpu_block,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=5.0)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-mix", default="stated", choices=sorted(SERVE_MIXES))
    ap.add_argument("--serve-whole-gpu-slots", type=int, default=8)
    ap.add_argument("--serve-dense-pool", type=int, default=6)
    ap.add_argument("--serve-iterations", type=int, default=1000)
    ap.add_argument("--serve-budget-ms", type=float, default=20.0)
    ap.add_argument("--workload", default="sos_batch", choices=["sos_batch", *INSTANCE_WORKLOADS])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp64_tensor", "mixed"],
                    help="instance workloads: FP64, FP64 products emulated on tensor cores (whole-GPU engine), "
                         "or mixed precision in one thread block (the batch engine)")
    args = ap.parse_args()
    if args.workload != "sos_batch":
        if args.impl == "reference":
            run_instance_reference(args)
            return
        run_instance(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
