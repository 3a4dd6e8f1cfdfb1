"""The reference arm of bench.py (the oracle on the host cores) prints one
JSON line with the contract's keys; runs on CPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    return json.loads(lines[0])


def check_common(d):
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_batched_sos():
    d = run_bench("--steps", "1", "--warmup", "1", "--cpu-seconds", "4", "--instances", "64")
    check_common(d)
    assert d["value"] > 0 and d["e2e"]["value"] == d["value"]
    assert d["config"]["workload"] == "sos_hankel_batch"


def test_reference_arm_single_instance():
    d = run_bench("--workload", "maxcut_n100", "--cpu-seconds", "3")
    check_common(d)
    assert d["value"] > 0 and d["config"]["workload"] == "maxcut_n100"


def test_fifo_latencies():
    sys.path.insert(0, ROOT)
    import bench
    # two workers, three simultaneous requests: the third waits for the first
    assert bench.fifo_latencies([0.0, 0.0, 0.0], [1.0, 2.0, 1.0], 2) == [1.0, 2.0, 2.0]
    # idle workers: latency = service time
    assert bench.fifo_latencies([0.0, 5.0, 10.0], [1.0, 1.0, 1.0], 1) == [1.0, 1.0, 1.0]
    # one worker, a backlog
    assert bench.fifo_latencies([0.0, 0.5, 1.0], [1.0, 1.0, 1.0], 1) == [1.0, 1.5, 2.0]


def test_cpu_serve_replay_small_stream():
    sys.path.insert(0, ROOT)
    import bench
    from madsdp_gpu.serving import poisson_stream
    stream = poisson_stream(20.0, 1.0, seed=3, sos_d=(5, 12), maxcut_n=(10, 20), dense_n=(6, 10), dense_m=20)
    r = bench.cpu_serve_replay(stream, 2, 30.0)
    assert r["requests"] == r["of"] == len(stream) and r["converged"] == r["requests"]
    assert 0 < r["p50_latency_s"] <= r["p99_latency_s"]
    assert sum(v["count"] for v in r["per_kind"].values()) == r["requests"]


def test_cpu_batch_baseline_block():
    """The GPU line's CPU leg, with the CPU solves standing in for the GPU
    stats: the block carries the contract's keys and a zero difference."""
    sys.path.insert(0, ROOT)
    import argparse

    import bench
    from oracle import cpu_ipm
    args = argparse.Namespace(instances=24, seed=4, cpu_seconds=3.0)
    cpu = bench.cpu_batch_sample(args)
    models = bench.workload(args.instances, args.seed)[0]
    stats = cpu_ipm.solve_many(models, threads=2)
    block, err = bench.cpu_batch_block(cpu, args, stats)
    assert block["kind"] == "port" and block["value"] > 0 and block["one_thread_solves_per_s"] > 0
    assert 0 < block["p50_latency_ms"] <= block["p99_latency_ms"]
    assert err == 0.0
    assert bench.cpu_batch_block(None, args, stats) == (None, None)
