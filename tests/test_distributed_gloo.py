"""Sharded batched solves on two gloo ranks (CPU): the cost-balanced split,
the gather back to rank 0 in input order, the max-over-ranks timing, and a
rank that fails before the gather."""

import datetime
import os
import pickle
import socket

import numpy as np
import pytest
import torch.multiprocessing as tmp

from madsdp_gpu import generators as g
from madsdp_gpu.distributed import max_over_ranks, shard_by_cost, solve_cost, solve_sharded


def models():
    return [g.sos_hankel(d, seed=70 + d) for d in (3, 9, 5, 12, 4, 7)] + [g.maxcut(8, 0.5, seed=2), g.trace_one()]


def oracle_solve(ms):
    from oracle import madsdp_oracle as o
    out = []
    for m in ms:
        s = o.Solver(m).solve()
        out.append((int(s.status), s.iter, s.primal_objective(), s.dual_objective()))
    return out


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, outdir, fail_rank):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "madsdp.jl_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    record = {}
    try:
        record["tmax"] = max_over_ranks(1.5 + rank)
        if rank == fail_rank:
            raise RuntimeError("planted failure before the gather")
        record["results"] = solve_sharded(models(), oracle_solve, rank, world)
    except Exception as e:  # recorded for the parent to inspect
        record["error"] = f"{type(e).__name__}: {e}"
    with open(os.path.join(outdir, f"rank{rank}.pkl"), "wb") as f:
        pickle.dump(record, f)
    if "error" not in record:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def run_ranks(tmp_path, fail_rank=-1, world=2):
    ctx = tmp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, str(tmp_path), fail_rank)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
        if p.is_alive():
            p.kill()
            pytest.fail("rank did not exit")
    out = []
    for r in range(world):
        with open(tmp_path / f"rank{r}.pkl", "rb") as f:
            out.append(pickle.load(f))
    return out


def test_shard_by_cost_balances_and_partitions():
    rng = np.random.default_rng(0)
    costs = list(rng.integers(6, 65, size=200).astype(float) ** 3)
    for world in (1, 2, 3, 8):
        shards = shard_by_cost(costs, world)
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in s) for s in shards]
        assert max(loads) - min(loads) <= max(costs)
    assert shard_by_cost([1.0], 3) == [[0], [], []]
    with pytest.raises(ValueError):
        shard_by_cost([1.0], 0)


def test_solve_cost_orders_by_size():
    assert solve_cost(g.sos_hankel(40)) > solve_cost(g.sos_hankel(10))


def test_two_ranks_gather_in_order(tmp_path):
    recs = run_ranks(tmp_path)
    assert all("error" not in r for r in recs), recs
    assert recs[0]["tmax"] == recs[1]["tmax"] == 2.5
    assert recs[1]["results"] is None
    assert recs[0]["results"] == oracle_solve(models())


def test_failed_rank_surfaces_on_the_others(tmp_path):
    recs = run_ranks(tmp_path, fail_rank=1)
    assert "planted failure" in recs[1]["error"]
    assert "error" in recs[0]
