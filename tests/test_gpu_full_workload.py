"""Parity at full size: every instance of the batched SOS workload (4096
univariate SOS lower bounds, Gram blocks of side 6..64, m = 2d+1 Hankel
constraints, seed 4) on the GPU, in FP64 and in mixed precision, against
the compiled oracle restatement (oracle/cpu_ipm.cpp, which takes the same
iterates as the NumPy oracle) on all host cores.

Tolerances: every instance converges; final objectives within
1e-7 * max(1, |p| + |d|) of the oracle in FP64 and in mixed precision.  FP64 iteration counts equal the oracle's within one
for at least 99% of the instances and within two for all: the termination
test compares measures that fall by about 10x per iteration with 1e-7, so
a difference in the last digits of an instance whose measure lands next to
the tolerance moves its stop by one iteration."""
import os

import numpy as np
import pytest

import bench
import madsdp_gpu as M
from oracle import cpu_ipm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload():
    models, _ = bench.workload(4096, 4)
    ref = cpu_ipm.solve_many(models, threads=os.cpu_count() or 1)
    assert all(r is not None and r["status"] == 1 for r in ref)
    return models, ref


def scale(r):
    return max(1.0, abs(r["pobj"]) + abs(r["dobj"]))


def test_full_workload_fp64(gpu_ctx, workload):
    models, ref = workload
    bt = M.Batch(models, precision="fp64")
    bt.solve()
    stats = bt.all_stats()
    bt.close()
    err = np.array([abs(s["pobj"] - r["pobj"]) / scale(r) for s, r in zip(stats, ref)])
    diter = np.array([abs(s["iter"] - r["iter"]) for s, r in zip(stats, ref)])
    assert all(s["status"] == M.Status.SOLVE_SUCCEEDED for s in stats)
    assert err.max() <= 1e-7, (int(err.argmax()), float(err.max()))
    assert np.mean(diter <= 1) >= 0.99 and diter.max() <= 2, np.bincount(diter)


def test_full_workload_mixed(gpu_ctx, workload):
    models, ref = workload
    bt = M.Batch(models, precision="mixed")
    bt.solve()
    stats = bt.all_stats()
    bt.close()
    err = np.array([abs(s["pobj"] - r["pobj"]) / scale(r) for s, r in zip(stats, ref)])
    assert all(s["status"] == M.Status.SOLVE_SUCCEEDED for s in stats)
    assert all(max(s["inf_pr"], s["inf_du"], s["gap"]) <= 1e-7 for s in stats)
    assert err.max() <= 1e-7, (int(err.argmax()), float(err.max()))
