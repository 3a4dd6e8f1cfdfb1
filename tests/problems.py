"""Model builders shared by the tests (the fixtures of the reference tests)."""
import numpy as np

from madsdp_gpu import generators as g
from madsdp_gpu.model import Model


def build(name: str) -> Model:
    if name == "trivial_2x2":
        return g.trivial_2x2()
    if name == "trace_one":
        return g.trace_one()
    if name == "mixed_lp":
        return g.mixed_lp_example()
    if name == "maxcut_weighted4":
        return g.maxcut_from_weights(g.weighted_4node_W())
    if name == "maxcut_cycle4":
        return g.maxcut_from_weights(g.cycle4_W())
    if name == "maxcut_K4":
        return g.maxcut_from_weights(np.ones((4, 4)) - np.eye(4))
    if name == "qr_example":
        return g.qr_example(0)
    if name == "qr_example2":
        return g.qr_example(2)
    raise KeyError(name)


def laplacian(W):
    W = np.asarray(W, dtype=float)
    return np.diag(W.sum(axis=1)) - W


def compare_trajectories(gpu_traj, ref_traj, gap_floor=1e-5, rtol=1e-6):
    """Per iteration, pobj and dobj agree to rtol while the gap is above gap_floor."""
    n = min(len(gpu_traj), len(ref_traj))
    for k in range(n):
        r, q = gpu_traj[k], ref_traj[k]
        if r["gap"] < gap_floor:
            break
        for key in ("pobj", "dobj"):
            assert abs(q[key] - r[key]) <= rtol * max(1.0, abs(r[key])), (k, key, q[key], r[key])
