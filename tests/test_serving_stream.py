"""Request stream of the serving workload (host only)."""

import numpy as np

from madsdp_gpu.serving import poisson_stream


def test_stream_is_seeded_and_mixed():
    a = poisson_stream(rate=500.0, duration=1.0, seed=7)
    b = poisson_stream(rate=500.0, duration=1.0, seed=7)
    assert [(t, k) for t, k, _ in a] == [(t, k) for t, k, _ in b]
    times = np.array([t for t, _, _ in a])
    assert np.all(np.diff(times) > 0) and times[-1] <= 1.0
    assert 400 < len(a) < 600
    kinds = [k for _, k, _ in a]
    frac = {k: kinds.count(k) / len(kinds) for k in ("sos", "maxcut", "dense")}
    assert abs(frac["sos"] - 0.5) < 0.08 and abs(frac["maxcut"] - 0.3) < 0.08 and abs(frac["dense"] - 0.2) < 0.08
    for _, kind, m in a[:50]:
        if kind == "sos":
            assert m.nblocks == 1 and 6 <= m.sides[0] <= 64 and m.m == 2 * m.sides[0] - 1
        elif kind == "maxcut":
            assert m.nblocks == 1 and 20 <= m.sides[0] <= 64 and m.m == m.sides[0]
        else:
            n = m.sides[0]
            assert m.ns == 0 and 8 <= n <= 24 and m.m <= min(60, n * (n + 1) // 2)


def test_whole_gpu_routing_of_the_stated_mix():
    """Requests shaped like the stated mix (SOS d <= 127, max-cut n in
    [50, 800]; dense models kept to n <= 64, m <= 400 here so the stream is
    quick to draw) take a whole-GPU slot exactly when a block is above 128
    or m is above 300; everything else runs in the batched waves.  The
    dense pool gives the same model objects to several arrivals."""
    from madsdp_gpu.serving import instance_bytes_estimate, serve_whole_gpu

    stated = {"sos_d": (5, 127), "maxcut_n": (50, 800), "dense_n": (32, 64), "dense_m": 400, "dense_m_min": 100}
    stream = poisson_stream(200.0, 0.4, seed=3, dense_pool=3, **stated)
    seen = {"batch": 0, "whole": 0}
    for _, kind, m in stream:
        whole = serve_whole_gpu(m)
        assert whole == (max(m.sides) > 128 or m.m > 300)
        seen["whole" if whole else "batch"] += 1
        if kind == "sos" and m.sides[0] <= 128:
            assert not whole  # SOS d <= 127 always fits the waves
        if whole:
            assert instance_bytes_estimate(m) > 0
    assert seen["batch"] > 0 and seen["whole"] > 0
    dense = [m for _, k, m in stream if k == "dense"]
    assert len({id(m) for m in dense}) <= 3
    # a narrower batch limit moves the 65-128 blocks to whole-GPU slots
    mid = [m for _, k, m in stream if 64 < max(m.sides) <= 128 and m.m <= 300]
    assert mid and all(serve_whole_gpu(m, batch_max_side=64) for m in mid)
