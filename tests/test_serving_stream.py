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
