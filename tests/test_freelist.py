"""The server arena's free list (madsdp.jl_gb300/csrc/freelist.h) on the
CPU: random allocate/free sequences against a model of the arena.  Ranges
handed out never overlap and stay inside the arena, allocation is first
fit, the free list stays coalesced and accounts for every free byte, and
freeing everything restores one range."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
I = C.POINTER(C.c_int64)


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("freelist") / "freelist_check.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "native", "freelist_check.cpp")], check=True)
    lib = C.CDLL(so)
    lib.freelist_run.argtypes = [C.c_int64, C.c_int64, I, I, I, I, C.c_int64, I, I]
    lib.freelist_run.restype = C.c_int64
    return lib


def run(lib, capacity, ops, offs, sizes):
    n = len(ops)
    arr = [np.ascontiguousarray(x, dtype=np.int64) for x in (ops, offs, sizes)]
    out = np.zeros(max(n, 1), np.int64)
    fo, fs = np.zeros(4096, np.int64), np.zeros(4096, np.int64)
    k = lib.freelist_run(capacity, n, *(a.ctypes.data_as(I) for a in arr), out.ctypes.data_as(I), 4096,
                         fo.ctypes.data_as(I), fs.ctypes.data_as(I))
    return out[:n], list(zip(fo[:k], fs[:k]))


def first_fit(used, capacity, size):
    """Lowest offset of `size` free bytes in the model (a boolean map)."""
    run_start, run_len = 0, 0
    for off in range(capacity):
        if used[off]:
            run_len = 0
            run_start = off + 1
        else:
            run_len += 1
            if run_len == size:
                return run_start
    return -1


@pytest.mark.parametrize("seed", range(6))
def test_random_sequences(lib, seed):
    rng = np.random.default_rng(seed)
    capacity = 4000
    # build the sequence step by step against the model, then replay it
    used = np.zeros(capacity, bool)
    live = {}  # op index -> (off, size)
    ops, offs, sizes, expect = [], [], [], []
    for i in range(600):
        if live and rng.random() < 0.45:
            j = list(live)[rng.integers(len(live))]
            off, size = live.pop(j)
            used[off:off + size] = False
            ops.append(-(j + 1)); offs.append(off); sizes.append(size); expect.append(0)
        else:
            size = int(rng.integers(1, 300))
            off = first_fit(used, capacity, size)
            ops.append(size); offs.append(0); sizes.append(0); expect.append(off)
            if off >= 0:
                used[off:off + size] = True
                live[i] = (off, size)
    out, free = run(lib, capacity, ops, offs, sizes)
    assert list(out) == expect
    # the free list is the complement of the model, coalesced
    model_free = []
    off = 0
    while off < capacity:
        if not used[off]:
            end = off
            while end < capacity and not used[end]:
                end += 1
            model_free.append((off, end - off))
            off = end
        else:
            off += 1
    assert [(int(a), int(b)) for a, b in free] == model_free


def test_free_everything_restores_one_range(lib):
    sizes = [100, 200, 50, 400, 10]
    ops = list(sizes)
    out, _ = run(lib, 1000, ops, [0] * 5, [0] * 5)
    order = [3, 0, 4, 2, 1]
    ops2 = ops + [-(j + 1) for j in order]
    offs2 = [0] * 5 + [int(out[j]) for j in order]
    sizes2 = [0] * 5 + [sizes[j] for j in order]
    _, free = run(lib, 1000, ops2, offs2, sizes2)
    assert free == [(0, 1000)]


def test_exhaustion(lib):
    out, free = run(lib, 100, [60, 60, 40], [0] * 3, [0] * 3)
    assert list(out) == [0, -1, 60] and free == []
