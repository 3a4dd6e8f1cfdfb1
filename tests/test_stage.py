"""Host staging of a batch (madsdp.jl_gb300/csrc/stage.h), compiled with g++
into a CPU harness (tests/native/stage_check.cpp): every staged array equals
a NumPy restatement of the layout, the result does not depend on the number
of threads, unsorted entries are sorted and out-of-range entries are
rejected; runs on CPU."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from madsdp_gpu import _lib
from madsdp_gpu import generators as g
from madsdp_gpu.solver import _MarshalledBatch
from problems import build

HERE = os.path.dirname(os.path.abspath(__file__))
STRUCT_GENERAL, STRUCT_HANKEL, STRUCT_DENSE = 0, 1, 2


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("stage") / "stage_check.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "native", "stage_check.cpp"), "-lpthread"], check=True)
    lib = C.CDLL(so)
    P = C.POINTER
    lib.stage_sizes.argtypes = [P(_lib.ProblemDesc), C.c_int32, P(C.c_int64)]
    lib.stage_sizes.restype = None
    lib.stage_run.argtypes = [P(_lib.ProblemDesc), C.c_int32, C.c_int, P(C.c_double), P(C.c_int32), P(C.c_int32),
                              P(C.c_double), P(C.c_int32), P(C.c_double), P(C.c_int64), P(C.c_int64), P(C.c_int32),
                              P(C.c_double)]
    lib.stage_run.restype = C.c_int
    return lib


def stage(lib, mb, threads):
    sizes = np.zeros(4, dtype=np.int64)
    lib.stage_sizes(mb.descs(), mb.count, sizes.ctypes.data_as(C.POINTER(C.c_int64)))
    n_dd, n_ent, n_ptr, n_blk = (int(v) for v in sizes)
    # garbage everywhere: staging must write every element it owns
    out = {"dd": np.full(max(n_dd, 1), np.nan), "erow": np.full(max(n_ent, 1), -7, np.int32),
           "ecol": np.full(max(n_ent, 1), -7, np.int32), "eval": np.full(max(n_ent, 1), np.nan),
           "pcon": np.full(max(n_ent, 1), -7, np.int32), "pval": np.full(max(n_ent, 1), np.nan),
           "ptr": np.full(max(n_ptr, 1), -7, np.int64), "off": np.zeros((max(n_blk, 1), 4), np.int64),
           "structure": np.full(max(n_blk, 1), -1, np.int32), "cnorm": np.full(max(n_blk, 1), np.nan)}
    ptrs = [out[k].ctypes.data_as(C.POINTER({np.float64: C.c_double, np.int32: C.c_int32,
                                             np.int64: C.c_int64}[out[k].dtype.type]))
            for k in ("dd", "erow", "ecol", "eval", "pcon", "pval", "ptr", "off", "structure", "cnorm")]
    ok = lib.stage_run(mb.descs(), mb.count, threads, *ptrs)
    out["sizes"] = (n_dd, n_ent, n_ptr, n_blk)
    return ok, out


def expected_block(A, n, m):
    """Entries by (constraint, column, row) and by position (constraint order)."""
    con, row, col, val = (np.asarray(x) for x in (A.con, A.row, A.col, A.val))
    o = np.lexsort((row, col, con))
    cptr = np.concatenate([[0], np.cumsum(np.bincount(con, minlength=m))])
    pos = row + col * n
    # stable by position, within a position in constraint order
    po = o[np.argsort(pos[o], kind="stable")]
    pptr = np.concatenate([[0], np.cumsum(np.bincount(pos, minlength=n * n))])
    return row[o], col[o], val[o], cptr, con[po], val[po], pptr


def check_against_numpy(models, out):
    dd = out["dd"]
    k = 0
    for model in models:
        # the problem's data range starts at the first block's offset minus its own length, padded
        m, ns = model.m, model.ns
        blk_offsets = out["off"][k:k + model.nblocks]
        if model.nblocks:
            start = blk_offsets[0][0] - ((m + ns + m * ns + 3 + 3) // 4) * 4
        else:
            start = None
        if start is not None:
            dat = dd[start:start + m + ns + m * ns + 3]
            assert np.array_equal(dat[:m], model.b)
            assert np.array_equal(dat[m:m + ns], model.d_lin)
            assert np.array_equal(dat[m + ns:m + ns + m * ns], np.asarray(model.C_lin).ravel(order="F"))
            assert dat[-3] == (np.abs(model.b).max() if m else 0.0)
            assert dat[-2] == (np.abs(model.d_lin).max() if ns else 0.0)
            assert dat[-1] == max(np.abs(c).max() for c in model.C)
        for i, (n, A) in enumerate(zip(model.sides, model.A)):
            cdat, ent, conptr, posptr = (int(v) for v in out["off"][k])
            assert np.array_equal(dd[cdat:cdat + n * n], np.asarray(model.C[i]).ravel(order="F"))
            assert out["cnorm"][k] == np.abs(model.C[i]).max()
            er, ec, ev, cptr, pc, pv, pptr = expected_block(A, n, m)
            e = slice(ent, ent + A.nnz)
            assert np.array_equal(out["erow"][e], er) and np.array_equal(out["ecol"][e], ec)
            assert np.array_equal(out["eval"][e], ev)
            assert np.array_equal(out["ptr"][conptr:conptr + m + 1], cptr)
            assert np.array_equal(out["pcon"][e], pc) and np.array_equal(out["pval"][e], pv)
            assert np.array_equal(out["ptr"][posptr:posptr + n * n + 1], pptr)
            k += 1
    # padding of the data arena is zeroed, nothing is left unwritten
    assert not np.isnan(dd[:out["sizes"][0]]).any()


def models_mix():
    return [g.sos_hankel(5, seed=1), build("mixed_lp"), g.dense_random([6, 3, 2], 4, 9, seed=2),
            g.maxcut(10, 0.3, seed=3), build("trivial_2x2"), g.sos_hankel(12, seed=4), build("maxcut_weighted4")] * 7


@pytest.mark.parametrize("threads", [1, 3, 16])
def test_stage_matches_numpy(harness, threads):
    models = models_mix()
    ok, out = stage(harness, _MarshalledBatch(models), threads)
    assert ok == 1
    check_against_numpy(models, out)


def test_thread_count_does_not_change_the_result(harness):
    models = models_mix()
    mb = _MarshalledBatch(models)
    _, a = stage(harness, mb, 1)
    _, b = stage(harness, mb, 8)
    n_dd, n_ent, n_ptr, n_blk = a["sizes"]
    for key, n in (("dd", n_dd), ("erow", n_ent), ("ecol", n_ent), ("eval", n_ent), ("pcon", n_ent),
                   ("pval", n_ent), ("ptr", n_ptr), ("structure", n_blk), ("cnorm", n_blk)):
        assert np.array_equal(a[key][:n], b[key][:n]), key


def test_structure_detection(harness):
    models = [g.sos_hankel(7, seed=1), g.maxcut(12, 0.3, seed=2), g.dense_random([8], 0, 30, seed=3)]
    ok, out = stage(harness, _MarshalledBatch(models), 2)
    assert ok == 1
    assert out["structure"][0] == STRUCT_HANKEL
    assert out["structure"][1] == STRUCT_GENERAL
    assert out["structure"][2] in (STRUCT_GENERAL, STRUCT_DENSE)


def test_unsorted_entries_are_sorted(harness):
    models = [g.sos_hankel(6, seed=1), g.dense_random([5, 4], 2, 7, seed=5)]
    rng = np.random.default_rng(0)
    # shuffle the entries of every block in place (the descriptors point to these arrays)
    for A in (A for m in models for A in m.A):
        perm = rng.permutation(A.nnz)
        for arr in (A.con, A.row, A.col, A.val):
            arr[:] = arr[perm]
    ok, out = stage(harness, _MarshalledBatch(models), 2)
    assert ok == 1
    check_against_numpy(models, out)


def test_out_of_range_entry_rejected(harness):
    models = models_mix()[:20]
    models[13] = g.maxcut(10, 0.3, seed=3)
    models[13].A[0].row[2] = 10_000
    ok, _ = stage(harness, _MarshalledBatch(models), 4)
    assert ok == 0
