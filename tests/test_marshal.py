"""The packed descriptor table of a batch (one structured array, pointers
into a few concatenated buffers) describes each problem exactly as the
per-problem descriptor does; runs on CPU."""
import ctypes as C

import numpy as np
import pytest

from madsdp_gpu import _lib, generators as g
from madsdp_gpu.model import BlockConstraints, Model
from madsdp_gpu.solver import _Marshalled, _MarshalledBatch
from problems import build


def read_desc(d):
    """Every array a msdp_problem_desc points to, copied out."""
    nb, m, ns = d.nblocks, d.m, d.ns
    out = {"nblocks": nb, "m": m, "ns": ns, "b": np.ctypeslib.as_array(d.b, (m,)).copy() if m else np.zeros(0),
           "d_lin": np.ctypeslib.as_array(d.d_lin, (ns,)).copy() if ns else np.zeros(0),
           "C_lin": np.ctypeslib.as_array(d.C_lin, (m * ns,)).copy() if m * ns else np.zeros(0), "blocks": []}
    for i in range(nb):
        n, nnz = d.sides[i], d.A_nnz[i]
        blk = {"n": n, "nnz": nnz, "C": np.ctypeslib.as_array(d.C[i], (n * n,)).copy()}
        for key, ptr in (("con", d.A_con), ("row", d.A_row), ("col", d.A_col), ("val", d.A_val)):
            blk[key] = np.ctypeslib.as_array(ptr[i], (nnz,)).copy() if nnz else np.zeros(0)
        out["blocks"].append(blk)
    return out


def same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        if k == "blocks":
            assert len(a[k]) == len(b[k])
            for x, y in zip(a[k], b[k]):
                same(x, y)
        elif isinstance(a[k], np.ndarray):
            assert np.array_equal(a[k], b[k]), k
        else:
            assert a[k] == b[k], k


def mixed_models():
    # a block with no constraint entries and a problem with no PSD block
    empty = Model([np.eye(3)], [BlockConstraints(3, 2, [], [], [], [])], np.array([1.0, 2.0]), sides=[3])
    lp = Model([], [], np.array([1.0]), d_lin=np.array([1.0, 2.0]), C_lin=np.array([[1.0, 1.0]]))
    return [g.sos_hankel(5, seed=1), build("mixed_lp"), g.dense_random([6, 3, 2], 4, 9, seed=2),
            g.maxcut(10, 0.3, seed=3), empty, build("trivial_2x2"), lp, g.sos_hankel(9, seed=4)]


def test_packed_table_equals_per_problem_descriptors():
    models = mixed_models()
    packed = _MarshalledBatch(models)
    assert packed.count == len(models) and packed.table.itemsize == C.sizeof(_lib.ProblemDesc)
    for k, m in enumerate(models):
        single = _Marshalled(m)  # owns the buffers its descriptor points to
        same(read_desc(packed.descs(k)[0]), read_desc(single.desc))


def test_no_copies_of_model_arrays():
    models = mixed_models()
    packed = _MarshalledBatch(models)
    assert packed._keep == []
    d = packed.descs(0)[0]
    A = models[0].A[0]
    assert C.addressof(d.A_con[0].contents) == A.con.ctypes.data
    assert C.addressof(d.A_val[0].contents) == A.val.ctypes.data


def test_other_layouts_are_converted():
    m = g.dense_random([5, 3], 3, 6, seed=1)
    m.C_lin = np.ascontiguousarray(m.C_lin)  # row-major: converted
    m.A[1].con = m.A[1].con.astype(np.int64)  # wider indices: converted
    ref = _Marshalled(m)
    packed = _MarshalledBatch([m])
    assert len(packed._keep) == 2
    same(read_desc(packed.descs(0)[0]), read_desc(ref.desc))


def test_descs_range_checked():
    packed = _MarshalledBatch(mixed_models()[:2])
    with pytest.raises(IndexError):
        packed.descs(3)


def test_table_keeps_the_models_alive():
    import gc
    packed = _MarshalledBatch([g.sos_hankel(6, seed=9), build("mixed_lp")])
    gc.collect()
    for _ in range(50):  # churn the allocator
        np.ones(1000)
    d = read_desc(packed.descs(0)[0])
    ref = g.sos_hankel(6, seed=9)
    assert np.array_equal(d["blocks"][0]["con"], ref.A[0].con) and np.array_equal(d["b"], ref.b)
