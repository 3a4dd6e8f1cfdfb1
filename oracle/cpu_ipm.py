"""Build and ctypes binding of the compiled CPU restatement (cpu_ipm.cpp).

TEST INFRASTRUCTURE ONLY, like ``madsdp_oracle``: it times the CPU baseline
of the batched workloads without interpreter overhead and checks GPU
results at sizes the NumPy restatement is slow on.  It restates the
PrimalDual path (NT or HKM, EigenStep or CholeskyBacktrack, Mehrotra or
AdaptiveMu, with DenseCholesky and ScaledIdentity) of MadSDP.jl
(src/solver.jl, src/primal_dual.jl, src/directions.jl, src/step.jl,
src/blocks.jl) following ``madsdp_oracle`` step by step, and
``tests/test_oracle_cpp.py`` checks it against that module.

    build()                         g++ -O3 into oracle/lib/libmsdp_cpu.so
    solve(model, **options)         one solve, a dict of the stats; options:
                                    direction / step / centering (component
                                    objects of madsdp_oracle) and the
                                    options of src/options.jl
    solve_many(models, threads, seconds, **options)
    symeig(A)                       eigenvalues, eigenvectors (test hook)
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "cpu_ipm.cpp")
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libmsdp_cpu.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the library when it is missing or older than its sources."""
    header = os.path.join(ROOT, "include", "madsdp_gpu.h")
    newest = max(os.path.getmtime(SRC), os.path.getmtime(header))
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["g++", "-O3", "-std=c++17", "-shared", "-fPIC", "-Wall", "-o", tmp, SRC, "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def load():
    global _lib
    if _lib is not None:
        return _lib
    from madsdp_gpu import _lib as G
    build()
    try:
        lib = C.CDLL(LIB_PATH)
    except OSError:  # a library built for another machine: rebuild here
        build(force=True)
        lib = C.CDLL(LIB_PATH)
    P = C.POINTER
    lib.msdp_cpu_default_options.restype = None
    lib.msdp_cpu_default_options.argtypes = [P(G.Options)]
    lib.msdp_cpu_solve.restype = C.c_int32
    lib.msdp_cpu_solve.argtypes = [P(G.ProblemDesc), P(G.Components), P(G.Options), P(G.Stats)]
    lib.msdp_cpu_solve_many.restype = C.c_int32
    lib.msdp_cpu_solve_many.argtypes = [P(G.ProblemDesc), C.c_int32, C.c_int32, C.c_double, P(G.Components),
                                        P(G.Options), P(G.Stats)]
    lib.msdp_cpu_default_components.restype = None
    lib.msdp_cpu_default_components.argtypes = [P(G.Components)]
    lib.msdp_cpu_symeig.restype = C.c_int32
    lib.msdp_cpu_symeig.argtypes = [C.c_int32, P(C.c_double), P(C.c_double), P(C.c_double)]
    _lib = lib
    return lib


# component keyword -> (field, value) of msdp_components
_COMPONENTS = {
    ("direction", "NT"): ("direction", 0), ("direction", "HKM"): ("direction", 1),
    ("step", "EigenStep"): ("step", 0), ("step", "CholeskyBacktrack"): ("step", 1),
    ("centering", "Mehrotra"): ("centering", 0), ("centering", "AdaptiveMu"): ("centering", 1),
}


def _options(lib, options):
    """(msdp_components, msdp_options) from keywords: direction / step /
    centering given as component objects of madsdp_oracle (or their class
    names), the other keywords as options of src/options.jl."""
    from madsdp_gpu import _lib as G
    comp, o = G.Components(), G.Options()
    lib.msdp_cpu_default_components(C.byref(comp))
    lib.msdp_cpu_default_options(C.byref(o))
    for k, v in options.items():
        if k in ("direction", "step", "centering"):
            name = v if isinstance(v, str) else type(v).__name__
            if (k, name) not in _COMPONENTS:
                raise ValueError(f"the compiled restatement has no {k} {name}")
            setattr(comp, *_COMPONENTS[(k, name)])
            for field in ("tau", "shrink", "boundary", "sigma_exponent", "initial_ratio", "ratio"):
                if hasattr(v, field):
                    setattr(comp, field, getattr(v, field))
        elif hasattr(o, k):
            setattr(o, k, v)
        else:
            raise TypeError(f"unknown option {k}")
    return comp, o


def _stats(s) -> dict:
    return {k: getattr(s, k) for k, _ in s._fields_}


def solve(model, **options) -> dict:
    from madsdp_gpu.solver import _Marshalled
    lib = load()
    mm = _Marshalled(model)
    st = _stats_struct()
    comp, opts = _options(lib, options)
    rc = lib.msdp_cpu_solve(C.byref(mm.desc), C.byref(comp), C.byref(opts), C.byref(st))
    if rc != 0:
        raise ValueError(f"msdp_cpu_solve returned {rc}")
    return _stats(st)


def _stats_struct():
    from madsdp_gpu import _lib as G
    return G.Stats()


class Prepared:
    """Marshalled problems, kept alive across timed calls of solve_many."""

    def __init__(self, models: Sequence):
        from madsdp_gpu import _lib as G
        from madsdp_gpu.solver import _MarshalledBatch
        self.marsh = _MarshalledBatch(list(models))
        self.stats = (G.Stats * self.marsh.count)()

    def __len__(self):
        return self.marsh.count


def solve_many(models, threads: int, seconds: float = 0.0, start: int = 0, count: Optional[int] = None,
               **options) -> List[Optional[dict]]:
    """Solve models[start:start+count] on `threads` host threads, stopping
    new solves after `seconds` (> 0).  `models` is a sequence of models or a
    ``Prepared``.  Returns one stats dict per problem, None for the ones not
    started."""
    lib = load()
    prep = models if isinstance(models, Prepared) else Prepared(models)
    n = len(prep) - start if count is None else count
    if start < 0 or n < 0 or start + n > len(prep):
        raise ValueError("range outside the prepared problems")
    for i in range(start, start + n):
        prep.stats[i].status = -2
    stats = C.cast(C.byref(prep.stats, start * C.sizeof(prep.stats._type_)), C.POINTER(prep.stats._type_))
    comp, opts = _options(lib, options)
    lib.msdp_cpu_solve_many(prep.marsh.descs(start), n, threads, seconds, C.byref(comp), C.byref(opts), stats)
    out = []
    for i in range(start, start + n):
        s = prep.stats[i]
        out.append(None if s.status == -2 else _stats(s))
    return out


def symeig(A):
    lib = load()
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    w = np.zeros(n)
    V = np.zeros((n, n), order="F")
    dp = C.POINTER(C.c_double)
    rc = lib.msdp_cpu_symeig(n, A.ctypes.data_as(dp), w.ctypes.data_as(dp), V.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"msdp_cpu_symeig returned {rc}")
    return w, V
