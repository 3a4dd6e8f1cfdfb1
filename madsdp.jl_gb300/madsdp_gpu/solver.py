"""Host-side mirror of MadSDP's solver API over the C ABI.

``MadSDPSolver(model; components..., options...)`` / ``solve()`` /
``madsdp(model)`` follow src/solver.jl:55-160,385-404; ``Batch`` solves
many models in one persistent launch (one CTA per problem at a time).
Errors follow the reference: invalid configurations raise ``ValueError``
(Julia ``ArgumentError``), an impossible initial point raises
``RuntimeError`` (Julia ``ErrorException``).
"""

from __future__ import annotations

import ctypes as C
import math
import warnings
import weakref
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from .components import (DenseCholesky, DualCentering, DualShift, EigenStep, InitialPoint, MadNLPSchur, Mehrotra,
                         NT, Options, PRECISIONS, PrimalDual, QRSchur, ScaledIdentity, Status)
from .model import Model

__all__ = ["Context", "Batch", "MadSDPSolver", "madsdp", "GPUError", "default_context"]

P = C.POINTER
f64p = P(C.c_double)


class GPUError(RuntimeError):
    """A CUDA or library error reported through the C ABI."""


_default_ctx = None


class Context:
    """One CUDA device and one stream (msdp_context)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.msdp_context_create(device, C.byref(h))
        if rc != 0:
            raise GPUError(f"msdp_context_create failed ({_lib.ERRORS.get(rc, rc)})")
        self.h = h
        self.device = device
        self._children = weakref.WeakSet()

    def adopt(self, child):
        """Register a batch or server so that closing the context closes it first."""
        self._children.add(child)

    @property
    def stream_handle(self) -> int:
        """The cudaStream_t of this context as an integer."""
        return int(self.lib.msdp_context_stream(self.h) or 0)

    def error(self) -> str:
        return self.lib.msdp_last_error(self.h).decode()

    def check(self, rc: int, what: str):
        if rc == 0:
            return
        msg = self.error()
        if rc == -1:
            raise ValueError(msg)
        if rc == -5:
            raise RuntimeError(msg)
        if rc == -4:
            raise NotImplementedError(msg)
        raise GPUError(f"{what}: {_lib.ERRORS.get(rc, rc)}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            for child in list(getattr(self, "_children", ())):
                child.close()
            self.lib.msdp_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _ptr(a: np.ndarray, ctype=C.c_double):
    return a.ctypes.data_as(P(ctype))


def _components(algorithm, initial_point, schur, precision) -> _lib.Components:
    c = _lib.Components()
    _lib.load().msdp_default_components(C.byref(c))
    if isinstance(algorithm, DualCentering):
        c.algorithm = 1
        c.dc_beta, c.dc_delta = algorithm.beta, algorithm.delta
        c.dc_A = math.nan if algorithm.A is None else float(algorithm.A)
        c.centering_max_iter = algorithm.centering_max_iter
    else:
        c.algorithm = 0
        d, s, ce = algorithm.direction, algorithm.step, algorithm.centering
        c.direction = d.code
        c.step = s.code
        if isinstance(s, EigenStep):
            c.tau = s.tau
        else:
            c.shrink, c.boundary = s.shrink, s.boundary
        c.centering = ce.code
        if isinstance(ce, Mehrotra):
            c.sigma_exponent = ce.sigma_exponent
        else:
            c.initial_ratio, c.ratio = ce.initial_ratio, ce.ratio
    c.initial_point = initial_point.code
    if isinstance(initial_point, ScaledIdentity):
        c.scale = 0.0 if initial_point.scale is None else initial_point.scale
    elif isinstance(initial_point, DualShift):
        c.initial_shift, c.max_shift = initial_point.initial_shift, initial_point.max_shift
    c.schur = schur.code
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
    c.precision = PRECISIONS[precision]
    return c


def _options(opt: Options) -> _lib.Options:
    o = _lib.Options()
    _lib.load().msdp_default_options(C.byref(o))
    o.tol, o.max_iter, o.max_wall_time = opt.tol, opt.max_iter, opt.max_wall_time
    o.mu_min, o.regularize_schur, o.max_schur_reg = opt.mu_min, opt.regularize_schur, opt.max_schur_reg
    o.datasparsity, o.switch_tol, o.mixed_refine = opt.datasparsity, opt.switch_tol, opt.mixed_refine
    return o


class _Marshalled:
    """Keeps the numpy buffers of one problem alive while the C call runs."""

    def __init__(self, model: Model):
        nb = model.nblocks
        self.sides = np.array(model.sides, dtype=np.int32)
        self.C = [np.asfortranarray(c, dtype=np.float64) for c in model.C]
        self.nnz = np.array([a.nnz for a in model.A], dtype=np.int64)
        self.con = [np.ascontiguousarray(a.con, dtype=np.int32) for a in model.A]
        self.row = [np.ascontiguousarray(a.row, dtype=np.int32) for a in model.A]
        self.col = [np.ascontiguousarray(a.col, dtype=np.int32) for a in model.A]
        self.val = [np.ascontiguousarray(a.val, dtype=np.float64) for a in model.A]
        self.b = np.ascontiguousarray(model.b, dtype=np.float64)
        self.d = np.ascontiguousarray(model.d_lin, dtype=np.float64)
        self.Cl = np.asfortranarray(model.C_lin, dtype=np.float64)
        self.Cp = (f64p * max(nb, 1))(*[_ptr(c) for c in self.C])
        self.conp = (P(C.c_int32) * max(nb, 1))(*[_ptr(a, C.c_int32) for a in self.con])
        self.rowp = (P(C.c_int32) * max(nb, 1))(*[_ptr(a, C.c_int32) for a in self.row])
        self.colp = (P(C.c_int32) * max(nb, 1))(*[_ptr(a, C.c_int32) for a in self.col])
        self.valp = (f64p * max(nb, 1))(*[_ptr(a) for a in self.val])
        d = _lib.ProblemDesc()
        d.nblocks, d.m, d.ns = nb, model.m, model.ns
        d.sides = _ptr(self.sides, C.c_int32)
        d.C = self.Cp
        d.A_nnz = _ptr(self.nnz, C.c_int64)
        d.A_con, d.A_row, d.A_col, d.A_val = self.conp, self.rowp, self.colp, self.valp
        d.b, d.d_lin, d.C_lin = _ptr(self.b), _ptr(self.d), _ptr(self.Cl)
        self.desc = d


def _offsets(sizes: np.ndarray) -> np.ndarray:
    """Exclusive prefix sum, as uint64 element offsets."""
    off = np.zeros(sizes.size, dtype=np.uint64)
    if sizes.size > 1:
        np.cumsum(sizes[:-1].astype(np.uint64), out=off[1:])
    return off


def _desc_dtype() -> np.dtype:
    names = [f for f, _ in _lib.ProblemDesc._fields_]
    formats = [np.int32 if t is C.c_int32 else np.uint64 for _, t in _lib.ProblemDesc._fields_]
    offsets = [getattr(_lib.ProblemDesc, f).offset for f in names]
    return np.dtype({"names": names, "formats": formats, "offsets": offsets,
                     "itemsize": C.sizeof(_lib.ProblemDesc)})


def _addr(a: np.ndarray) -> int:
    return a.__array_interface__["data"][0]


class _MarshalledBatch:
    """The table of msdp_problem_desc of many problems, built as one numpy
    structured array whose pointers are the addresses of the models' own
    arrays (a Model stores them in the layout of the C ABI: int32 indices,
    contiguous float64 values, column-major C_lin), so nothing is copied.
    An array in another layout is converted and the copy kept here.  C is
    passed as stored: a C-ordered buffer read column-major is C', and
    <C, X> for symmetric X and sym(C - A*(y)) are the same for C and C'.
    Holds every buffer the descriptors point to while the C call runs."""

    def __init__(self, models: Sequence[Model]):
        n = len(models)
        self._keep = []
        # the descriptors point into these models' arrays: keep them alive
        self.models = list(models)

        def as_is(a, dtype, fortran=False):
            ok = a.dtype == dtype and (a.flags.f_contiguous if fortran else a.flags.c_contiguous)
            if not ok:
                a = np.asfortranarray(a, dtype=dtype) if fortran else np.ascontiguousarray(a, dtype=dtype)
                self._keep.append(a)
            return _addr(a)

        def dense(c):
            if c.dtype == np.float64 and (c.flags.c_contiguous or c.flags.f_contiguous):
                return _addr(c)
            return as_is(c, np.float64, fortran=True)

        nb = np.fromiter((mm.nblocks for mm in models), dtype=np.int64, count=n)
        ms = np.fromiter((mm.m for mm in models), dtype=np.int64, count=n)
        ns = np.fromiter((mm.ns for mm in models), dtype=np.int64, count=n)
        blocks = [A for mm in models for A in mm.A]
        nblk = len(blocks)
        self.sides = np.zeros(max(nblk, 1), dtype=np.int32)
        self.nnz = np.zeros(max(nblk, 1), dtype=np.int64)
        self.Cp, self.conp, self.rowp, self.colp, self.valp = (np.zeros(max(nblk, 1), dtype=np.uint64)
                                                                for _ in range(5))
        if nblk:
            self.sides[:] = [s for mm in models for s in mm.sides]
            self.nnz[:] = [A.val.size for A in blocks]
            self.Cp[:] = [dense(c) for mm in models for c in mm.C]
            self.conp[:] = [as_is(A.con, np.int32) for A in blocks]
            self.rowp[:] = [as_is(A.row, np.int32) for A in blocks]
            self.colp[:] = [as_is(A.col, np.int32) for A in blocks]
            self.valp[:] = [as_is(A.val, np.float64) for A in blocks]
        boff = _offsets(nb)
        d = np.zeros(n, dtype=_desc_dtype())
        d["nblocks"], d["m"], d["ns"] = nb, ms, ns
        d["sides"] = np.uint64(_addr(self.sides)) + np.uint64(4) * boff
        d["A_nnz"] = np.uint64(_addr(self.nnz)) + np.uint64(8) * boff
        for field, arr in (("C", self.Cp), ("A_con", self.conp), ("A_row", self.rowp), ("A_col", self.colp),
                           ("A_val", self.valp)):
            d[field] = np.uint64(_addr(arr)) + np.uint64(8) * boff
        d["b"] = [as_is(mm.b, np.float64) for mm in models]
        d["d_lin"] = [as_is(mm.d_lin, np.float64) for mm in models]
        d["C_lin"] = [as_is(mm.C_lin, np.float64, fortran=True) for mm in models]
        self.table = d
        self.count = n

    def descs(self, start: int = 0):
        """Pointer to the descriptor of problem `start` (and those after it)."""
        if not 0 <= start <= self.count:
            raise IndexError(start)
        return C.cast(self.table.ctypes.data + start * self.table.itemsize, P(_lib.ProblemDesc))


class Batch:
    """Many problems resident on one GPU, solved by one persistent launch."""

    def __init__(self, models: Sequence[Model], algorithm=None, direction=None, step=None,
                 centering=None, initial_point=None, schur=None, precision: str = "fp64",
                 context: Optional[Context] = None, **options):
        self.ctx = context or default_context()
        self.lib = self.ctx.lib
        direction = NT() if direction is None else direction
        step = EigenStep() if step is None else step
        centering = Mehrotra() if centering is None else centering
        self.algorithm = PrimalDual(direction, step, centering) if algorithm is None else algorithm
        if initial_point is None:
            initial_point = DualShift() if isinstance(self.algorithm, DualCentering) else ScaledIdentity()
        self.initial_point = initial_point
        self.schur = DenseCholesky() if schur is None else schur
        self.precision = precision
        self.opt = Options(**options)
        self.models = list(models)
        if not self.models:
            raise ValueError("a batch needs at least one model")
        if isinstance(self.schur, QRSchur):
            if not (isinstance(self.algorithm, PrimalDual) and isinstance(self.algorithm.direction, NT)):
                raise ValueError("QRSchur requires PrimalDual with the NT direction.")
        if isinstance(self.algorithm, DualCentering):
            for m in self.models:
                if m.ns > 0:
                    raise RuntimeError("MadSDP: `DualCentering` does not support scalar (LP) blocks yet.")
                if m.nblocks == 0:
                    raise RuntimeError("MadSDP: `DualCentering` needs at least one PSD block.")
        marsh = _MarshalledBatch(self.models)
        comp = _components(self.algorithm, self.initial_point, self.schur, precision)
        opts = _options(self.opt)
        h = C.c_void_p()
        rc = self.lib.msdp_batch_create(self.ctx.h, marsh.descs(), marsh.count, C.byref(comp), C.byref(opts),
                                        C.byref(h))
        self.ctx.check(rc, "msdp_batch_create")
        self.h = h
        self.ctx.adopt(self)
        self.nprob = marsh.count
        if isinstance(self.initial_point, InitialPoint):
            for p in range(self.nprob):
                self.set_initial_point(p, self.initial_point)

    # --- lifecycle -------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.msdp_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def device_bytes(self) -> int:
        return int(self.lib.msdp_batch_device_bytes(self.h))

    @property
    def launch_count(self) -> int:
        return int(self.lib.msdp_batch_launch_count(self.h))

    def set_initial_point(self, p: int, ip: InitialPoint):
        m = self.models[p]
        Xs = [np.asfortranarray(x, dtype=np.float64) for x in ip.X]
        Xp = (f64p * max(len(Xs), 1))(*[_ptr(x) for x in Xs])
        y = np.ascontiguousarray(ip.y, dtype=np.float64)
        x = None if ip.x is None else np.ascontiguousarray(ip.x, dtype=np.float64)
        rc = self.lib.msdp_batch_set_initial_point(self.h, p, Xp, _ptr(y), None if x is None else _ptr(x))
        self.ctx.check(rc, "msdp_batch_set_initial_point")

    def set_iterate(self, p: int, X=None, S=None, y=None, x=None, z=None):
        nb = self.models[p].nblocks
        keep = []

        def mats(Ms):
            if Ms is None:
                return None
            arrs = [np.asfortranarray(a, dtype=np.float64) for a in Ms]
            keep.append(arrs)
            return (f64p * max(nb, 1))(*[_ptr(a) for a in arrs])

        def vec(v):
            if v is None:
                return None
            a = np.ascontiguousarray(v, dtype=np.float64)
            keep.append(a)
            return _ptr(a)

        rc = self.lib.msdp_batch_set_iterate(self.h, p, mats(X), mats(S), vec(y), vec(x), vec(z))
        self.ctx.check(rc, "msdp_batch_set_iterate")

    def initialize(self):
        self.ctx.check(self.lib.msdp_batch_initialize(self.h), "msdp_batch_initialize")

    def iterate(self, max_iterations: int = 0, sync: bool = True):
        self.ctx.check(self.lib.msdp_batch_iterate(self.h, max_iterations), "msdp_batch_iterate")
        if sync:
            self.synchronize()

    def synchronize(self):
        self.ctx.check(self.lib.msdp_batch_synchronize(self.h), "msdp_batch_synchronize")

    def solve(self):
        self.ctx.check(self.lib.msdp_batch_solve(self.h), "msdp_batch_solve")
        return self

    def launch_initialize(self):
        """Enqueue initialize! on the context stream; returns at once."""
        self.ctx.check(self.lib.msdp_batch_launch_initialize(self.h), "msdp_batch_launch_initialize")

    @property
    def upload_bytes(self) -> int:
        return int(self.lib.msdp_batch_upload_bytes(self.h))

    def launch_solve(self):
        """Enqueue initialize + solve on the context stream; returns at once."""
        self.ctx.check(self.lib.msdp_batch_launch_solve(self.h), "msdp_batch_launch_solve")

    # --- results -----------------------------------------------------------------
    def stats(self, p: int) -> dict:
        s = _lib.Stats()
        self.ctx.check(self.lib.msdp_batch_get_stats(self.h, p, C.byref(s)), "msdp_batch_get_stats")
        return _stats_dict(s)

    def all_stats(self) -> List[dict]:
        arr = (_lib.Stats * self.nprob)()
        self.ctx.check(self.lib.msdp_batch_get_all_stats(self.h, arr), "msdp_batch_get_all_stats")
        return [_stats_dict(s) for s in arr]

    def solution(self, p: int):
        m = self.models[p]
        X = [np.zeros((n, n), order="F") for n in m.sides]
        Xp = (f64p * max(len(X), 1))(*[_ptr(a) for a in X])
        y, x, z = np.zeros(m.m), np.zeros(m.ns), np.zeros(m.ns)
        rc = self.lib.msdp_batch_get_solution(self.h, p, Xp, _ptr(y), _ptr(x), _ptr(z))
        self.ctx.check(rc, "msdp_batch_get_solution")
        return [np.ascontiguousarray(a) for a in X], y, x, z

    def all_solutions(self) -> list:
        """(X blocks, y, x, z) of every problem from one packed download;
        the arrays are views of one host buffer."""
        total = int(self.lib.msdp_batch_solution_size(self.h))
        buf = np.empty(max(total, 1))
        rc = self.lib.msdp_batch_get_all_solutions(self.h, _ptr(buf))
        self.ctx.check(rc, "msdp_batch_get_all_solutions")
        out, off = [], 0
        for m in self.models:
            X = []
            for n in m.sides:
                X.append(buf[off:off + n * n].reshape(n, n, order="F"))
                off += n * n
            y = buf[off:off + m.m]
            off += m.m
            x, z = buf[off:off + m.ns], buf[off + m.ns:off + 2 * m.ns]
            off += 2 * m.ns
            out.append((X, y, x, z))
        return out

    def trajectory(self, p: int) -> List[dict]:
        cap = self.opt.max_iter + 2
        arr = (_lib.IterRecord * cap)()
        cnt = C.c_int32()
        rc = self.lib.msdp_batch_get_trajectory(self.h, p, arr, cap, C.byref(cnt))
        self.ctx.check(rc, "msdp_batch_get_trajectory")
        return [{k: getattr(arr[i], k) for k, _ in _lib.IterRecord._fields_} for i in range(min(cnt.value, cap))]

    def profile(self, p: int) -> dict:
        """Device cycle counters per phase and work counters of problem p."""
        buf = (C.c_double * 128)()
        n = self.lib.msdp_batch_get_profile(self.h, p, buf, 128)
        if n < 0:
            self.ctx.check(n, "msdp_batch_get_profile")
        return {self.lib.msdp_profile_field_name(i).decode(): buf[i] for i in range(n)}

    # --- component-granular steps (identity tests) -------------------------------
    def update_residuals(self):
        self.ctx.check(self.lib.msdp_batch_update_residuals(self.h), "msdp_batch_update_residuals")

    def prepare(self) -> np.ndarray:
        ok = np.zeros(self.nprob, dtype=np.int32)
        self.ctx.check(self.lib.msdp_batch_prepare(self.h, _ptr(ok, C.c_int32)), "msdp_batch_prepare")
        return ok.astype(bool)

    def solve_directions(self, mu: float, corrected: bool):
        self.ctx.check(self.lib.msdp_batch_solve_directions(self.h, float(mu), int(bool(corrected))),
                       "msdp_batch_solve_directions")

    def correction(self):
        self.ctx.check(self.lib.msdp_batch_correction(self.h), "msdp_batch_correction")

    def directions(self, p: int):
        m = self.models[p]
        dX = [np.zeros((n, n), order="F") for n in m.sides]
        dS = [np.zeros((n, n), order="F") for n in m.sides]
        dXp = (f64p * max(len(dX), 1))(*[_ptr(a) for a in dX])
        dSp = (f64p * max(len(dS), 1))(*[_ptr(a) for a in dS])
        dy, dx, dz = np.zeros(m.m), np.zeros(m.ns), np.zeros(m.ns)
        rc = self.lib.msdp_batch_get_directions(self.h, p, dXp, dSp, _ptr(dy), _ptr(dx), _ptr(dz))
        self.ctx.check(rc, "msdp_batch_get_directions")
        return [np.ascontiguousarray(a) for a in dX], [np.ascontiguousarray(a) for a in dS], dy, dx, dz

    def residuals(self, p: int):
        m = self.models[p]
        Rd = [np.zeros((n, n), order="F") for n in m.sides]
        Rdp = (f64p * max(len(Rd), 1))(*[_ptr(a) for a in Rd])
        Rp, Rdl = np.zeros(m.m), np.zeros(m.ns)
        rc = self.lib.msdp_batch_get_residuals(self.h, p, _ptr(Rp), Rdp, _ptr(Rdl))
        self.ctx.check(rc, "msdp_batch_get_residuals")
        return Rp, [np.ascontiguousarray(a) for a in Rd], Rdl

    def block_matrix(self, p: int, block: int, which: str) -> np.ndarray:
        code = {"W": 0, "corr": 1, "Si": 2, "S": 3, "X": 4}[which]
        n = self.models[p].sides[block]
        out = np.zeros((n, n), order="F")
        rc = self.lib.msdp_batch_get_block_matrix(self.h, p, block, code, _ptr(out))
        self.ctx.check(rc, "msdp_batch_get_block_matrix")
        return np.ascontiguousarray(out)


def _stats_dict(s) -> dict:
    d = {k: getattr(s, k) for k, _ in _lib.Stats._fields_}
    d["status"] = Status(d["status"]) if d["status"] in Status._value2member_map_ else d["status"]
    return d


class InstanceSolver:
    """One large problem on the whole GPU (msdp_solver): each iteration runs
    as device-wide operations instead of one thread block per problem."""

    def __init__(self, model: Model, algorithm=None, direction=None, step=None, centering=None,
                 initial_point=None, schur=None, precision: str = "fp64", context: Optional[Context] = None,
                 **options):
        self.ctx = context or default_context()
        self.lib = self.ctx.lib
        self.model = model
        direction = NT() if direction is None else direction
        step = EigenStep() if step is None else step
        centering = Mehrotra() if centering is None else centering
        self.algorithm = PrimalDual(direction, step, centering) if algorithm is None else algorithm
        self.initial_point = ScaledIdentity() if initial_point is None else initial_point
        self.schur = DenseCholesky() if schur is None else schur
        self.opt = Options(**options)
        mm = _Marshalled(model)
        comp = _components(self.algorithm, self.initial_point, self.schur, precision)
        opts = _options(self.opt)
        h = C.c_void_p()
        rc = self.lib.msdp_solver_create(self.ctx.h, C.byref(mm.desc), C.byref(comp), C.byref(opts), C.byref(h))
        if rc == -4:
            raise NotImplementedError("the whole-GPU solver runs PrimalDual with DenseCholesky, in FP64 or, "
                                      "with the NT direction, in mixed precision")
        if rc != 0:
            raise (ValueError if rc == -1 else GPUError)(f"msdp_solver_create: {_lib.ERRORS.get(rc, rc)}")
        self.h = h
        self.ctx.adopt(self)
        if isinstance(self.initial_point, InitialPoint):
            ip = self.initial_point
            X = [np.asfortranarray(np.asarray(a, dtype=np.float64)) for a in ip.X]
            Xp = (f64p * max(len(X), 1))(*[_ptr(a) for a in X])
            y = np.ascontiguousarray(ip.y, dtype=np.float64)
            x = None if ip.x is None else np.ascontiguousarray(ip.x, dtype=np.float64)
            rc = self.lib.msdp_solver_set_initial_point(self.h, Xp, _ptr(y), None if x is None else _ptr(x))
            if rc != 0:
                raise ValueError("msdp_solver_set_initial_point: invalid initial point")
        self._stats = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.msdp_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self):
        rc = self.lib.msdp_solver_solve(self.h)
        if rc == -5:
            raise RuntimeError("MadSDP: could not find a dual interior point `y = -ρ 1`; use `InitialPoint` to give one.")
        if rc != 0:
            msg = self.lib.msdp_solver_last_error(self.h).decode()
            raise GPUError(f"msdp_solver_solve: {_lib.ERRORS.get(rc, rc)}: {msg}")
        self._stats = None
        return self

    @property
    def device_bytes(self) -> int:
        return int(self.lib.msdp_solver_device_bytes(self.h))

    @property
    def launch_count(self) -> int:
        return int(self.lib.msdp_solver_launch_count(self.h))

    def profile(self) -> dict:
        """Device seconds per phase of the last solve."""
        buf = (C.c_double * 16)()
        n = self.lib.msdp_solver_get_profile(self.h, buf, 16)
        return {self.lib.msdp_solver_profile_field_name(i).decode(): buf[i] for i in range(max(n, 0))}

    def counters(self) -> dict:
        """Work counters of the last solve (refinement steps and fallbacks,
        NT eigendecompositions by FP32 + refinement or dense FP64, tensor-core
        products)."""
        buf = (C.c_int64 * 16)()
        n = self.lib.msdp_solver_get_counters(self.h, buf, 16)
        return {self.lib.msdp_solver_counter_name(i).decode(): int(buf[i]) for i in range(max(n, 0))}

    def stats(self) -> dict:
        st = _lib.Stats()
        self.lib.msdp_solver_get_stats(self.h, C.byref(st))
        return _stats_dict(st)

    # --- component-granular calls (src/primal_dual.jl:29-37, solver.jl:304, step.jl:150-183)
    MATRICES = {"W": 0, "G": 1, "Sinv": 2, "Ls": 3, "Lx": 4, "D": 5}

    def set_iterate(self, X, S, y, x=None, z=None):
        """Load an iterate of the host driver (and update the residuals)."""
        m = self.model
        Xs = [np.asfortranarray(np.asarray(a, dtype=np.float64)) for a in X]
        Ss = [np.asfortranarray(np.asarray(a, dtype=np.float64)) for a in S]
        Xp = (f64p * max(len(Xs), 1))(*[_ptr(a) for a in Xs])
        Sp = (f64p * max(len(Ss), 1))(*[_ptr(a) for a in Ss])
        yv = np.ascontiguousarray(y, dtype=np.float64)
        xv = np.ascontiguousarray(np.zeros(m.ns) if x is None else x, dtype=np.float64)
        zv = np.ascontiguousarray(np.zeros(m.ns) if z is None else z, dtype=np.float64)
        rc = self.lib.msdp_solver_set_iterate(self.h, Xp, Sp, _ptr(yv), _ptr(xv), _ptr(zv))
        if rc != 0:
            raise GPUError(f"msdp_solver_set_iterate: {_lib.ERRORS.get(rc, rc)}")

    def prepare(self) -> bool:
        """_prepare!: Cholesky of S, S^-1, NT scaling, Cholesky of X."""
        ok = C.c_int32()
        rc = self.lib.msdp_solver_prepare(self.h, C.byref(ok))
        if rc != 0:
            raise GPUError(f"msdp_solver_prepare: {_lib.ERRORS.get(rc, rc)}")
        return bool(ok.value)

    def schur_assemble(self, precision: str = "fp64") -> np.ndarray:
        """The Schur complement matrix of the prepared scaling (lower triangle)."""
        m = self.model.m
        H = np.zeros((m, m), order="F")
        code = {"fp64": 0, "mixed": 1}[precision]
        rc = self.lib.msdp_solver_schur_assemble(self.h, code, _ptr(H))
        if rc == -4:
            raise NotImplementedError("split-precision assembly needs an NT solver created in mixed precision")
        if rc != 0:
            raise GPUError(f"msdp_solver_schur_assemble: {_lib.ERRORS.get(rc, rc)}")
        return np.tril(H)

    def block_matrix(self, block: int, which: str) -> np.ndarray:
        n = self.model.sides[block]
        out = np.zeros(n) if which == "D" else np.zeros((n, n), order="F")
        rc = self.lib.msdp_solver_get_block_matrix(self.h, block, self.MATRICES[which], _ptr(out))
        if rc != 0:
            raise GPUError(f"msdp_solver_get_block_matrix: {_lib.ERRORS.get(rc, rc)}")
        return out

    def step_eig(self, block: int, L, D) -> float:
        """lambda_min(L^-1 D L^-T) (EigenStep, src/step.jl:150-183)."""
        Lf = np.asfortranarray(L, dtype=np.float64)
        Df = np.asfortranarray(D, dtype=np.float64)
        lam = C.c_double()
        rc = self.lib.msdp_solver_step_eig(self.h, block, _ptr(Lf), _ptr(Df), C.byref(lam))
        if rc != 0:
            raise GPUError(f"msdp_solver_step_eig: {_lib.ERRORS.get(rc, rc)}")
        return lam.value

    def solution(self):
        m = self.model
        X = [np.zeros((n, n), order="F") for n in m.sides]
        Xp = (f64p * max(len(X), 1))(*[_ptr(a) for a in X])
        y, x, z = np.zeros(m.m), np.zeros(m.ns), np.zeros(m.ns)
        rc = self.lib.msdp_solver_get_solution(self.h, Xp, _ptr(y), _ptr(x), _ptr(z))
        if rc != 0:
            raise GPUError(f"msdp_solver_get_solution: {_lib.ERRORS.get(rc, rc)}")
        return [np.ascontiguousarray(a) for a in X], y, x, z

    def trajectory(self) -> List[dict]:
        cap = self.opt.max_iter + 2
        arr = (_lib.IterRecord * cap)()
        cnt = C.c_int32()
        self.lib.msdp_solver_get_trajectory(self.h, arr, cap, C.byref(cnt))
        return [{k: getattr(r, k) for k, _ in _lib.IterRecord._fields_} for r in arr[:min(cnt.value, cap)]]


class SchurWorkspace:
    """A Schur-solver component on the GPU (src/components.jl:253-266):
    schur_workspace(DenseCholesky(), Float64, m), factorize!(ws) of a
    host-assembled H, schur_solve!(ws, rhs).  precision "mixed": FP32-class
    factor refined in FP64 against H, FP64 after a stalled refinement or a
    breakdown of the FP32-class factorization."""

    def __init__(self, m: int, precision: str = "fp64", context: Optional[Context] = None):
        self.ctx = context or default_context()
        self.lib = self.ctx.lib
        self.m = int(m)
        h = C.c_void_p()
        rc = self.lib.msdp_schur_create(self.ctx.h, self.m, {"fp64": 0, "mixed": 1}[precision], C.byref(h))
        if rc != 0:
            raise GPUError(f"msdp_schur_create: {_lib.ERRORS.get(rc, rc)}")
        self.h = h
        self.ctx.adopt(self)

    def factorize(self, H) -> bool:
        Hf = np.asfortranarray(H, dtype=np.float64)
        if Hf.shape != (self.m, self.m):
            raise ValueError("H must be m x m")
        ok = C.c_int32()
        rc = self.lib.msdp_schur_factorize(self.h, _ptr(Hf), C.byref(ok))
        if rc != 0:
            raise GPUError(f"msdp_schur_factorize: {_lib.ERRORS.get(rc, rc)}")
        return bool(ok.value)

    def solve(self, rhs) -> np.ndarray:
        x = np.array(rhs, dtype=np.float64, copy=True)
        rc = self.lib.msdp_schur_solve(self.h, _ptr(x))
        if rc != 0:
            raise GPUError(f"msdp_schur_solve: {_lib.ERRORS.get(rc, rc)}")
        return x

    @property
    def fp64_active(self) -> bool:
        return bool(self.lib.msdp_schur_fp64_active(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.msdp_schur_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _use_instance_engine(model: Model) -> bool:
    """A single problem with a block above 64 or more than 300 constraints
    runs on the whole GPU (measured on GB300: max-cut n = 100 takes 0.23 s
    there against 0.95 s in one thread block); smaller ones in one thread
    block.  Batches always use one thread block per problem."""
    return max(model.sides, default=0) > 64 or model.m > 300


class MadSDPSolver:
    """One problem on the GPU with the constructor of src/solver.jl:87-160.

    engine = "batch" runs it as a one-problem batch (one thread block),
    "instance" on the whole GPU, "auto" picks by size."""

    def __init__(self, model: Model, engine: str = "auto", **kwargs):
        self.model = model
        if engine not in ("auto", "batch", "instance"):
            raise ValueError("engine must be 'auto', 'batch' or 'instance'")
        if engine == "auto":
            # the whole-GPU engine runs PrimalDual with DenseCholesky (FP64,
            # or mixed for NT) or MadNLPSchur (FP64)
            schur = kwargs.get("schur")
            prec = kwargs.get("precision", "fp64")
            alg = kwargs.get("algorithm")
            direction = kwargs.get("direction") or (alg.direction if isinstance(alg, PrimalDual) else None)
            dense_chol = schur is None or isinstance(schur, DenseCholesky)
            supported = (not isinstance(alg, DualCentering)
                         and (dense_chol or isinstance(schur, MadNLPSchur))
                         and (prec in ("fp64", "fp64_tensor")
                              or (prec == "mixed" and dense_chol and (direction is None or isinstance(direction, NT)))))
            large = _use_instance_engine(model)
            engine = "instance" if supported and (prec == "fp64_tensor" or large) else "batch"
            if large and not supported:
                warnings.warn("this problem (largest block %d, m = %d) runs in one thread block: the whole-GPU "
                              "engine does not take %s" % (max(model.sides, default=0), model.m,
                                                          "DualCentering" if isinstance(alg, DualCentering)
                                                          else type(schur).__name__ if not dense_chol
                                                          else "mixed precision with HKM"),
                              stacklevel=2)
        self.engine = engine
        self.batch = Batch([model], **kwargs) if engine == "batch" else None
        self.instance = InstanceSolver(model, **kwargs) if engine == "instance" else None
        self._stats = None

    def close(self):
        """Release the device memory of the underlying batch or solver."""
        for h in (self.batch, self.instance):
            if h is not None:
                h.close()

    def initialize(self):
        if self.batch is None:
            raise NotImplementedError("the whole-GPU engine solves in one call")
        self.batch.initialize()
        self._stats = None

    def solve(self, verbose: bool = False):
        """solve!(solver) (src/solver.jl:385-396)."""
        if self.instance is not None:
            self.instance.solve()
            self._stats = self.instance.stats()
        else:
            self.batch.solve()
            self._stats = self.batch.stats(0)
        if verbose:
            print_trajectory(self.trajectory())
        return self

    def iterate(self, k: int = 1):
        if self.batch is None:
            raise NotImplementedError("the whole-GPU engine solves in one call")
        self.batch.iterate(k)
        self._stats = None

    @property
    def stats(self) -> dict:
        if self._stats is None:
            self._stats = self.instance.stats() if self.instance is not None else self.batch.stats(0)
        return self._stats

    @property
    def status(self) -> Status:
        return self.stats["status"]

    @property
    def iter(self) -> int:
        return self.stats["iter"]

    def primal_objective(self) -> float:
        return self.stats["pobj"]

    def dual_objective(self) -> float:
        return self.stats["dobj"]

    @property
    def inf_pr(self):
        return self.stats["inf_pr"]

    @property
    def inf_du(self):
        return self.stats["inf_du"]

    @property
    def inf_compl(self):
        return self.stats["gap"]

    def solution(self):
        return self.instance.solution() if self.instance is not None else self.batch.solution(0)

    def trajectory(self):
        return self.instance.trajectory() if self.instance is not None else self.batch.trajectory(0)


def print_trajectory(traj):
    """The iteration table of src/solver.jl:353-383."""
    for r in traj:
        if int(r["iter"]) % 10 == 0:
            print("%4s %14s %14s %9s %9s %9s %9s %9s" % ("iter", "p_obj", "d_obj", "inf_pr", "inf_du", "gap", "mu", "α/β"))
        print("%4d %14.6e %14.6e %9.2e %9.2e %9.2e %9.2e %4.2f/%4.2f" % (
            r["iter"], r["pobj"], r["dobj"], r["inf_pr"], r["inf_du"], r["gap"], r["mu"], r["alpha"], r["beta"]))


def madsdp(model: Model, **kwargs) -> MadSDPSolver:
    """madsdp(model; kwargs...) (src/solver.jl:404)."""
    return MadSDPSolver(model, **kwargs).solve()
