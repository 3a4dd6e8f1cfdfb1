"""Float-float arithmetic (madsdp.jl_gb300/csrc/ff.cuh) on the CPU: the
error-free transformations are exact, each operation is accurate to about
2^-44 relative, and a float-float Cholesky factorization of the ill-
conditioned Gram and slack matrices at the end of SOS solves (cond up to
4.5e12, where FP32 fails) reaches residuals near 1e-15."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from madsdp_gpu import generators as g
from oracle import madsdp_oracle as o

HERE = os.path.dirname(os.path.abspath(__file__))
D = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("ff") / "ff_check.so")
    # no contraction of a*b+c on the host: the header writes its FMAs out
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "native", "ff_check.cpp")], check=True)
    lib = C.CDLL(so)
    lib.ff_eft_check.argtypes = [C.c_int, C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                 C.POINTER(C.c_int32)]
    lib.ff_elementwise.argtypes = [C.c_int, C.c_int64, D, D, D, D, D]
    lib.ff_dot.argtypes = [C.c_int64, D, D]
    lib.ff_dot.restype = C.c_double
    lib.ff_cholesky.argtypes = [C.c_int, D, D]
    lib.ff_cholesky.restype = C.c_int
    return lib


def values(rng, n, lo=-20, hi=20, signed=True):
    v = rng.uniform(1, 2, n) * 2.0 ** rng.integers(lo, hi, n)
    return v * rng.choice([-1.0, 1.0], n) if signed else v


@pytest.mark.parametrize("op", [0, 1])
def test_error_free_transformations(lib, op):
    rng = np.random.default_rng(op)
    a = values(rng, 20000).astype(np.float32)
    b = values(rng, 20000).astype(np.float32)
    ok = np.zeros(a.size, np.int32)
    lib.ff_eft_check(op, a.size, a.ctypes.data_as(C.POINTER(C.c_float)), b.ctypes.data_as(C.POINTER(C.c_float)),
                     ok.ctypes.data_as(C.POINTER(C.c_int32)))
    assert ok.all()


def elementwise(lib, op, a, b):
    ain, bin_, out = np.zeros_like(a), np.zeros_like(a), np.zeros_like(a)
    lib.ff_elementwise(op, a.size, *(x.ctypes.data_as(D) for x in (a, b, ain, bin_, out)))
    return ain, bin_, out


@pytest.mark.parametrize("op,bound", [(0, 2.0 ** -44), (1, 2.0 ** -44), (2, 2.0 ** -44), (3, 2.0 ** -43),
                                      (4, 2.0 ** -44), (5, 2.0 ** -43)])
def test_operation_accuracy(lib, op, bound):
    """Error relative to the magnitude of the operands' contribution (for
    sums |a| + |b|, so cancellation is covered); float64 arithmetic on the
    float-float inputs (exact in float64) is the reference."""
    rng = np.random.default_rng(10 + op)
    a = values(rng, 20000, signed=op != 4)
    b = values(rng, 20000)
    ain, bin_, out = elementwise(lib, op, a, b)
    ref, mag = {
        0: lambda: (ain + bin_, np.abs(ain) + np.abs(bin_)),
        1: lambda: (ain - bin_, np.abs(ain) + np.abs(bin_)),
        2: lambda: (ain * bin_, np.abs(ain * bin_)),
        3: lambda: (ain / bin_, np.abs(ain / bin_)),
        4: lambda: (np.sqrt(ain), np.sqrt(ain)),
        5: lambda: (ain * bin_ + ain, np.abs(ain * bin_) + np.abs(ain)),
    }[op]()
    assert np.max(np.abs(out - ref) / mag) <= bound


def test_dot_product(lib):
    rng = np.random.default_rng(3)
    for n in (16, 64, 256):
        x, y = rng.standard_normal(n), rng.standard_normal(n)
        r = lib.ff_dot(n, x.ctypes.data_as(D), y.ctypes.data_as(D))
        assert abs(r - x @ y) <= 4 * n * 2.0 ** -44 * (np.abs(x) @ np.abs(y))


@pytest.mark.parametrize("d,centering", [(15, "Mehrotra"), (31, "Mehrotra"), (11, "AdaptiveMu")])
def test_cholesky_of_final_iterates(lib, d, centering):
    s = o.Solver(g.sos_hankel(d, seed=2), centering=getattr(o, centering)()).solve()
    for M in (s.blocks[0].X, s.blocks[0].S):
        M = np.asfortranarray((M + M.T) / 2)
        n = M.shape[0]
        L = np.zeros((n, n), order="F")
        assert lib.ff_cholesky(n, M.ctypes.data_as(D), L.ctypes.data_as(D)) == 1
        assert np.linalg.norm(L @ L.T - M) / np.linalg.norm(M) <= 2e-14


def test_cholesky_rejects_indefinite(lib):
    M = np.asfortranarray(np.diag([1.0, -1e-3, 2.0]))
    L = np.zeros((3, 3), order="F")
    assert lib.ff_cholesky(3, M.ctypes.data_as(D), L.ctypes.data_as(D)) == 0


def test_operators_match_the_functions_and_order(lib):
    """The operator forms give the named operations' results, and the
    comparisons order float-float values as float64 orders their sums."""
    lib.ff_operators.argtypes = [C.c_int64, D, D, D, C.POINTER(C.c_int32)]
    rng = np.random.default_rng(8)
    a = values(rng, 5000)
    b = np.where(rng.random(5000) < 0.1, a, values(rng, 5000))  # some equal pairs
    out = np.zeros(6 * a.size)
    cmp = np.zeros(4 * a.size, np.int32)
    lib.ff_operators(a.size, a.ctypes.data_as(D), b.ctypes.data_as(D), out.ctypes.data_as(D),
                     cmp.ctypes.data_as(C.POINTER(C.c_int32)))
    out, cmp = out.reshape(-1, 6), cmp.reshape(-1, 4)
    ain, bin_, _ = elementwise(lib, 0, a, b)
    for op, col in ((0, 0), (1, 1), (2, 2), (3, 3)):
        assert np.array_equal(out[:, col], elementwise(lib, op, a, b)[2])
    assert np.array_equal(out[:, 5], np.abs(ain))
    assert np.max(np.abs(out[:, 4] - np.sqrt(np.abs(ain))) / np.sqrt(np.abs(ain))) <= 2.0 ** -44
    assert np.array_equal(cmp[:, 0], ain < bin_) and np.array_equal(cmp[:, 1], ain > bin_)
    assert np.array_equal(cmp[:, 2], ain <= bin_) and np.array_equal(cmp[:, 3], ain == bin_)


def test_constructors_and_fma(lib):
    lib.ff_constructors.argtypes = [C.c_int64, D, D, D]
    lib.ff_constructors.restype = C.c_int
    rng = np.random.default_rng(9)
    a, b, c = values(rng, 2000), values(rng, 2000), values(rng, 2000)
    assert lib.ff_constructors(a.size, a.ctypes.data_as(D), b.ctypes.data_as(D), c.ctypes.data_as(D)) == 0


def test_conversion_beyond_float_range(lib):
    """Values beyond the float range become the infinity of their sign (not
    NaN); finite values round-trip to within float-float precision."""
    lib.ff_roundtrip.argtypes = [C.c_int64, D, D, D]
    v = np.array([1e300, -1e300, np.inf, -np.inf, 3.5e38, 1.0 / 3.0, -2.0 ** -100, 0.0])
    a, b = np.zeros_like(v), np.zeros_like(v)
    lib.ff_roundtrip(v.size, v.ctypes.data_as(D), a.ctypes.data_as(D), b.ctypes.data_as(D))
    for out in (a, b):
        assert np.array_equal(out[:5], [np.inf, -np.inf, np.inf, -np.inf, np.inf])
        assert np.all(np.abs(out[5:] - v[5:]) <= 2.0 ** -47 * np.abs(v[5:]))


def test_cta_cholesky_instantiates_with_float_float(tmp_path):
    """The CTA Cholesky of la.cuh compiles for sm_103a with T = ff (compile
    only; nothing is launched)."""
    import shutil
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc) and shutil.which(nvcc) is None:
        pytest.skip("nvcc not available")
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        "--expt-relaxed-constexpr", "-Xptxas", "-v", "-c",
                        os.path.join(HERE, "native", "ff_potrf_compile.cu"), "-o", str(tmp_path / "p.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "ff_potrf_probe" in r.stderr and "registers" in r.stderr
