"""Tridiagonal helpers of the whole-GPU solver's Lanczos iteration
(madsdp.jl_gb300/csrc/tridiag.h) against numpy.linalg.eigh on the CPU:
Sturm counts, the smallest eigenvalue by bisection and the last component
of its eigenvector (the Ritz residual of the stopping rule)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
D = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("tridiag") / "tridiag_check.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "native", "tridiag_check.cpp")], check=True)
    lib = C.CDLL(so)
    lib.check_tridiag_min.argtypes = [C.c_int, D, D, D]
    lib.check_tridiag_min.restype = C.c_double
    lib.check_last_component.argtypes = [C.c_int, D, D, C.c_double, C.c_double]
    lib.check_last_component.restype = C.c_double
    lib.check_sturm_count.argtypes = [C.c_int, D, D, C.c_double]
    lib.check_sturm_count.restype = C.c_int
    return lib


def tridiagonals():
    rng = np.random.default_rng(0)
    out = []
    for k in (1, 2, 3, 10, 60, 200):
        out.append((rng.standard_normal(k), rng.standard_normal(max(k - 1, 0))))
    # graded and clustered spectra, as Lanczos on ill-conditioned congruences gives
    out.append((np.logspace(-8, 2, 40), 1e-3 * np.ones(39)))
    out.append((np.ones(30), 1e-9 * np.ones(29)))
    return out


def full(a, b):
    return np.diag(a) + np.diag(b, 1) + np.diag(b, -1)


@pytest.mark.parametrize("case", range(8))
def test_smallest_eigenvalue_and_norm(lib, case):
    a, b = tridiagonals()[case]
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b if b.size else np.zeros(1))
    w = np.linalg.eigvalsh(full(a, b[:a.size - 1]))
    norm = C.c_double()
    lam = lib.check_tridiag_min(a.size, a.ctypes.data_as(D), b.ctypes.data_as(D), C.byref(norm))
    assert abs(lam - w[0]) <= 1e-13 * max(1.0, np.abs(w).max())
    assert norm.value >= np.abs(w).max() - 1e-12  # a Gershgorin bound


@pytest.mark.parametrize("case", range(8))
def test_sturm_counts(lib, case):
    a, b = tridiagonals()[case]
    b = np.ascontiguousarray(b if b.size else np.zeros(1))
    w = np.linalg.eigvalsh(full(a, b[:a.size - 1]))
    for x in np.concatenate([w[:-1] + np.diff(w) / 2, [w[0] - 1.0, w[-1] + 1.0]]):
        if np.min(np.abs(w - x)) < 1e-9 * max(1.0, np.abs(w).max()):
            continue
        assert lib.check_sturm_count(a.size, a.ctypes.data_as(D), b.ctypes.data_as(D), x) == np.sum(w < x)


@pytest.mark.parametrize("case", [1, 2, 3, 4, 5, 6])
def test_last_component_gives_the_ritz_residual(lib, case):
    a, b = tridiagonals()[case]
    T = full(a, b)
    w, V = np.linalg.eigh(T)
    norm = np.abs(w).max()
    s = lib.check_last_component(a.size, a.ctypes.data_as(D), np.ascontiguousarray(b).ctypes.data_as(D), w[0], norm)
    # accurate where the smallest eigenvalue is separated from the next
    if w[1] - w[0] > 1e-6 * norm:
        assert abs(s - abs(V[-1, 0])) <= 1e-8 + 1e-6 * abs(V[-1, 0])
