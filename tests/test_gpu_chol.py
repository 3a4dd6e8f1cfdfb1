"""Blocked Cholesky with tensor-core trailing updates (msdp_dense_cholesky)
against LAPACK's factor of the same matrix: FP64 to 1e-13 relative (the
products are FP64-accurate), the mixed precision to FP32 level; the strict
upper triangle is left as it was; a pivot that is not positive and finite
is reported at the same index as LAPACK potrf."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _factor(prec, A):
    import torch

    from madsdp_gpu import _lib
    lib = _lib.load()
    n = A.shape[0]
    Ad = torch.tensor(A.T.copy(), dtype=torch.float64, device="cuda")  # column-major
    info = C.c_int32(-7)
    st = torch.cuda.current_stream().cuda_stream
    rc = lib.msdp_dense_cholesky(prec, n, C.c_void_p(Ad.data_ptr()), n, C.byref(info), C.c_void_p(st))
    assert rc == 0, rc
    return Ad.cpu().numpy().T, info.value


def _spd(n, rng, cond=1e3):
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = np.exp(np.linspace(0.0, np.log(cond), n))
    return (Q * lam) @ Q.T


@pytest.mark.parametrize("n", [1, 31, 32, 33, 100, 257, 1000])
@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 2e-5)])
def test_cholesky_matches_lapack(gpu_ctx, n, prec, tol):
    rng = np.random.default_rng(n + 10 * prec)
    A = _spd(n, rng)
    A[np.triu_indices(n, 1)] = 7.0  # the upper triangle must not be read or written
    Lref = np.linalg.cholesky(np.tril(A) + np.tril(A, -1).T)
    got, info = _factor(prec, A)
    assert info == 0
    L = np.tril(got)
    assert np.abs(L - Lref).max() / np.abs(Lref).max() <= tol
    assert np.array_equal(got[np.triu_indices(n, 1)], A[np.triu_indices(n, 1)])


@pytest.mark.parametrize("k", [0, 17, 40, 95])
def test_cholesky_reports_first_bad_pivot(gpu_ctx, k):
    n = 96
    A = np.eye(n) * 4.0
    A[k, k] = -1.0
    _, info = _factor(0, A)
    assert info == k + 1


def test_cholesky_reports_nonfinite_pivot(gpu_ctx):
    n = 70
    A = np.eye(n)
    A[50, 50] = np.nan
    _, info = _factor(0, A)
    assert info == 51


def test_cholesky_large_spd_residual(gpu_ctx):
    """n = 2000 (the Schur matrix of the configuration-2/3 workloads): the
    factor reproduces A to FP64 accuracy."""
    rng = np.random.default_rng(3)
    n = 2000
    B = rng.standard_normal((n, n + 50))
    A = B @ B.T / n
    got, info = _factor(0, A)
    assert info == 0
    L = np.tril(got)
    assert np.abs(L @ L.T - A).max() / np.abs(A).max() <= 1e-13
