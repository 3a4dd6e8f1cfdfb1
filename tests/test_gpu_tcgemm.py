"""Tensor-core split-precision products (msdp_tc_gemm) against float64
products of the same operands on the GPU.

Each row of an operand is sliced relative to its largest entry, so the error
of entry (r, c) is bounded by max_k |a_rk| sum_k |b_kc| + sum_k |a_rk| max_k
|b_kc| (times |alpha|, plus |beta| |C0|), which equals |op(A)| |op(B)| when
the entries of a row have similar magnitudes.  Tolerances against that
bound: 1e-13 for the FP64 precision (7 bf16 slices) and 2e-6 for the mixed
precision (3 slices, FP32-class).  On rows of similar magnitude the error
against |op(A)| |op(B)| itself is checked too: 2e-14 and 1e-6.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-13, 1: 2e-6}  # MSDP_FP64, MSDP_MIXED


def _run(lib, torch, prec, ta, tb, M, N, K, alpha, beta, lower, A, B, C0):
    Cd = C0.clone()
    lda = A.shape[1]
    ldb = B.shape[1]
    # column-major views: a torch (rows, cols) tensor stored as its transpose
    st = torch.cuda.current_stream().cuda_stream
    rc = lib.msdp_tc_gemm(prec, ta, tb, M, N, K, alpha, C.c_void_p(A.data_ptr()), lda, C.c_void_p(B.data_ptr()), ldb,
                          beta, C.c_void_p(Cd.data_ptr()), M, lower, C.c_void_p(st))
    assert rc == 0, rc
    return Cd


def _colmajor(torch, rows, cols, rng, scale_rows=None, scale_cols=None):
    a = rng.standard_normal((rows, cols))
    if scale_rows is not None:
        a *= scale_rows[:, None]
    if scale_cols is not None:
        a *= scale_cols[None, :]
    # column-major storage of a (rows x cols): a torch tensor of shape (cols, rows)
    return torch.tensor(a.T.copy(), dtype=torch.float64, device="cuda"), a


CASES = [
    # M, N, K, transa, transb, alpha, beta, lower
    (1, 1, 1, 0, 0, 1.0, 0.0, 0),
    (200, 130, 77, 0, 0, 1.0, 0.0, 0),
    (300, 257, 700, 1, 0, -1.0, 0.0, 0),
    (129, 129, 2000, 1, 1, 0.7, 1.3, 1),
    (256, 384, 5000, 0, 1, 2.0, 0.0, 0),
    (130, 130, 333, 1, 0, 1.0, 1.0, 1),
]


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("case", CASES)
def test_tc_gemm_matches_float64(gpu_ctx, prec, case):
    import torch

    from madsdp_gpu import _lib
    lib = _lib.load()
    M, N, K, ta, tb, alpha, beta, lower = case
    rng = np.random.default_rng(M * 7 + N * 3 + K + prec)
    # op(A) is M x K, stored column-major as A (M x K) or A^T (K x M)
    ar, ac = (K, M) if ta else (M, K)
    br, bc = (N, K) if tb else (K, N)
    rs_a = np.exp(rng.uniform(-6, 6, ar))
    cs_b = np.exp(rng.uniform(-6, 6, bc))
    Ad, A = _colmajor(torch, ar, ac, rng, scale_rows=rs_a)
    Bd, B = _colmajor(torch, br, bc, rng, scale_cols=cs_b)
    if ar > 3:
        Ad[:, 2] = 0.0  # a zero row of the stored A
        A[2, :] = 0.0
    C0d, C0 = _colmajor(torch, M, N, rng)
    Cd = _run(lib, torch, prec, ta, tb, M, N, K, alpha, beta, lower, Ad, Bd, C0d)
    opA = A.T if ta else A
    opB = B.T if tb else B
    ref = alpha * (opA @ opB) + beta * C0
    aa, bb = np.abs(opA), np.abs(opB)
    slicing = np.maximum(aa.max(axis=1)[:, None] * bb.sum(axis=0)[None, :],
                         aa.sum(axis=1)[:, None] * bb.max(axis=0)[None, :])
    bound = abs(alpha) * np.maximum(aa @ bb, slicing) + abs(beta) * np.abs(C0) + 1e-300
    got = Cd.cpu().numpy().T
    if lower:
        mask = np.tril(np.ones((M, N), dtype=bool))
        assert np.array_equal(got[~mask], C0[~mask])  # the upper triangle is not touched
    else:
        mask = np.ones((M, N), dtype=bool)
    err = (np.abs(got - ref) / bound)[mask].max()
    assert err <= TOL[prec], err
    # the accumulation is exact per chunk and integer across chunks: a second
    # call gives the same bits
    Cd2 = _run(lib, torch, prec, ta, tb, M, N, K, alpha, beta, lower, Ad, Bd, C0d)
    assert torch.equal(Cd, Cd2)


@pytest.mark.parametrize("prec,tol", [(0, 2e-14), (1, 1e-6)])
def test_tc_gemm_accuracy_on_uniform_rows(gpu_ctx, prec, tol):
    import torch

    from madsdp_gpu import _lib
    lib = _lib.load()
    rng = np.random.default_rng(5 + prec)
    M, N, K = 384, 320, 3000
    Ad, A = _colmajor(torch, M, K, rng)
    Bd, B = _colmajor(torch, K, N, rng)
    C0d, C0 = _colmajor(torch, M, N, rng)
    Cd = _run(lib, torch, prec, 0, 0, M, N, K, 1.0, 0.0, 0, Ad, Bd, C0d)
    err = (np.abs(Cd.cpu().numpy().T - A @ B) / (np.abs(A) @ np.abs(B))).max()
    assert err <= tol, err


def test_tc_gemm_rejects_bad_arguments(gpu_ctx):
    from madsdp_gpu import _lib
    lib = _lib.load()
    null = C.c_void_p(0)
    assert lib.msdp_tc_gemm(5, 0, 0, 4, 4, 4, 1.0, null, 4, null, 4, 0.0, null, 4, 0, null) == -1
    assert lib.msdp_tc_gemm(0, 0, 0, 4, 3, 4, 1.0, null, 4, null, 4, 0.0, null, 4, 1, null) == -1
    assert lib.msdp_tc_gemm(0, 0, 0, 0, 0, 4, 1.0, null, 4, null, 4, 0.0, null, 1, 0, null) == 0


@pytest.mark.parametrize("prec,tol", [(0, 5e-14), (1, 1e-6)])
def test_tc_gemm_config3_schur_shape(gpu_ctx, prec, tol):
    """The Schur-complement product of the dense-constraint workload at full
    size: H = B B' (lower) with B of 2000 rows and K = 20100 (the symmetric
    vectors of the 200 x 200 block), against a float64 product on the GPU.
    At this K the float64 reference itself is off by about sqrt(K) * 2^-53
    = 1.6e-14 of |B||B'|, hence the bound."""
    import torch

    from madsdp_gpu import _lib
    lib = _lib.load()
    m, K = 2000, 20100
    gen = torch.Generator(device="cuda").manual_seed(7)
    B = torch.randn(m, K, dtype=torch.float64, device="cuda", generator=gen)  # column-major K x m: op(A) = B
    Cout = torch.zeros(m, m, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    rc = lib.msdp_tc_gemm(prec, 1, 0, m, m, K, 1.0, C.c_void_p(B.data_ptr()), K, C.c_void_p(B.data_ptr()), K, 0.0,
                          C.c_void_p(Cout.data_ptr()), m, 1, C.c_void_p(st))
    assert rc == 0
    ref = B @ B.T
    bound = B.abs() @ B.abs().T
    low = torch.tril(torch.ones(m, m, dtype=torch.bool, device="cuda"))
    got = Cout.T  # column-major result
    err = ((got - ref).abs() / bound)[low].max().item()
    assert err <= tol, err
    assert (got[~low] == 0).all()
