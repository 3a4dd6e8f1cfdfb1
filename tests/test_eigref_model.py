"""CPU model of the eigendecomposition refinement (csrc/eigref.h).

The NT scaling of the whole-GPU solver takes N = V diag(lam) V' from an
FP32 eigensolver and refines it to FP64 accuracy: Ogita-Aishima steps
(first-order corrections of the separated pairs), and for clusters of
eigenvalues too close for them, first-order orthonormalization inside the
cluster followed by the exact rotation that diagonalizes the cluster's
block in that frame, applied to the cluster's whole columns; the matrix is
shifted by its mean eigenvalue first, and pairs whose residual is at
rounding level are only orthonormalized.  This restates one step in NumPy with the kernels'
decisions (coupling test, clusters as ranges closed under the coupled
pairs, Jacobi in the cluster) and checks that it reaches FP64 accuracy
from FP32 eigenvectors, also with exactly repeated and nearly repeated
eigenvalues and a wide eigenvalue range.
"""

import numpy as np
import pytest

TAU = 3e-2
MAX_CLUSTER = 64


def jacobi(C):
    """Cyclic Jacobi with the kernel's rotation rule; returns Q with Q'CQ diagonal."""
    C = C.copy()
    k = C.shape[0]
    Q = np.eye(k)
    for _ in range(40):
        rotated = False
        for p in range(k):
            for q in range(p + 1, k):
                app, aqq, apq = C[p, p], C[q, q], C[p, q]
                if abs(apq) > 1e-15 * np.sqrt(abs(app * aqq)) and abs(apq) > 1e-300:
                    z = (aqq - app) / (2 * apq)
                    t = (1.0 if z >= 0 else -1.0) / (abs(z) + np.sqrt(1 + z * z))
                    c = 1 / np.sqrt(1 + t * t)
                    s = t * c
                    J = np.eye(k)
                    J[p, p] = J[q, q] = c
                    J[p, q], J[q, p] = s, -s
                    C = J.T @ C @ J
                    Q = Q @ J
                    rotated = True
        if not rotated:
            break
    return Q


def step(N, V):
    """One refinement step: returns (V (I + E), lam, the residual measure
    max(max_{i != j} |S_ij + lam_j R~_ij| / max|lam|, max |R~_ij|) of the
    basis the step started from, cluster sizes)."""
    n = N.shape[0]
    S = V.T @ N @ V
    R = V.T @ V
    lam = np.diag(S) / np.diag(R)
    Rt = np.eye(n) - R
    E = np.zeros((n, n))
    reach = np.arange(n)
    num_max, rt_max = 0.0, np.max(np.abs(Rt))
    negligible = 64 * np.finfo(float).eps * np.max(np.abs(lam))
    for i in range(n):
        for j in range(n):
            if i == j:
                E[i, i] = 1 + 0.5 * Rt[i, i]
                continue
            s = S[max(i, j), min(i, j)]
            rt = Rt[max(i, j), min(i, j)]
            nij, nji = s + lam[j] * rt, s + lam[i] * rt
            gap = lam[j] - lam[i]
            num_max = max(num_max, abs(nij), abs(nji))
            if max(abs(nij), abs(nji)) <= negligible:
                E[i, j] = 0.5 * rt
            elif gap != 0 and max(abs(nij), abs(nji)) <= TAU * abs(gap):
                E[i, j] = nij / gap
            else:
                a, b = min(i, j), max(i, j)
                reach[a] = max(reach[a], b)
    sizes = []
    a, end = 0, reach[0]
    for i in range(1, n + 1):
        if i == n or i > end:
            k = end - a + 1
            if k >= 2:
                assert k <= MAX_CLUSTER
                sizes.append(k)
                # orthonormalize inside the cluster (first order), then the
                # rotation that diagonalizes the cluster's block in that
                # frame, applied to the cluster's whole columns of I + E
                Oc = np.eye(k) + 0.5 * Rt[a:a + k, a:a + k]
                E[a:a + k, a:a + k] = Oc
                Q = jacobi(Oc @ S[a:a + k, a:a + k] @ Oc)
                E[:, a:a + k] = E[:, a:a + k] @ Q
            if i == n:
                break
            a, end = i, reach[i]
        else:
            end = max(end, reach[i])
    lmax = np.max(np.abs(lam))
    off = num_max / lmax if lmax > 0 else (0.0 if num_max == 0 else np.inf)
    return V @ E, lam, max(off, rt_max), sizes


def refine(N):
    """FP32 eigenvectors of N - (trace N / n) I, refined on the shifted
    matrix; returns the basis, N's eigenvalues, the step count and the last
    step's cluster sizes."""
    n = N.shape[0]
    sigma = np.trace(N) / n
    Ns = N - sigma * np.eye(n)
    w32, V32 = np.linalg.eigh(Ns.astype(np.float32))
    V = V32.astype(np.float64)
    steps = 0
    for _ in range(8):
        V, lam, resid, sizes = step(Ns, V)
        steps += 1
        # the step just applied started below 1e-12: what remains is second order
        if resid <= 1e-12:
            return V, lam + sigma, steps, sizes
    raise AssertionError("refinement did not converge")


def spectrum_matrix(lam, seed):
    rng = np.random.default_rng(seed)
    n = lam.size
    Qm, _ = np.linalg.qr(rng.standard_normal((n, n)))
    N = (Qm * lam) @ Qm.T
    return 0.5 * (N + N.T)


@pytest.mark.parametrize("case", ["spread", "near_pairs", "repeated", "wide", "central", "identity", "centered"])
def test_refinement_reaches_fp64_accuracy(case):
    n = 60
    rng = np.random.default_rng(7)
    if case == "spread":
        lam = np.sort(rng.uniform(1, 10, n))
    elif case == "near_pairs":
        lam = np.sort(rng.uniform(1, 10, n))
        lam[10] = lam[9] * (1 + 1e-9)          # below FP32 resolution
        lam[30] = lam[29] * (1 + 3e-7)
        lam[31] = lam[29] * (1 + 6e-7)         # a cluster of three
    elif case == "repeated":
        lam = np.concatenate([np.full(20, 2.0), np.sort(rng.uniform(3, 5, n - 20))])
    elif case == "wide":
        lam = np.sort(10.0 ** rng.uniform(-5, 0, n))
    elif case == "central":                   # near the central path: XS close to mu I
        lam = np.sort(1e-3 * (1 + 0.5 * rng.uniform(-1, 1, n)))
    elif case == "identity":                  # the start X = a I, S = b I: N = ab I
        lam = np.full(n, 3.0)
    else:                                     # tightly centered: a spread of 1e-6 relative
        lam = np.sort(2.0 * (1 + 1e-6 * rng.uniform(-1, 1, n)))
    N = spectrum_matrix(lam, 3)
    V, lm, steps, _ = refine(N)
    nrm = np.linalg.norm(N, 2)
    # orthonormal and diagonalizing to FP64 accuracy, at least as good as a
    # dense FP64 eigensolver's backward error
    _, Vd = np.linalg.eigh(N)
    dense_res = np.linalg.norm(N @ Vd - Vd * np.linalg.eigvalsh(N)) / nrm
    assert np.linalg.norm(V.T @ V - np.eye(n)) < 1e-13
    assert np.linalg.norm(N @ V - V * lm) / nrm < max(1e-13, 20 * dense_res)
    assert np.max(np.abs(np.sort(lm) - np.sort(lam))) < 1e-13 * nrm
    assert steps <= 6


def test_nt_scaling_from_refined_basis_matches_dense():
    """W = Lx V D^-1 V' Lx' (D = sqrt(lam)) from the refined basis equals the
    one from a dense FP64 eigendecomposition, also with a near-degenerate
    cluster (mixing inside it does not change W beyond rounding)."""
    n = 40
    rng = np.random.default_rng(11)
    lam = np.sort(rng.uniform(0.5, 2.0, n))
    lam[5:9] = lam[5] * (1 + np.array([0, 1e-10, 2e-10, 4e-10]))
    N = spectrum_matrix(lam, 5)
    Lx = np.linalg.cholesky(np.eye(n) + 0.1 * spectrum_matrix(rng.uniform(0, 1, n), 9))
    V, lm, _, _ = refine(N)
    wd, Vd = np.linalg.eigh(N)
    W = (Lx @ V) / np.sqrt(lm) @ (Lx @ V).T
    Wd = (Lx @ Vd) / np.sqrt(wd) @ (Lx @ Vd).T
    assert np.linalg.norm(W - Wd) / np.linalg.norm(Wd) < 1e-12
