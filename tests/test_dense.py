"""CPU tests of the dense steps of the device Krylov-Schur solvers (hymor_dense_schur,
hymor_dense_symeig: Francis QR, Schur reordering by block swaps, Jacobi) against numpy's
LAPACK on random and structured matrices. These run on the host part of libhymor and need
no GPU."""
import ctypes

import numpy as np
import pytest

from hymor_gb300 import _lib
from hymor_gb300._lib import dp, ip


def schur(A, nsel):
    L = _lib.load()
    n = A.shape[0]
    Af = np.asfortranarray(A, dtype=np.float64)
    T, Z = np.zeros((n, n), order="F"), np.zeros((n, n), order="F")
    wr, wi = np.zeros(n), np.zeros(n)
    lead = np.zeros(1, dtype=np.int32)
    rc = L.hymor_dense_schur(n, dp(Af), nsel, dp(T), dp(Z), dp(wr), dp(wi), ip(lead))
    assert rc == 0
    return T, Z, wr + 1j * wi, int(lead[0])


def matrices():
    rng = np.random.Generator(np.random.PCG64(12))
    out = []
    for n in (1, 2, 3, 7, 24, 60, 97):
        out.append(rng.standard_normal((n, n)))
    # a projected-operator-like matrix: eigenvalues clustered near the unit circle
    n = 40
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    D = np.diag(0.8 + 0.15 * rng.random(n)) + np.triu(0.01 * rng.standard_normal((n, n)), 1)
    out.append(Q @ D @ Q.T)
    # block rotation: conjugate pairs of equal modulus
    R = np.zeros((12, 12))
    for k in range(6):
        a = 0.3 * k
        R[2 * k:2 * k + 2, 2 * k:2 * k + 2] = (1 - 0.05 * k) * np.array([[np.cos(a), -np.sin(a)], [np.sin(a), np.cos(a)]])
    Q, _ = np.linalg.qr(rng.standard_normal((12, 12)))
    out.append(Q @ R @ Q.T)
    # upper Hessenberg with a Krylov-Schur restart's leading dense block
    H = np.triu(rng.standard_normal((30, 30)), -1)
    H[:10, :10] = rng.standard_normal((10, 10))
    out.append(H)
    return out


@pytest.mark.parametrize("idx", range(10))
def test_dense_schur(idx):
    A = matrices()[idx]
    n = A.shape[0]
    nsel = max(1, n // 3)
    T, Z, w, lead = schur(A, nsel)
    scale = max(np.linalg.norm(A), 1e-300)
    assert np.linalg.norm(Z.T @ Z - np.eye(n)) < 1e-13 * n
    assert np.linalg.norm(Z @ T @ Z.T - A) < 1e-13 * n * scale
    assert np.all(np.tril(T, -2) == 0)
    # sub-diagonal entries only inside 2 x 2 blocks of complex pairs
    for k in range(n - 1):
        if T[k + 1, k] != 0:
            assert abs(w[k].imag) > 0 and np.isclose(w[k], np.conj(w[k + 1]))
    # each eigenvalue within its condition number (1 / |y^H x|, unit left and right
    # eigenvectors) times the backward error of numpy's and this factorisation
    sla = pytest.importorskip("scipy.linalg")
    ref, yl, xr = sla.eig(A, left=True, right=True)
    cond = 1.0 / np.maximum(np.abs(np.sum(np.conj(yl) * xr, axis=0)), 1e-300)
    for x in w:
        i = np.argmin(np.abs(ref - x))
        assert abs(ref[i] - x) <= 1e-13 * n * scale * cond[i] + 1e-14 * scale
    # the leading rows hold the nsel largest moduli of the factorisation (whole pairs)
    assert lead >= nsel
    if lead < n:
        assert np.max(np.abs(w[lead:])) <= np.min(np.abs(w[:lead])) * (1 + 1e-12)


@pytest.mark.parametrize("n", [1, 5, 33, 80])
def test_dense_symeig(n):
    L = _lib.load()
    rng = np.random.Generator(np.random.PCG64(n))
    B = rng.standard_normal((n, n))
    A = np.asfortranarray(B + B.T)
    w, V = np.zeros(n), np.zeros((n, n), order="F")
    assert L.hymor_dense_symeig(n, dp(A), dp(w), dp(V)) == 0
    ref = np.linalg.eigvalsh(A)
    assert np.allclose(np.sort(w), ref, rtol=0, atol=1e-12 * np.max(np.abs(ref)))
    assert np.linalg.norm(V.T @ V - np.eye(n)) < 1e-12 * n
    assert np.linalg.norm(A @ V - V * w) < 1e-12 * n * np.linalg.norm(A)


def test_dense_rejects_bad_sizes():
    L = _lib.load()
    A = np.zeros(4)
    out = np.zeros(4)
    assert L.hymor_dense_schur(0, dp(A), 0, dp(out), dp(out), dp(out), dp(out), None) == -1
    assert L.hymor_dense_schur(2, dp(A), 3, dp(out), dp(out), dp(out), dp(out), None) == -1
