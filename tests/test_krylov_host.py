"""The Krylov-Schur drivers (single-vector and block) on the CPU: the device building
blocks of libhymor (allocation, copies, Gram-Schmidt, restart rotation) are replaced by a
numpy stand-in with the same C-ABI signatures, so the host logic of the restarts, the
block Hessenberg bookkeeping and the convergence test run against dense eigensolvers."""
import ctypes

import numpy as np
import pytest

from hymor_gb300 import krylov as K


class _NumpyLib:
    """hymor_device_alloc / memcpy / krylov_orthogonalize / krylov_rotate over host memory."""

    def __init__(self):
        self.bufs = {}

    @staticmethod
    def _addr(p):
        if isinstance(p, ctypes.c_void_p):
            return p.value
        if isinstance(p, int):
            return p
        return ctypes.cast(p, ctypes.c_void_p).value

    def _view(self, addr, count):
        return np.ctypeslib.as_array(ctypes.cast(ctypes.c_void_p(addr), ctypes.POINTER(ctypes.c_double)),
                                     shape=(count,))

    def hymor_device_alloc(self, h, nbytes, pptr):
        a = np.zeros(max(1, nbytes // 8))
        self.bufs[a.ctypes.data] = a
        pptr._obj.value = a.ctypes.data  # pptr = ctypes.byref(c_void_p)
        return 0

    def hymor_device_free(self, h, ptr):
        self.bufs.pop(self._addr(ptr), None)
        return 0

    def hymor_memcpy_h2d(self, h, dst, src, nbytes):
        ctypes.memmove(self._addr(dst), self._addr(src), nbytes)
        return 0

    hymor_memcpy_d2h = hymor_memcpy_h2d
    hymor_memcpy_d2d = hymor_memcpy_h2d

    def hymor_krylov_orthogonalize(self, h, n, m, dV, ldv, dw, hout, out_col):
        V = self._view(self._addr(dV), ldv * (max(m, out_col + 1))).reshape(-1, ldv).T[:n]
        w = self._view(self._addr(dw), n)
        hh = np.ctypeslib.as_array(hout, shape=(m + 1,))
        c = np.zeros(m)
        for _ in range(2):
            if m:
                d = V[:, :m].T @ w
                w -= V[:, :m] @ d
                c += d
        hh[:m] = c
        hh[m] = np.linalg.norm(w)
        if out_col >= 0:
            V[:, out_col] = w / hh[m]
        return 0

    def hymor_krylov_rotate(self, h, n, m, k, dV, ldv, Q):
        V = self._view(self._addr(dV), ldv * m).reshape(m, ldv).T[:n]
        q = np.ctypeslib.as_array(Q, shape=(m * k,)).reshape(k, m).T
        V[:, :k] = V[:, :m] @ q
        return 0


class _Ctx:
    def __init__(self):
        self.L = _NumpyLib()
        self.h = None

    def check(self, rc):
        assert rc == 0


def _op(A, ctx):
    n = A.shape[0]

    def one(src, dst):
        x = ctx.L._view(src, n)
        ctx.L._view(dst, n)[:] = A @ x

    def block(src, dst, k):
        X = ctx.L._view(src, n * k).reshape(k, n).T
        ctx.L._view(dst, n * k).reshape(k, n)[:] = (A @ X).T
    return one, block


def _matrix(n, symmetric, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    lam = 0.97 ** np.arange(n)
    if symmetric:
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        return (Q * lam) @ Q.T, lam
    # a few complex pairs among the dominant eigenvalues
    Q = rng.standard_normal((n, n))
    D = np.diag(lam)
    for k in (1, 5):
        D[k, k + 1], D[k + 1, k] = 0.05, -0.05
        D[k + 1, k + 1] = D[k, k]
    A = Q @ D @ np.linalg.inv(Q)
    return A, np.linalg.eigvals(D)


@pytest.mark.parametrize("symmetric", [False, True])
@pytest.mark.parametrize("block", [1, 3, 4])
def test_block_krylov_schur_matches_dense(symmetric, block):
    n, nev = 240, 5  # the 5 largest in magnitude split no complex pair
    A, lam = _matrix(n, symmetric, 11)
    ctx = _Ctx()
    _, blk = _op(A, ctx)
    theta, resid, nops = K.block_krylov_schur(ctx, n, blk, nev, ncv=30, block=block, tol=1e-10, maxit=400,
                                              seed=5, symmetric=symmetric)
    ref = lam[np.argsort(-np.abs(lam))][:nev]
    got = np.sort_complex(np.asarray(theta, dtype=complex))
    want = np.sort_complex(np.asarray(ref, dtype=complex))
    assert np.max(np.abs(got - want)) < 1e-8
    assert np.all(resid <= 1e-10 * np.abs(theta))
    assert nops % block == 0


def test_block_size_one_is_the_single_vector_method():
    n, nev = 200, 4
    A, _ = _matrix(n, False, 12)
    ctx = _Ctx()
    one, blk = _op(A, ctx)
    t1, _, n1 = K.krylov_schur(ctx, n, one, nev, 20, tol=1e-10, maxit=400, seed=7)
    t2, _, n2 = K.block_krylov_schur(ctx, n, blk, nev, 20, block=1, tol=1e-10, maxit=400, seed=7)
    assert np.max(np.abs(np.sort_complex(t1.astype(complex)) - np.sort_complex(t2.astype(complex)))) < 1e-9


def test_block_krylov_schur_rejects_small_basis():
    ctx = _Ctx()
    with pytest.raises(K.HymorError):
        K.block_krylov_schur(ctx, 50, None, 4, ncv=10, block=4)


@pytest.mark.parametrize("symmetric", [False, True])
@pytest.mark.parametrize("block", [0, 3])
def test_ritz_vectors_are_eigenvectors(symmetric, block):
    """want_vectors: the Ritz vectors come back with unit norm and A x = theta x to the
    residual the solve reached (block 0: the single-vector driver)."""
    n, nev = 240, 5
    A, _ = _matrix(n, symmetric, 11)
    ctx = _Ctx()
    one, blk = _op(A, ctx)
    if block:
        theta, resid, nops, X = K.block_krylov_schur(ctx, n, blk, nev, ncv=30, block=block, tol=1e-10,
                                                     maxit=400, seed=5, symmetric=symmetric, want_vectors=True)
    else:
        theta, resid, nops, X = K.krylov_schur(ctx, n, one, nev, 30, tol=1e-10, maxit=400, seed=5,
                                               symmetric=symmetric, want_vectors=True)
    assert X.shape == (n, nev)
    assert np.iscomplexobj(X) == (not symmetric)
    for i in range(nev):
        x = X[:, i]
        assert abs(np.linalg.norm(x) - 1) < 1e-12
        assert np.linalg.norm(A @ x - theta[i] * x) <= 1e-9 * abs(theta[i])


def test_lockstep_solves_match_separate_solves():
    """krylov_schur_many runs one solve per operator in lockstep (one batched application
    per round): each solve gives exactly its own krylov_schur result, also when the solves
    converge after different numbers of restarts."""
    n, nev = 200, 3
    mats = [_matrix(n, True, seed)[0] * scale for seed, scale in ((21, 1.0), (22, 3.0), (23, 0.5))]
    ctx = _Ctx()
    separate = []
    for i, A in enumerate(mats):
        one, _ = _op(A, ctx)
        separate.append(K.krylov_schur(ctx, n, one, nev, ncv=14, tol=1e-10, maxit=300, seed=7 + i, symmetric=True))
    calls = []

    def apply_many(idx, srcs, dsts):
        calls.append(len(idx))
        for i, src, dst in zip(idx, srcs, dsts):
            ctx.L._view(dst, n)[:] = mats[i] @ ctx.L._view(src, n)
    probs = [dict(nev=nev, ncv=14, tol=1e-10, maxit=300, seed=7 + i, symmetric=True) for i in range(3)]
    together = K.krylov_schur_many(ctx, n, apply_many, probs)
    for (t1, r1, n1), (t2, r2, n2) in zip(separate, together):
        assert np.array_equal(t1, t2) and np.array_equal(r1, r2) and n1 == n2
    assert max(calls) == 3 and sum(calls) == sum(s[2] for s in separate)
