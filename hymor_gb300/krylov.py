"""Device-resident Krylov–Schur eigensolver over libhymor.

The reference runs Arpack's implicitly restarted Arnoldi on the host and ships
every Krylov vector host→device→host around a CuSparse propagation
(Eigenvalues/EIGENVALUES.jl:153-159, ARNOLDI_POWER_GPU.jl:36-45). Here the Krylov
basis stays in HBM: the operator, the classical Gram–Schmidt (twice) with
deterministic device reductions and the restart rotation all run through the C
ABI, and only the small projected matrix (<= ncv x ncv) comes back to the host,
where its Schur form is computed (Stewart's Krylov–Schur restart, SIAM J. Matrix
Anal. Appl. 23 (2001) 601-614).
"""
from __future__ import annotations

import ctypes

import numpy as np
import scipy.linalg as sla

from ._lib import HymorError, dp


class DeviceBuffer:
    """A device allocation owned by a libhymor context."""

    def __init__(self, ctx, nbytes: int):
        self.ctx = ctx
        self.ptr = ctypes.c_void_p()
        ctx.check(ctx.L.hymor_device_alloc(ctx.h, int(nbytes), ctypes.byref(self.ptr)))
        self.nbytes = nbytes

    def addr(self, offset_doubles: int = 0) -> int:
        return self.ptr.value + 8 * int(offset_doubles)

    def upload(self, a: np.ndarray, offset_doubles: int = 0):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.ctx.check(self.ctx.L.hymor_memcpy_h2d(self.ctx.h, self.addr(offset_doubles), a.ctypes.data, a.nbytes))

    def download(self, n: int, offset_doubles: int = 0) -> np.ndarray:
        out = np.empty(n)
        self.ctx.check(self.ctx.L.hymor_memcpy_d2h(self.ctx.h, out.ctypes.data, self.addr(offset_doubles), out.nbytes))
        return out

    def free(self):
        if self.ptr.value:
            self.ctx.L.hymor_device_free(self.ctx.h, self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def ritz_vectors(ctx, V, n: int, m: int, Y: np.ndarray) -> np.ndarray:
    """Ritz vectors V[:, :m] Y (columns of unit norm when Y's are) on the device. A complex Y
    goes as its real and imaginary parts in one rotation of the basis (V[:, :2k] =
    V[:, :m] [Re Y, Im Y]), which overwrites the basis: call it last."""
    k = Y.shape[1]
    cplx = np.iscomplexobj(Y)
    Q = np.hstack([Y.real, Y.imag]) if cplx else np.asarray(Y, dtype=np.float64)
    if Q.shape[1] > m:
        raise HymorError(-1, "too many Ritz vectors for the basis")
    ctx.check(ctx.L.hymor_krylov_rotate(ctx.h, n, m, Q.shape[1], V.ptr, n, dp(np.asfortranarray(Q))))
    X = V.download(n * Q.shape[1]).reshape(Q.shape[1], n).T
    return X[:, :k] + 1j * X[:, k:] if cplx else X.copy()


def krylov_schur(ctx, n: int, apply_op, nev: int, ncv: int, tol: float = 1e-8, maxit: int = 200,
                 seed: int = 3, symmetric: bool = False, v0: np.ndarray | None = None,
                 want_vectors: bool = False):
    """Largest-magnitude eigenpairs of a real operator held on the device.

    apply_op(src_addr, dst_addr) writes OP(v) for device vectors of length n.
    Returns (theta, resid, nops): Ritz values, their residual norms ||OP x - theta x||
    (x of unit norm) and the number of operator applications; with want_vectors also the
    Ritz vectors (n x nev, complex unless symmetric), or None when tol was not reached."""
    steps = krylov_schur_steps(ctx, n, nev, ncv, tol, maxit, seed, symmetric, v0, want_vectors)
    try:
        req = next(steps)
        while True:
            apply_op(*req)
            req = steps.send(None)
    except StopIteration as done:
        return done.value


def krylov_schur_many(ctx, n: int, apply_many, problems: list[dict]):
    """Several Krylov-Schur solves in lockstep, so that each round applies the operators of
    all unfinished solves in one batched call.

    problems: keyword arguments of krylov_schur (nev, ncv, tol, maxit, seed, symmetric, v0,
    want_vectors) per solve. apply_many(idx, srcs, dsts) applies operator idx[c] to the
    device vector at srcs[c] into dsts[c] for every c; idx is increasing. Each solve makes
    the same operations, in the same order, as its own krylov_schur call. Returns the
    results of krylov_schur, one per problem."""
    gens = [krylov_schur_steps(ctx, n, **p) for p in problems]
    results: list = [None] * len(gens)
    pending = {}
    for i, g in enumerate(gens):
        try:
            pending[i] = next(g)
        except StopIteration as done:
            results[i] = done.value
    while pending:
        idx = sorted(pending)
        apply_many(idx, [pending[i][0] for i in idx], [pending[i][1] for i in idx])
        for i in idx:
            try:
                pending[i] = gens[i].send(None)
            except StopIteration as done:
                results[i] = done.value
                del pending[i]
    return results


def krylov_schur_steps(ctx, n: int, nev: int, ncv: int, tol: float = 1e-8, maxit: int = 200, seed: int = 3,
                       symmetric: bool = False, v0: np.ndarray | None = None, want_vectors: bool = False):
    """krylov_schur as a generator: yields (src_addr, dst_addr) whenever it needs the
    operator applied, and returns krylov_schur's result."""
    if not (0 < nev < ncv):
        raise HymorError(-1, "need 0 < nev < ncv")
    L = ctx.L
    V = DeviceBuffer(ctx, 8 * n * (ncv + 1))
    w = DeviceBuffer(ctx, 8 * n)
    rng = np.random.Generator(np.random.PCG64(seed))
    x0 = rng.standard_normal(n) if v0 is None else np.asarray(v0, dtype=np.float64)
    V.upload(x0 / np.linalg.norm(x0))
    H = np.zeros((ncv + 1, ncv))
    h = np.empty(ncv + 2)
    p = 0       # columns of the current Krylov decomposition already built
    nops = 0
    theta = resid = X = None
    for it in range(maxit):
        for j in range(p, ncv):
            yield V.addr(j * n), w.addr()
            nops += 1
            ctx.check(L.hymor_krylov_orthogonalize(ctx.h, n, j + 1, V.ptr, n, w.ptr, dp(h), j + 1))
            H[: j + 1, j] = h[: j + 1]
            H[j + 1, j] = h[j + 1]
            if h[j + 1] == 0:
                raise HymorError(-3, "Krylov breakdown (invariant subspace found)")
        Hm = H[:ncv, :ncv]
        b = H[ncv, :ncv]
        if symmetric:
            Hs = 0.5 * (Hm + Hm.T)
            vals, Y = np.linalg.eigh(Hs)
            order = np.argsort(-np.abs(vals))
            vals, Y = vals[order], Y[:, order]
            res = np.abs(b @ Y)
        else:
            vals, Y = np.linalg.eig(Hm)
            order = np.argsort(-np.abs(vals))
            vals, Y = vals[order], Y[:, order]
            Y = Y / np.linalg.norm(Y, axis=0)
            res = np.abs(b @ Y)
        theta, resid = vals[:nev], res[:nev]
        if np.all(resid <= tol * np.abs(theta)):
            if want_vectors:
                X = ritz_vectors(ctx, V, n, ncv, Y[:, :nev])
            break
        # Krylov-Schur restart: keep the wanted Schur vectors
        keep = min(nev + max(2, (ncv - nev) // 2), ncv - 1)
        if symmetric:
            T = np.diag(vals[:keep])
            Q = Y[:, :keep]
        else:
            thr = np.sort(np.abs(vals))[::-1][keep - 1]
            Tfull, Qfull, sdim = sla.schur(Hm, output="real", sort=lambda re, im: np.hypot(re, im) >= thr * (1 - 1e-12))
            keep = max(1, min(sdim, ncv - 1))
            T = Tfull[:keep, :keep]
            Q = Qfull[:, :keep]
        Qc = np.asfortranarray(Q)
        ctx.check(L.hymor_krylov_rotate(ctx.h, n, ncv, keep, V.ptr, n, dp(Qc)))
        # the residual vector becomes column `keep`
        ctx.check(L.hymor_memcpy_d2d(ctx.h, V.addr(keep * n), V.addr(ncv * n), 8 * n))
        Hn = np.zeros_like(H)
        Hn[:keep, :keep] = T
        Hn[keep, :keep] = b @ Q
        H = Hn
        p = keep
    V.free()
    w.free()
    return (theta, resid, nops, X) if want_vectors else (theta, resid, nops)


def block_krylov_schur(ctx, n: int, apply_block, nev: int, ncv: int, block: int, tol: float = 1e-8,
                       maxit: int = 200, seed: int = 3, symmetric: bool = False, start_mask=None,
                       want_vectors: bool = False):
    """Block Krylov-Schur: the Krylov basis grows `block` vectors at a time, so that every
    operator application propagates a whole block in one batched call (Zhou and Saad,
    "Block Krylov-Schur method for large symmetric eigenvalue problems", Numer. Algorithms 47
    (2008) 341-359; the non-symmetric restart is Stewart's, as in krylov_schur).

    apply_block(src_addr, dst_addr, k) writes OP(v_i) for k contiguous device vectors of
    length n. Each new vector is orthogonalised (classical Gram-Schmidt, twice, on the
    device) against the basis and the block's earlier vectors, so the projected matrix is
    block upper Hessenberg with `block` subdiagonals: A V[:, :m] = V[:, :m+block] H.
    Returns (theta, resid, nops) like krylov_schur; nops counts single-vector
    applications (block per call); with want_vectors also the Ritz vectors, as
    krylov_schur. start_mask (length n, optional) multiplies the random start block, e.g.
    to keep it on a subspace the operator leaves invariant."""
    b = int(block)
    if b < 1 or not (0 < nev < ncv) or ncv < nev + 2 * b:
        raise HymorError(-1, "need block >= 1 and 0 < nev, nev + 2 block <= ncv")
    L = ctx.L
    cap = ncv + 2 * b  # a cycle may grow up to block - 1 columns past ncv
    V = DeviceBuffer(ctx, 8 * n * cap)
    W = DeviceBuffer(ctx, 8 * n * b)
    rng = np.random.Generator(np.random.PCG64(seed))
    X0 = rng.standard_normal((b, n))
    if start_mask is not None:
        X0 *= np.asarray(start_mask, dtype=np.float64)[None, :]
    W.upload(X0.ravel())
    h = np.empty(cap + 2)
    for i in range(b):  # orthonormal start block
        ctx.check(L.hymor_krylov_orthogonalize(ctx.h, n, i, V.ptr, n, W.addr(i * n), dp(h), i))
        if h[i] == 0:
            raise HymorError(-3, "start block is rank deficient")
    H = np.zeros((cap, cap))
    p = 0
    nops = 0
    theta = resid = X = None
    for it in range(maxit):
        m = p + b * max(1, -(-(ncv - p) // b))
        for j in range(p, m, b):
            apply_block(V.addr(j * n), W.addr(), b)
            nops += b
            for i in range(b):
                J = j + b + i  # orthonormal basis vectors so far
                ctx.check(L.hymor_krylov_orthogonalize(ctx.h, n, J, V.ptr, n, W.addr(i * n), dp(h), J))
                H[:J, j + i] = h[:J]
                H[J, j + i] = h[J]
                if h[J] == 0:
                    raise HymorError(-3, "Krylov breakdown (invariant subspace found)")
        Hm = H[:m, :m]
        B = H[m:m + b, :m]
        if symmetric:
            vals, Y = np.linalg.eigh(0.5 * (Hm + Hm.T))
        else:
            vals, Y = np.linalg.eig(Hm)
        order = np.argsort(-np.abs(vals))
        vals, Y = vals[order], Y[:, order]
        if not symmetric:
            Y = Y / np.linalg.norm(Y, axis=0)
        res = np.linalg.norm(B @ Y, axis=0)
        theta, resid = vals[:nev], res[:nev]
        if np.all(resid <= tol * np.abs(theta)):
            if want_vectors:
                X = ritz_vectors(ctx, V, n, m, Y[:, :nev])
            break
        # restart: keep the wanted Schur vectors, leave room for the residual block
        keep = min(nev + max(2, (m - nev) // 2), m - b)
        if symmetric:
            T = np.diag(vals[:keep])
            Q = Y[:, :keep]
        else:
            thr = np.sort(np.abs(vals))[::-1][keep - 1]
            Tfull, Qfull, sdim = sla.schur(Hm, output="real", sort=lambda re, im: np.hypot(re, im) >= thr * (1 - 1e-12))
            keep = max(1, min(sdim, m - b))
            if keep < m and Tfull[keep, keep - 1] != 0:
                keep -= 1  # never split a 2 x 2 block of a complex pair
            T = Tfull[:keep, :keep]
            Q = Qfull[:, :keep]
        ctx.check(L.hymor_krylov_rotate(ctx.h, n, m, keep, V.ptr, n, dp(np.asfortranarray(Q))))
        # the residual block becomes columns keep .. keep + b - 1 (keep + b <= m: no overlap)
        ctx.check(L.hymor_memcpy_d2d(ctx.h, V.addr(keep * n), V.addr(m * n), 8 * n * b))
        Hn = np.zeros_like(H)
        Hn[:keep, :keep] = T
        Hn[keep:keep + b, :keep] = B @ Q
        H = Hn
        p = keep
    V.free()
    W.free()
    return (theta, resid, nops, X) if want_vectors else (theta, resid, nops)
