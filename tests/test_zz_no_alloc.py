"""The allocation-free Taylor propagator (hymor_expm_apply_dev_noalloc).

Some callers cannot call cudaMalloc during a solve: a service that reserves its whole
device-memory budget at start-up, or a host runtime whose own pool allocator owns the
device memory. This entry point takes its work vectors from one fixed device array
instead of allocating them, and launches every Taylor step directly. It must give the
same result as the allocating entry point (hymor_expm_apply_dev), call after call,
since every call reuses the same array: on the stencil operator and on the operator
with the shock-position unknowns (where the allocating entry point replays a CUDA
graph of one step and this one launches each step). This file sorts last so that a
run stopping at the first failure has already run every other test."""
import os
import subprocess
import sys

import numpy as np
import pytest

from hymor_gb300 import case as C
from hymor_gb300 import solver as S
from hymor_gb300.krylov import DeviceBuffer

pytestmark = pytest.mark.gpu


def _compare(sol, k, nsteps, order, seed, tol):
    # both entry points in FP64 (the allocating one would otherwise run its cooperative
    # launches in float-float)
    sol.set_expm_arith(0)
    lib, h = sol.ctx.L, sol.ctx.h
    n = sol.operator_size() * k
    X, Y_ref, Y_new = (DeviceBuffer(sol.ctx, 8 * n) for _ in range(3))
    rng = np.random.Generator(np.random.PCG64(seed))
    dt = 0.5 * S.CFL_TIMESTEP(sol)
    for call in range(2):  # two calls in a row reuse the shared scratch
        x = rng.standard_normal(n)
        X.upload(x)
        sol.ctx.check(lib.hymor_expm_apply_dev(h, k, dt, nsteps, order, X.ptr, Y_ref.ptr, call % 2))
        sol.ctx.check(lib.hymor_expm_apply_dev_noalloc(h, k, dt, nsteps, order, X.ptr, Y_new.ptr, call % 2))
        sol.ctx.check(lib.hymor_synchronize(h))
        a, b = Y_new.download(n), Y_ref.download(n)
        assert np.isfinite(b).all()
        assert np.max(np.abs(a - b)) <= tol * np.max(np.abs(b)), call


def test_noalloc_propagator_matches_allocating_one(require_gpu):
    sol = S.Solution(C.initial_state(C.cylinder_config(40, 24)))
    S.LINEARIZE_L(sol)
    # 7 steps of order 5: the allocating entry point runs its cooperative kernel here,
    # the same per-cell arithmetic in another launch structure
    _compare(sol, k=2, nsteps=7, order=5, seed=21, tol=1e-13)
    sol.close()


def test_noalloc_propagator_with_shock_unknowns(require_gpu):
    """With the shock-position unknowns both entry points launch the same kernels (the
    allocating one replays them from a CUDA graph), so the results agree bit for bit."""
    cfg = C.cylinder_config(30, 24, perturb_shock=True)
    sol = S.Solution(C.initial_state(cfg))
    S.ADVECT_FLOW(sol, 5)
    S.LINEARIZE_L(sol)
    assert sol.operator_size() == 4 * sol.N + cfg.nchi
    _compare(sol, k=1, nsteps=6, order=5, seed=22, tol=0.0)
    sol.close()


def test_noalloc_rejects_oversized_request(require_gpu):
    sol = S.Solution(C.initial_state(C.cylinder_config(40, 24)))
    S.LINEARIZE_L(sol)
    lib, h = sol.ctx.L, sol.ctx.h
    k = (1 << 20) // (4 * sol.N) + 1
    X = DeviceBuffer(sol.ctx, 8)
    rc = lib.hymor_expm_apply_dev_noalloc(h, k, 1e-3, 1, 5, X.ptr, X.ptr, 0)
    assert rc == -1
    assert "exceeds its fixed work size" in lib.hymor_last_error(h).decode()
    sol.close()


def test_noalloc_in_fresh_process(require_gpu):
    """The first call of a process looks up the array's address: run the comparison alone
    in a new interpreter."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.path[:0] = [%r, %r]; import test_zz_no_alloc as t; "
            "from hymor_gb300 import case as C, solver as S; "
            "s = S.Solution(C.initial_state(C.cylinder_config(40, 24))); S.LINEARIZE_L(s); "
            "t._compare(s, k=2, nsteps=7, order=5, seed=23, tol=1e-13); print('fresh ok')"
            % (root, os.path.join(root, "tests")))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "fresh ok" in r.stdout, r.stdout + r.stderr
