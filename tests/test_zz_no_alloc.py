"""The allocation-free Taylor propagator (hymor_expm_apply_dev_noalloc).

Some callers cannot allocate device memory while they call us: a host framework
that calls from inside its own CUDA stream capture, or a service that reserves its
whole memory budget up front. This entry point takes its work vectors from one
fixed device array instead of allocating them. It must give the same result as the
allocating entry point (hymor_expm_apply_dev), call after call, since every call
reuses the same array. This file sorts last so that a run stopping at the first
failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from hymor_gb300 import case as C
from hymor_gb300 import solver as S
from hymor_gb300.krylov import DeviceBuffer

pytestmark = pytest.mark.gpu


def test_noalloc_propagator_matches_allocating_one(require_gpu):
    cfg = C.cylinder_config(40, 24)
    cs = C.initial_state(cfg)
    sol = S.Solution(cs)
    _, L = S.LINEARIZE_L(sol)
    lib, h = sol.ctx.L, sol.ctx.h
    k = 2
    n = 4 * sol.N * k
    X, Y_ref, Y_new = (DeviceBuffer(sol.ctx, 8 * n) for _ in range(3))
    rng = np.random.Generator(np.random.PCG64(21))
    dt = 0.5 * S.CFL_TIMESTEP(sol)
    for call in range(2):  # two calls in a row reuse the shared scratch
        x = rng.standard_normal(n)
        X.upload(x)
        sol.ctx.check(lib.hymor_expm_apply_dev(h, k, dt, 7, 5, X.ptr, Y_ref.ptr, call % 2))
        sol.ctx.check(lib.hymor_expm_apply_dev_noalloc(h, k, dt, 7, 5, X.ptr, Y_new.ptr, call % 2))
        sol.ctx.check(lib.hymor_synchronize(h))
        a, b = Y_new.download(n), Y_ref.download(n)
        assert np.isfinite(b).all()
        assert np.max(np.abs(a - b)) <= 1e-13 * np.max(np.abs(b)), call


def test_noalloc_rejects_oversized_request(require_gpu):
    cfg = C.cylinder_config(40, 24)
    sol = S.Solution(C.initial_state(cfg))
    S.LINEARIZE_L(sol)
    lib, h = sol.ctx.L, sol.ctx.h
    k = (1 << 20) // (4 * sol.N) + 1
    X = DeviceBuffer(sol.ctx, 8)
    rc = lib.hymor_expm_apply_dev_noalloc(h, k, 1e-3, 1, 5, X.ptr, X.ptr, 0)
    assert rc == -1
    assert "exceeds its fixed work size" in lib.hymor_last_error(h).decode()
