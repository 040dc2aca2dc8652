"""ctypes binding of libhymor.so (the C ABI declared in include/hymor.h).

The library is built in-tree (hymor_gb300/_build/libhymor.so). There is no CPU
fallback: every entry point runs on the GPU and raises :class:`HymorError` when
the library or a device is missing.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_LIB = None

HYMOR_ERRORS = {
    -1: "HYMOR_ERR_INVALID",
    -2: "HYMOR_ERR_CUDA",
    -3: "HYMOR_ERR_NUMERIC",
    -4: "HYMOR_ERR_SHOCK_RANGE",
    -5: "HYMOR_ERR_TIMEOUT",
    -6: "HYMOR_ERR_NOT_READY",
}

EXPORTS = [
    "hymor_ctx_create", "hymor_ctx_destroy", "hymor_last_error", "hymor_set_state",
    "hymor_get_state", "hymor_residual", "hymor_set_flux", "hymor_step",
    "hymor_update_flow_cells", "hymor_cfl_timestep", "hymor_counters", "hymor_timer_start",
    "hymor_timer_stop", "hymor_profile_flux", "hymor_synchronize", "hymor_linearize",
    "hymor_jacobian_get", "hymor_jacobian_set", "hymor_matvec", "hymor_matvec_dev",
    "hymor_expm_apply", "hymor_expm_apply_dev", "hymor_device_alloc", "hymor_device_free",
    "hymor_memcpy_h2d", "hymor_memcpy_d2h", "hymor_bench_steps", "hymor_dot_dev",
    "hymor_krylov_orthogonalize", "hymor_krylov_rotate", "hymor_block4_apply_dev", "hymor_memcpy_d2d",
    "hymor_expm_apply_dev_noalloc", "hymor_step_kernels", "hymor_fp64_peak",
    "hymor_profile_phases", "hymor_advect", "hymor_bench_matvec", "hymor_operator_size",
    "hymor_shock_blocks_get", "hymor_shock_blocks_set", "hymor_shock_fields", "hymor_block4_apply_ext_dev",
    "hymor_expm_apply_multi_dev", "hymor_linearize_b", "hymor_b_get", "hymor_b_set", "hymor_recept_size",
    "hymor_recept_apply_dev", "hymor_recept_expm_dev", "hymor_set_upstream", "hymor_eigs", "hymor_tg_gain",
    "hymor_dense_schur", "hymor_dense_symeig", "hymor_set_step_viscous", "hymor_set_cfl_screen",
    "hymor_set_expm_arith",
    "hymor_autotune", "hymor_set_flux_tiling",
]


class KrylovOpts(ctypes.Structure):
    """hymor_krylov_opts (include/hymor.h)."""
    _fields_ = [("nev", ctypes.c_int32), ("ncv", ctypes.c_int32), ("maxit", ctypes.c_int32),
                ("block", ctypes.c_int32), ("order", ctypes.c_int32), ("flow_start", ctypes.c_int32),
                ("seed", ctypes.c_uint64), ("tol", ctypes.c_double)]


class HymorError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{HYMOR_ERRORS.get(code, code)}: {msg}")
        self.code = code


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libhymor.so (building it first if it is missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.build() if build_if_missing else _build.LIB
    if not os.path.exists(path):
        raise HymorError(-2, f"libhymor.so not found at {path}")
    L = ctypes.CDLL(path)
    vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)
    i, d = ctypes.c_int, ctypes.c_double
    sig = {
        "hymor_ctx_create": [vp, vp, ctypes.POINTER(vp)],
        "hymor_ctx_destroy": [vp],
        "hymor_set_state": [vp, dp, dp, dp, dp, dp, ip, d, dp],
        "hymor_get_state": [vp, dp, dp, dp, dp, dp, ip, dp, dp],
        "hymor_residual": [vp, dp],
        "hymor_set_flux": [vp, dp],
        "hymor_step": [vp, i],
        "hymor_advect": [vp, i, dp, dp, dp, dp, dp, ip, dp],
        "hymor_update_flow_cells": [vp],
        "hymor_cfl_timestep": [vp, dp],
        "hymor_counters": [vp, ip, ip],
        "hymor_step_kernels": [vp, ip],
        "hymor_fp64_peak": [vp, dp],
        "hymor_profile_phases": [vp, ctypes.POINTER(ctypes.c_float)],
        "hymor_timer_start": [vp],
        "hymor_timer_stop": [vp, ctypes.POINTER(ctypes.c_float)],
        "hymor_profile_flux": [vp, i, ctypes.POINTER(ctypes.c_float), ip],
        "hymor_synchronize": [vp],
        "hymor_linearize": [vp],
        "hymor_jacobian_get": [vp, dp],
        "hymor_jacobian_set": [vp, dp],
        "hymor_matvec": [vp, i, dp, dp, i],
        "hymor_matvec_dev": [vp, i, vp, vp, i],
        "hymor_bench_matvec": [vp, i, vp, vp, i, i, i, ctypes.POINTER(ctypes.c_float)],
        "hymor_expm_apply": [vp, i, d, i, i, dp, dp, i],
        "hymor_expm_apply_dev": [vp, i, d, i, i, vp, vp, i],
        "hymor_expm_apply_dev_noalloc": [vp, i, d, i, i, vp, vp, i],
        "hymor_expm_apply_multi_dev": [vp, i, dp, ip, i, vp, vp, i],
        "hymor_device_alloc": [vp, ctypes.c_uint64, ctypes.POINTER(vp)],
        "hymor_device_free": [vp, vp],
        "hymor_memcpy_h2d": [vp, vp, vp, ctypes.c_uint64],
        "hymor_memcpy_d2h": [vp, vp, vp, ctypes.c_uint64],
        "hymor_memcpy_d2d": [vp, vp, vp, ctypes.c_uint64],
        "hymor_bench_steps": [vp, i, ctypes.c_uint64, ctypes.POINTER(ctypes.c_float)],
        "hymor_dot_dev": [vp, ctypes.c_int64, i, vp, ctypes.c_int64, vp, dp],
        "hymor_krylov_orthogonalize": [vp, ctypes.c_int64, i, vp, ctypes.c_int64, vp, dp, i],
        "hymor_krylov_rotate": [vp, ctypes.c_int64, i, i, vp, ctypes.c_int64, dp],
        "hymor_block4_apply_dev": [vp, i, vp, vp, vp],
        "hymor_block4_apply_ext_dev": [vp, i, ctypes.c_int64, vp, vp, vp, vp],
        "hymor_operator_size": [vp, ctypes.POINTER(ctypes.c_int64)],
        "hymor_shock_blocks_get": [vp, ip, dp, dp, dp],
        "hymor_shock_blocks_set": [vp, ip, dp, dp, dp],
        "hymor_shock_fields": [vp, dp, dp],
        "hymor_linearize_b": [vp],
        "hymor_set_upstream": [vp, dp],
        "hymor_b_get": [vp, ip, dp, dp],
        "hymor_b_set": [vp, ip, dp, dp],
        "hymor_recept_size": [vp, i, ctypes.POINTER(ctypes.c_int64)],
        "hymor_recept_apply_dev": [vp, i, i, dp, d, vp, vp, i],
        "hymor_recept_expm_dev": [vp, i, i, dp, d, i, i, vp, vp, i],
        "hymor_eigs": [vp, vp, d, i, dp, dp, dp, dp, ip, vp],
        "hymor_tg_gain": [vp, vp, i, dp, dp, dp, dp, ip, dp, ip, vp],
        "hymor_dense_schur": [i, dp, i, dp, dp, dp, dp, ip],
        "hymor_dense_symeig": [i, dp, dp, dp],
        "hymor_set_step_viscous": [vp, i],
        "hymor_set_cfl_screen": [vp, i],
        "hymor_set_expm_arith": [vp, i],
        "hymor_autotune": [vp, i, ip, ctypes.POINTER(ctypes.c_float)],
        "hymor_set_flux_tiling": [vp, i, i, i],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.hymor_last_error.argtypes = [vp]
    L.hymor_last_error.restype = ctypes.c_char_p
    _LIB = L
    return L


def dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class Context:
    """One libhymor context: a solution resident on the GPU."""

    def __init__(self, cfg_struct, mesh_struct):
        self.L = load()
        h = ctypes.c_void_p()
        rc = self.L.hymor_ctx_create(ctypes.byref(cfg_struct), ctypes.byref(mesh_struct), ctypes.byref(h))
        self.h = h
        if rc != 0:
            msg = self.L.hymor_last_error(h).decode() if h else "context creation failed"
            if h:
                self.L.hymor_ctx_destroy(h)
                self.h = None
            raise HymorError(rc, msg)

    def check(self, rc: int):
        if rc != 0:
            raise HymorError(rc, self.L.hymor_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.hymor_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
