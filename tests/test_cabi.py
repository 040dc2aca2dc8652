"""CPU tests of the C ABI boundary: the library builds, loads and exports every entry
point include/hymor.h declares; configuration errors surface before any device work."""
import ctypes
import os
import re

import pytest

from hymor_gb300 import _lib
from hymor_gb300 import case as C

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "hymor.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hymor_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for needed in ("hymor_ctx_create", "hymor_residual", "hymor_step", "hymor_linearize",
                   "hymor_matvec", "hymor_expm_apply"):
        assert needed in syms


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


@pytest.mark.parametrize("kw, text", [
    (dict(bc_eta1="symmetry"), "shock fitting needs boundary_eta1 = shock"),
    (dict(bc_chi0="shock", shock_enabled=False), "only valid on eta1"),
    (dict(Re=-1.0), "Re and Pr must be positive"),
])
def test_invalid_config_rejected(kw, text):
    """Input validation (VERIFY_INPUT_DATA.jl / APPLY_BOUNDARY_CONDITIONS.jl error paths)
    happens in hymor_ctx_create before any CUDA call."""
    cfg = C.cylinder_config(20, 16, **kw)
    cs = C.initial_state(C.cylinder_config(20, 16))
    L = _lib.load()
    st = C.config_struct(cfg)
    ms, keep = cs.mesh_struct()
    h = ctypes.c_void_p()
    rc = L.hymor_ctx_create(ctypes.byref(st), ctypes.byref(ms), ctypes.byref(h))
    assert rc == -1
    assert text in L.hymor_last_error(h).decode()
    L.hymor_ctx_destroy(h)


@pytest.mark.parametrize("name", ["hymor_set_step_viscous", "hymor_set_cfl_screen", "hymor_set_expm_arith"])
def test_switches_reject_bad_arguments(name):
    """The arithmetic and schedule switches of the step and the propagator reject a null
    context and modes other than 0 and 1 before touching a device."""
    L = _lib.load()
    fn = getattr(L, name)
    for ctx, mode in ((None, 1), (None, 0), (None, 2)):
        assert fn(ctx, mode) == -1
