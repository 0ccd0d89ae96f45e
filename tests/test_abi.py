"""The C-ABI library loads and exports every entry point include/dluxgb.h declares."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(dlx_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_entry_points():
    names = _declared()
    assert "dlx_poly_psf" in names and "dlx_mft_forward" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    import dlux_gb300._lib as L
    lib = L.load()
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_signatures_cover_header():
    import dlux_gb300._lib as L
    assert set(_declared()) <= set(L.exported_symbols())


def test_version_and_error_string_need_no_gpu():
    import dlux_gb300._lib as L
    lib = L.load()
    assert lib.dlx_version() == 100
    assert isinstance(lib.dlx_last_error(), bytes)


def test_argument_errors_are_reported_without_a_gpu():
    """Validation happens before any device call: bad sizes map to ValueError."""
    import dlux_gb300._lib as L
    lib = L.load()
    st = lib.dlx_downsample(None, 10, 3, 0, None, None, None)
    assert st == L.DLX_ERR_SHAPE
    assert b"not divisible" in lib.dlx_last_error()
    with pytest.raises(ValueError):
        L.check(st)
    st = lib.dlx_downsample(None, 10, 0, 0, None, None, None)
    assert st == L.DLX_ERR_ARG
    plan = ctypes.c_void_p()
    d = L.MftDesc(0, 16, 8, 0.1, 0.05, 0.0, 0.0, 0.0, 0, 0)
    st = lib.dlx_mft_plan_create(ctypes.byref(d), L.dbl_array([1.0]), ctypes.byref(plan))
    assert st == L.DLX_ERR_SHAPE


def test_plan_state_calls_refuse_a_null_plan():
    """The forward-state calls of poly plans check their plan before any device work."""
    import dlux_gb300._lib as L
    lib = L.load()
    assert lib.dlx_poly_keep_focal(None, 1) == L.DLX_ERR_ARG
    assert b"null plan" in lib.dlx_last_error()
    assert lib.dlx_poly_reuse_forward(None, 1) == L.DLX_ERR_ARG
    tok = ctypes.c_ulonglong(0)
    assert lib.dlx_poly_forward_token(None, ctypes.byref(tok)) == L.DLX_ERR_ARG
