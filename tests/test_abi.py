"""The C-ABI library loads and exports every symbol include/fdadi.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

from fd_adi_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    with open(os.path.join(ROOT, "include", "fdadi.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|void)\s+(fdadi_\w+)\s*\(", src, re.M)))


def test_header_declares_entry_points():
    names = declared()
    assert "fdadi_heston_run" in names and "fdadi_tri_solve" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in declared():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, "binding missing for " + name


def test_version_and_error_text():
    lib = _lib.load()
    assert lib.fdadi_version() >= 10000
    buf = ctypes.create_string_buffer(64)
    lib.fdadi_last_error(buf, 64)


def test_argument_errors_without_gpu():
    """Shape validation happens on the host before any launch."""
    lib = _lib.load()
    t = _lib.Tri(100, 7, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0)
    rc = lib.fdadi_tri_apply(ctypes.byref(t), None, None, 10, 10, None)
    assert rc == 1
    assert "divide" in _lib.last_error()
    with pytest.raises(ValueError):
        _lib.check(rc, "fdadi_tri_apply")
    b = _lib.HestonBatch(0, 2, 10, 0, 0.5, 0.5, 0, 0, None, None, None, None, None, None, None)
    assert lib.fdadi_heston_workspace_bytes(ctypes.byref(b)) == -1
