"""The C ABI library loads (without a GPU) and exports every entry point include/gbdyn.h
declares; the ctypes layer binds each of them."""

import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared():
    text = (ROOT / "include" / "gbdyn.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared()
    assert "gb_create" in names and "gb_advect_x" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(built):
    import ctypes

    from pydyn_gb300.build import LIBGBDYN

    lib = ctypes.CDLL(str(LIBGBDYN))
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert missing == []


def test_ctypes_binds_every_declared_symbol(built):
    from pydyn_gb300 import _native

    assert sorted(set(declared()) - set(_native.SIGNATURES)) == []
    _native.lib()  # loads and sets every prototype


def test_no_cpu_fallback_without_library(tmp_path, monkeypatch):
    """The product path raises when its library is missing; it has no CPU route."""
    import pytest

    from pydyn_gb300 import _native

    monkeypatch.setattr(_native, "LIBGBDYN", tmp_path / "absent.so")
    monkeypatch.setattr(_native, "_LIB", [])
    with pytest.raises(RuntimeError, match="not built"):
        _native.lib()
