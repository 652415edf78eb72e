"""CPU tests of the C-ABI library: it builds, loads and exports every entry
point declared in include/tsph.h (no compute calls: no GPU here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HEADER = os.path.join(ROOT, "include", "tsph.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(tsph_[a-z_0-9]+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("tsph_create", "tsph_grav_all", "tsph_smooth", "tsph_kick",
                 "tsph_drift", "tsph_get_gravity"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from gasoline_gb300 import build
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_error_strings():
    from gasoline_gb300 import build
    lib = ctypes.CDLL(build.build())
    lib.tsph_error_string.restype = ctypes.c_char_p
    assert lib.tsph_error_string(0) == b"ok"
    assert b"overflow" in lib.tsph_error_string(3)


def test_no_cpu_fallback_without_library(tmp_path, monkeypatch):
    import gasoline_gb300 as g
    monkeypatch.setattr(g, "LIBPATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(g, "_lib", None)
    with pytest.raises(RuntimeError):
        g.load()
