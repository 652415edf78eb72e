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


STRUCTS = {   # C typedef in include/tsph.h -> ctypes class in gasoline_gb300
    "tsph_grav_params": "GravParams",
    "tsph_grav_out": "GravOut",
    "tsph_sph_params": "SphParams",
    "tsph_smooth_out": "SmoothOut",
    "tsph_tuning": "Tuning",
    "tsph_step_params": "StepParams",
    "tsph_step_out": "StepOut",
    "tsph_render_params": "RenderParams",
    "tsph_tipsy_header": "TipsyHeader",
    "tsph_store_layout": "StoreLayout",
}


def test_struct_layouts_match_the_header(tmp_path):
    """Every parameter and output struct of the binding has the C layout:
    the size and every field's offset, as gcc lays out include/tsph.h."""
    import shutil
    import subprocess
    import gasoline_gb300 as g
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "tsph.h"', 'int main(void) {']
    for cname, pyname in STRUCTS.items():
        cls = getattr(g, pyname)
        lines.append(f'printf("{pyname} size %zu\\n", sizeof({cname}));')
        for field in cls._fields_:
            f = field[0]
            lines.append(f'printf("{pyname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split("\n")
    for line in filter(None, out):
        pyname, what, val = line.split()
        cls = getattr(g, pyname)
        got = ctypes.sizeof(cls) if what == "size" else getattr(cls, what).offset
        assert got == int(val), (pyname, what, got, int(val))
