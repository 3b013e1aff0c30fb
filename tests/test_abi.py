"""The C-ABI library loads and exports every entry point include/reaxgpu.h
declares (no GPU needed: symbol resolution only)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


def declared():
    names = []
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"^[a-z][\w \*]*?\b(rg_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared()
    for need in ("rg_create", "rg_qeq", "rg_compute", "rg_run", "rg_nve_initial"):
        assert need in names


def test_library_exports_all_declared_symbols():
    from sw_reaxff_gb300 import build
    lib = build.build()
    L = ctypes.CDLL(lib)
    missing = [n for n in declared() if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_exports():
    from sw_reaxff_gb300.api import EXPORTED
    assert set(EXPORTED) <= set(declared())
