"""The C-ABI library builds, loads (no GPU needed) and exports every entry
point declared in include/tacs_gb300.h; the ctypes binding covers them."""
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "tacs_gb300.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tg_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared()
    assert "tg_assemble_jacobian" in names and "tg_ksm_solve" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    from tacs_gb300 import build as gb
    if not os.path.exists(gb.LIB):
        try:
            gb.build()
        except Exception as e:  # no toolkit: nothing to check here
            pytest.skip(f"cannot build the library here: {e}")
    out = subprocess.run(["nm", "-D", "--defined-only", gb.LIB],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s+(tg_\w+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing


def test_ctypes_binding_covers_header():
    from tacs_gb300 import _lib
    bound = set(_lib.exported_symbols())
    missing = [n for n in declared() if n not in bound]
    assert not missing, missing
    import ctypes
    ctypes.CDLL(_lib.LIB_PATH)  # loads without a GPU
