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


def _prototypes():
    """name -> list of parameter declarations, from the header."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for m in re.finditer(
            r"\b(?:int\s+|const char\s*\*\s*)(tg_\w+)\s*\(([^)]*)\)\s*;", src):
        params = [p.strip() for p in m.group(2).split(",") if p.strip()]
        if params == ["void"]:
            params = []
        out[m.group(1)] = params
    return out


def _kind(decl):
    """'ptr', 'double' or 'int' for one C parameter declaration."""
    if "*" in decl or "[" in decl:
        return "ptr"
    if re.match(r"(const\s+)?double\b", decl):
        return "double"
    return "int"


def test_ctypes_signatures_match_header():
    """Every binding has the header's number of parameters and, parameter
    by parameter, the same kind (pointer, double or integer)."""
    import ctypes as C
    from tacs_gb300 import _lib
    protos = _prototypes()
    assert len(protos) >= 30
    bad = []
    for name, _res, args in _lib.SIGNATURES:
        if name not in protos:
            bad.append((name, "not in header"))
            continue
        params = protos[name]
        if len(params) != len(args):
            bad.append((name, f"{len(args)} bound, {len(params)} declared"))
            continue
        for i, (decl, a) in enumerate(zip(params, args)):
            want = _kind(decl)
            if a in (C.c_void_p, C.c_char_p) or \
                    getattr(a, "_type_", None) is not None and \
                    isinstance(a, type) and issubclass(a, C._Pointer):
                got = "ptr"
            elif a is C.c_double:
                got = "double"
            else:
                got = "int"
            if got != want:
                bad.append((name, i, decl, got))
    assert not bad, bad
