"""The fixed-geometry plan (tacs_gb300/csrc/geo_plan.h), on the CPU.

* contribution lists: for every BCSR block slot (i, j), exactly the
  (element, a, b) pairs with conn[e][a] = i and conn[e][b] = j, in element
  order, nelem * npe^2 in all (brute force on plates, hex blocks and random
  connectivities);
* geometry classes: one class for a uniform structured mesh whose spacing
  is a power of two, a new class for each element that touches a moved
  node, one class per element for distorted elements, and the
  representative is the first element of its class;
* the row schedule: the longest row of each 32-row group.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "geo_plan_check.cpp")
INC = os.path.join(ROOT, "tacs_gb300", "csrc")


@pytest.fixture(scope="module")
def gp(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("gp") / "libgp.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", INC,
                    SRC, "-o", out], check=True)
    lib = C.CDLL(out)
    P = C.c_void_p
    lib.gp_contributions.argtypes = [C.c_int, C.c_int, C.c_int, P, C.c_int,
                                     P, P, P, P, P]
    lib.gp_classes.argtypes = [C.c_int, C.c_int, P, P, P, P]
    lib.gp_row_lengths.argtypes = [C.c_int, P, P]
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _meshes():
    from tacs_gb300 import meshes
    out = []
    p = meshes.plate(5, 3, 1.0, 0.75)
    out.append((p["nnodes"], 4, p["conn"]))
    h = meshes.hex_block(3, 2, 2, 1.5, 1.0, 1.0)
    out.append((h["nnodes"], 8, h["conn"]))
    rng = np.random.default_rng(5)
    for npe in (4, 8):
        nn, ne = 30, 25
        conn = np.concatenate([rng.choice(nn, npe, replace=False)
                               for _ in range(ne)]).astype(np.int32)
        out.append((nn, npe, conn))
    return out


def test_contribution_lists_match_brute_force(gp):
    for nn, npe, conn in _meshes():
        conn = np.ascontiguousarray(conn, np.int32)
        ne = len(conn) // npe
        cap = 64 * nn * nn + ne * npe * npe
        rowp = np.zeros(nn + 1, np.int32)
        cols, cptr, contrib = (np.zeros(cap, np.int32) for _ in range(3))
        nc = C.c_int(0)
        nnz = gp.gp_contributions(nn, npe, ne, _p(conn), cap, _p(rowp),
                                  _p(cols), _p(cptr), _p(contrib),
                                  C.byref(nc))
        assert nnz > 0 and nc.value == ne * npe * npe
        ce = conn.reshape(ne, npe)
        expect = {}
        for e in range(ne):
            for a in range(npe):
                for b in range(npe):
                    expect.setdefault((ce[e, a], ce[e, b]), []).append(
                        (e << 6) | (npe * a + b))
        got = {}
        for i in range(nn):
            for s in range(rowp[i], rowp[i + 1]):
                lst = list(contrib[cptr[s]:cptr[s + 1]])
                if lst:
                    got[(i, cols[s])] = lst
        assert got == expect  # same pairs, element order within each slot


def test_geometry_classes(gp):
    from tacs_gb300 import meshes
    p = meshes.plate(8, 4, 2.0, 1.0)  # spacing 1/4: exact differences
    conn = np.ascontiguousarray(p["conn"], np.int32)
    x = np.ascontiguousarray(p["xpts"], np.float64)
    ne = p["nelem"]
    cls, reps = np.zeros(ne, np.int32), np.zeros(ne, np.int32)
    assert gp.gp_classes(ne, 4, _p(conn), _p(x), _p(cls), _p(reps)) == 1
    assert cls.max() == 0 and reps[0] == 0
    # move one interior node: the four elements around it change class
    node = 2 + 9 * 2
    x2 = x.copy()
    x2[3 * node + 2] += 1e-3
    n2 = gp.gp_classes(ne, 4, _p(conn), _p(x2), _p(cls), _p(reps))
    touched = np.nonzero((conn.reshape(-1, 4) == node).any(axis=1))[0]
    assert n2 == 1 + len(touched)
    assert len(set(cls[touched])) == len(touched)
    assert np.all(np.delete(cls, touched) == 0)
    for c in range(n2):  # the representative is the first of its class
        assert reps[c] == np.nonzero(cls == c)[0][0]
    # distorted elements: one class each
    r = meshes.random_hex_elements(12, seed=3)
    rc = np.ascontiguousarray(r["conn"], np.int32)
    rx = np.ascontiguousarray(r["xpts"], np.float64)
    cls = np.zeros(12, np.int32)
    assert gp.gp_classes(12, 8, _p(rc), _p(rx), _p(cls), _p(reps)) == 12


def test_row_schedule(gp):
    rng = np.random.default_rng(2)
    lens = rng.integers(1, 28, 100)
    rowp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    kmax = np.zeros(4, np.int32)
    gp.gp_row_lengths(100, _p(rowp), _p(kmax))
    for w in range(4):
        assert kmax[w] == lens[32 * w:32 * w + 32].max()
