"""Host-side mesh graph work and argument checks, on the CPU.

* The element colouring (no two elements of one colour share a node) and
  the node colouring of the colour-reordered ILU(0) (no two neighbours share
  a colour) of tacs_gb300/csrc/mesh_graph.h: valid beyond 64 colours (a
  pole where 96 quads meet; a nearly complete node graph), and identical
  to the plain greedy rule (smallest free colour, in order) on structured
  and random meshes.
* The C ABI's argument validation (tg_assembler_create and the host
  setters, which do no device work): negative status codes with a message,
  and no partial update before an error is found.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "mesh_graph_check.cpp")
INC = os.path.join(ROOT, "tacs_gb300", "csrc")


@pytest.fixture(scope="module")
def mg(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("mg") / "libmg.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", INC,
                    SRC, "-o", out], check=True)
    lib = C.CDLL(out)
    P = C.c_void_p
    lib.mg_color_elements.argtypes = [C.c_int, C.c_int, C.c_int, P, P]
    lib.mg_pattern_and_node_colors.argtypes = [C.c_int, C.c_int, C.c_int, P,
                                               C.c_int, P, P, P, P]
    lib.mg_first_writers.argtypes = [C.c_int, C.c_int, P, P]
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _fan(n):
    """n quads around a pole (node 0): rim nodes 1..n, outer nodes
    n+1..2n; quad k = (0, rim k, outer k, rim k+1)."""
    conn = []
    for k in range(n):
        r0, r1 = 1 + k, 1 + (k + 1) % n
        conn += [0, r0, n + 1 + k, r1]
    return 2 * n + 1, 4, np.array(conn, np.int32)


def _quad_plate(nx, ny):
    conn = []
    for j in range(ny):
        for i in range(nx):
            a = i + (nx + 1) * j
            conn += [a, a + 1, a + nx + 1, a + nx + 2]
    return (nx + 1) * (ny + 1), 4, np.array(conn, np.int32)


def _hex_block(nx, ny, nz):
    def nd(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)
    conn = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                conn += [nd(i + a, j + b, k + c) for c in (0, 1)
                         for b in (0, 1) for a in (0, 1)]
    return (nx + 1) * (ny + 1) * (nz + 1), 8, np.array(conn, np.int32)


def _random_mesh(seed):
    rng = np.random.default_rng(seed)
    nn = 60
    conn = np.concatenate([rng.choice(nn, 4, replace=False)
                           for _ in range(150)]).astype(np.int32)
    return nn, 4, conn


def _greedy_elements(nn, npe, conn):
    """The plain greedy rule, in Python."""
    ne = len(conn) // npe
    used = [set() for _ in range(nn)]
    col = np.zeros(ne, int)
    for e in range(ne):
        nd = conn[npe * e:npe * (e + 1)]
        taken = set().union(*(used[v] for v in nd))
        c = 0
        while c in taken:
            c += 1
        col[e] = c
        for v in nd:
            used[v].add(c)
    return col


def _colors(mg, nn, npe, conn):
    ne = len(conn) // npe
    col = np.zeros(ne, np.int32)
    ncol = mg.mg_color_elements(nn, npe, ne, _p(conn), _p(col))
    rowp = np.zeros(nn + 1, np.int32)
    cap = nn * nn
    cols = np.zeros(cap, np.int32)
    ncol_nodes = C.c_int(0)
    ncolor = np.zeros(nn, np.int32)
    nnz = mg.mg_pattern_and_node_colors(nn, npe, ne, _p(conn), cap, _p(rowp),
                                        _p(cols), _p(ncolor),
                                        C.byref(ncol_nodes))
    assert nnz <= cap
    return col, ncol, rowp, cols[:nnz], ncolor, ncol_nodes.value


def _check_valid(nn, npe, conn, col, rowp, cols, ncolor):
    for c in np.unique(col):
        seen = {}
        for e in np.nonzero(col == c)[0]:
            for v in set(conn[npe * e:npe * (e + 1)].tolist()):
                assert v not in seen, (c, e, seen.get(v))
                seen[v] = e
    for i in range(nn):
        nb = cols[rowp[i]:rowp[i + 1]]
        assert i in nb  # the diagonal
        assert np.all(np.diff(nb) > 0)  # sorted, unique
        for j in nb:
            if j != i:
                assert ncolor[i] != ncolor[j], (i, j)


def test_pole_needs_more_than_64_colours(mg):
    """96 quads meet at a pole: 96 element colours."""
    nn, npe, conn = _fan(96)
    col, ncol, rowp, cols, ncolor, nncol = _colors(mg, nn, npe, conn)
    assert ncol == 96  # every quad touches the pole
    _check_valid(nn, npe, conn, col, rowp, cols, ncolor)


def test_dense_node_graph_needs_more_than_64_colours(mg):
    """100 nodes under 6,000 random quads: the node graph is nearly
    complete, so its colouring needs more than 64 colours."""
    rng = np.random.default_rng(8)
    nn = 100
    conn = np.concatenate([rng.choice(nn, 4, replace=False)
                           for _ in range(6000)]).astype(np.int32)
    col, ncol, rowp, cols, ncolor, nncol = _colors(mg, nn, 4, conn)
    assert nncol > 64 and ncol > 64
    _check_valid(nn, 4, conn, col, rowp, cols, ncolor)


@pytest.mark.parametrize("mesh", ["plate", "hex", "random", "fan"])
def test_colouring_is_the_greedy_rule(mg, mesh):
    nn, npe, conn = {"plate": lambda: _quad_plate(9, 7),
                     "hex": lambda: _hex_block(4, 3, 3),
                     "random": lambda: _random_mesh(3),
                     "fan": lambda: _fan(70)}[mesh]()
    col, ncol, rowp, cols, ncolor, _ = _colors(mg, nn, npe, conn)
    assert np.array_equal(col, _greedy_elements(nn, npe, conn))
    assert ncol == col.max() + 1
    _check_valid(nn, npe, conn, col, rowp, cols, ncolor)
    if mesh == "plate":
        assert ncol == 4
    if mesh == "hex":
        assert ncol == 8


# --------------------------------------------------- C ABI argument checks
@pytest.fixture(scope="module")
def L():
    from tacs_gb300 import _lib
    try:
        return _lib.lib()
    except _lib.TacsGpuError as e:
        pytest.skip(str(e))


def _create(L, elem_type, nn, ne, conn, transform=0, axis=None):
    h = C.c_void_p()
    rc = L.tg_assembler_create(elem_type, nn, ne,
                               _p(conn) if conn is not None else None,
                               2700.0, 70e9, 0.3, 2.7e8, transform,
                               _p(axis) if axis is not None else None,
                               C.byref(h))
    return rc, h


def test_create_rejects_bad_arguments(L):
    from tacs_gb300 import _lib
    nn, npe, conn = _quad_plate(2, 2)
    cases = [
        (7, nn, 4, conn, 0, None, "unknown element type"),
        (_lib.ELEM_MITC4, -1, 4, conn, 0, None, "bad sizes"),
        (_lib.ELEM_MITC4, nn, 4, None, 0, None, "bad sizes"),
        (_lib.ELEM_MITC4, nn - 1, 4, conn, 0, None, "out of range"),
        (_lib.ELEM_MITC4, nn, 4, conn, 1, None, "reference axis"),
    ]
    for et, n, ne, c, tr, ax, msg in cases:
        rc, h = _create(L, et, n, ne, c, tr, ax)
        assert rc == _lib.ERR_ARG and not h.value
        assert msg in L.tg_last_error().decode()
    # an empty mesh is a valid (if useless) assembler
    rc, h = _create(L, _lib.ELEM_MITC4, 0, 0, None)
    assert rc == 0 and h.value
    L.tg_assembler_decref(h)


def test_setters_validate_before_changing_state(L):
    from tacs_gb300 import _lib
    nn, npe, conn = _quad_plate(2, 2)
    rc, h = _create(L, _lib.ELEM_MITC4, nn, 4, conn)
    assert rc == 0
    try:
        bad_nodes = np.array([0, nn], np.int32)
        masks = np.array([7, 7], np.int32)
        assert L.tg_assembler_add_bcs(h, 2, _p(bad_nodes), _p(masks)) == \
            _lib.ERR_ARG
        assert "out of range" in L.tg_last_error().decode()
        ok_nodes = np.array([0, 1], np.int32)
        assert L.tg_assembler_add_bcs(h, 2, _p(ok_nodes), _p(masks)) == 0
        el = np.array([0, 9], np.int32)
        vals = np.ones(8)
        assert L.tg_assembler_set_pressure(h, 2, _p(el), _p(vals)) == \
            _lib.ERR_ARG
        el = np.array([0, 3], np.int32)
        assert L.tg_assembler_set_pressure(h, 2, _p(el), _p(vals)) == 0
        faces = np.array([0, 1], np.int32)
        assert L.tg_assembler_set_traction(h, 2, _p(el), _p(faces),
                                           _p(np.ones(6))) == _lib.ERR_ARG
        assert "hex" in L.tg_last_error().decode()
        assert L.tg_set_xpt_mode(h, 2) == _lib.ERR_ARG
        assert L.tg_set_xpt_mode(h, _lib.XPT_REVERSE) == 0
        sizes = [C.c_int() for _ in range(5)]
        assert L.tg_assembler_get_sizes(h, *[C.byref(s) for s in sizes]) == 0
        assert [s.value for s in sizes[:3]] == [6, nn, 4]
    finally:
        L.tg_assembler_decref(h)


@pytest.mark.parametrize("mesh", ["plate", "fan", "random"])
def test_first_writers(mg, mesh):
    """The shell assembly's first-writer masks (mesh_graph.h first_writers):
    every pattern block (node pair of an element) and every node has
    exactly one first writer, and it is the element of the lowest colour
    among those that touch it (colours are launched in order, and elements
    of one colour share no node).  A node in no element yields no masks."""
    nn, npe, conn = {"plate": lambda: _quad_plate(9, 7),
                     "fan": lambda: _fan(96),
                     "random": lambda: _random_mesh(3)}[mesh]()
    if npe != 4:
        pytest.skip("4-node meshes only")
    ne = len(conn) // 4
    col = np.zeros(ne, np.int32)
    mg.mg_color_elements(nn, 4, ne, _p(conn), _p(col))
    first = np.zeros(ne, np.uint32)
    assert mg.mg_first_writers(nn, ne, _p(conn), _p(first)) == 1
    c4 = conn.reshape(-1, 4)
    blk, nod = {}, {}
    for e in range(ne):
        for a in range(4):
            nod.setdefault(int(c4[e, a]), []).append(e)
            for b in range(4):
                blk.setdefault((int(c4[e, a]), int(c4[e, b])), []).append(
                    (e, a, b))
    for key, users in blk.items():
        owners = [(e, a, b) for e, a, b in users
                  if (int(first[e]) >> (4 * a + b)) & 1]
        assert len(owners) == 1
        assert col[owners[0][0]] == min(col[e] for e, _, _ in users)
    for node, users in nod.items():
        owners = [e for e in users
                  if any((int(first[e]) >> (16 + a)) & 1
                         for a in range(4) if c4[e, a] == node)]
        assert len(owners) == 1
        assert col[owners[0]] == min(col[e] for e in users)
    # a node in no element: no masks (the assembly falls back to zero fill)
    conn2 = np.concatenate([conn, np.zeros(0, np.int32)])
    assert mg.mg_first_writers(nn + 1, ne, _p(conn2), _p(first)) == 0
