"""Synthetic structured meshes for the MITC4-shell and hex8 workloads.

The node and element orderings follow the reference's own generated meshes:

* shell plates: node ``i + (nx+1)*j``, element connectivity
  ``(i,j), (i+1,j), (i,j+1), (i+1,j+1)`` (TACS examples/plate/plate.cpp:33-50
  with order 2; the tensor-product node order of TACSShellQuadBasis<2>);
* hex blocks: tensor-product order ``(i,j,k), (i+1,j,k), (i,j+1,k),
  (i+1,j+1,k), (i,j,k+1), ...`` (tests/integration_tests/
  test_elast_linhexa_element_3d.py:88-106; TACSLinearHexaBasis node order,
  src/elements/basis/TACSHexaBasis.cpp:137-146).

Every builder returns a plain dict of numpy arrays (the "problem" record
understood by :mod:`tacs_gb300.problem` and by the golden-vector tooling):

``elem_type`` 0 = MITC4 shell (6 dof/node), 1 = hex8 (3 dof/node);
``xpts`` (nnodes*3 f64), ``conn`` (nelem*npe i32), ``thick`` (nelem f64),
``dvnum`` (nelem i32), ``mat`` (rho, E, nu, ys), ``bc_nodes``/``bc_masks``,
``pres_elems``/``pres_vals`` (4 nodal pressures per loaded shell element),
``trac_elems``/``trac_faces``/``trac_vals`` (hex face tractions),
``force`` (nodal force vector, R = K u - f).
"""
from __future__ import annotations

import numpy as np

SHELL, HEX = 0, 1


def _base(elem_type, xpts, conn, thick, dvnum, mat):
    nn = xpts.shape[0]
    vpn = 6 if elem_type == SHELL else 3
    return {
        "elem_type": int(elem_type),
        "nnodes": int(nn),
        "nelem": int(len(thick)),
        "xpts": np.ascontiguousarray(xpts, dtype=np.float64).reshape(-1),
        "conn": np.ascontiguousarray(conn, dtype=np.int32).reshape(-1),
        "thick": np.ascontiguousarray(thick, dtype=np.float64),
        "dvnum": np.ascontiguousarray(dvnum, dtype=np.int32),
        "mat": np.asarray(mat, dtype=np.float64),
        "transform": 0,
        "ref_axis": np.array([1.0, 0.0, 0.0]),
        "bc_nodes": np.zeros(0, np.int32),
        "bc_masks": np.zeros(0, np.int32),
        "pres_elems": np.zeros(0, np.int32),
        "pres_vals": np.zeros(0),
        "trac_elems": np.zeros(0, np.int32),
        "trac_faces": np.zeros(0, np.int32),
        "trac_vals": np.zeros(0),
        "force": np.zeros(nn * vpn),
        "ks_weight": 100.0,
    }


def plate(nx, ny, Lx=1.0, Ly=1.0, t=0.01, E=70e9, nu=0.3, rho=2700.0, ys=2.7e8,
          zfun=None, thick=None):
    """Flat (or z-perturbed) rectangular MITC4 plate, one DV per element."""
    xs = np.linspace(0.0, Lx, nx + 1)
    ys_ = np.linspace(0.0, Ly, ny + 1)
    X, Y = np.meshgrid(xs, ys_, indexing="xy")  # [j, i]
    Z = np.zeros_like(X) if zfun is None else zfun(X, Y)
    xpts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    n0 = (i + (nx + 1) * j).ravel()
    conn = np.stack([n0, n0 + 1, n0 + nx + 1, n0 + nx + 2], axis=1)
    ne = nx * ny
    th = np.full(ne, t) if thick is None else np.asarray(thick, np.float64)
    p = _base(SHELL, xpts, conn, th, np.arange(ne), (rho, E, nu, ys))
    p["nx"], p["ny"] = nx, ny
    return p


def plate_edges(nx, ny):
    """Node ids on the boundary of an (nx x ny)-element plate."""
    ids = np.arange((nx + 1) * (ny + 1)).reshape(ny + 1, nx + 1)
    return np.unique(np.concatenate([ids[0], ids[-1], ids[:, 0], ids[:, -1]]))


def cylinder(nc, nz, R=1.0, L=3.0, t=0.005, E=70e9, nu=0.3, rho=2700.0,
             ys=2.7e8):
    """Cylindrical MITC4 shell, periodic in the circumferential direction.

    Node ``i + nc*j`` sits at angle 2*pi*i/nc and height L*j/nz; element
    (i, j) connects (i,j), (i+1,j), (i,j+1), (i+1,j+1) with i+1 wrapped.
    """
    th = 2.0 * np.pi * np.arange(nc) / nc
    zz = np.linspace(0.0, L, nz + 1)
    T, Zg = np.meshgrid(th, zz, indexing="xy")
    xpts = np.stack([R * np.cos(T).ravel(), R * np.sin(T).ravel(), Zg.ravel()],
                    axis=1)
    i, j = np.meshgrid(np.arange(nc), np.arange(nz), indexing="xy")
    i, j = i.ravel(), j.ravel()
    ip = (i + 1) % nc
    conn = np.stack([i + nc * j, ip + nc * j, i + nc * (j + 1),
                     ip + nc * (j + 1)], axis=1)
    ne = nc * nz
    p = _base(SHELL, xpts, conn, np.full(ne, t), np.arange(ne),
              (rho, E, nu, ys))
    p["nc"], p["nz"] = nc, nz
    return p


def hex_block(nx, ny, nz, Lx=2.0, Ly=2.0, Lz=1.0, E=70e9, nu=0.3, rho=2700.0,
              ys=2.7e8, thick=None, node_order="xyz"):
    """Structured hex8 block.

    node_order "xyz": node id = i + (nx+1)*(j + (ny+1)*k) (x fastest);
    node_order "ijk": node id = (i*(ny+1) + j)*(nz+1) + k (the ordering of the
    reference's cube test).
    """
    xs = np.linspace(0.0, Lx, nx + 1)
    ys_ = np.linspace(0.0, Ly, ny + 1)
    zs = np.linspace(0.0, Lz, nz + 1)
    I, J, K = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1),
                          np.arange(nz + 1), indexing="ij")
    if node_order == "xyz":
        nid = lambda a, b, c: a + (nx + 1) * (b + (ny + 1) * c)  # noqa: E731
    else:
        nid = lambda a, b, c: (a * (ny + 1) + b) * (nz + 1) + c  # noqa: E731
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    xpts = np.zeros((nn, 3))
    ids = nid(I, J, K).ravel()
    xpts[ids, 0] = xs[I.ravel()]
    xpts[ids, 1] = ys_[J.ravel()]
    xpts[ids, 2] = zs[K.ravel()]
    if node_order == "xyz":
        ei, ej, ek = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz),
                                 indexing="ij")
        order = np.lexsort((ei.ravel(), ej.ravel(), ek.ravel()))
    else:
        ei, ej, ek = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz),
                                 indexing="ij")
        order = np.arange(nx * ny * nz)
    ei, ej, ek = ei.ravel()[order], ej.ravel()[order], ek.ravel()[order]
    conn = np.stack([nid(ei, ej, ek), nid(ei + 1, ej, ek), nid(ei, ej + 1, ek),
                     nid(ei + 1, ej + 1, ek), nid(ei, ej, ek + 1),
                     nid(ei + 1, ej, ek + 1), nid(ei, ej + 1, ek + 1),
                     nid(ei + 1, ej + 1, ek + 1)], axis=1)
    ne = nx * ny * nz
    th = np.ones(ne) if thick is None else np.asarray(thick, np.float64)
    p = _base(HEX, xpts, conn, th, np.arange(ne), (rho, E, nu, ys))
    p["nx"], p["ny"], p["nz"] = nx, ny, nz
    p["elem_ijk"] = np.stack([ei, ej, ek], axis=1)
    return p


def random_shell_elements(n, seed=0, curved=True):
    """n disconnected, randomly shaped (and warped) MITC4 elements."""
    rng = np.random.default_rng(seed)
    xpts = []
    for _ in range(n):
        base = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0],
                         [1.0, 1.0, 0.0]])
        base[:, :2] += 0.15 * rng.standard_normal((4, 2))
        if curved:
            base[:, 2] += 0.2 * rng.standard_normal(4)
        Q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        xpts.append(base @ Q.T * (0.5 + rng.random()))
    xpts = np.concatenate(xpts)
    conn = np.arange(4 * n).reshape(n, 4)
    th = 0.005 + 0.02 * rng.random(n)
    return _base(SHELL, xpts, conn, th, np.arange(n), (2700.0, 70e9, 0.3, 2.7e8))


def random_hex_elements(n, seed=0):
    """n disconnected, randomly distorted hex8 elements."""
    rng = np.random.default_rng(seed)
    ref = np.array([[x, y, z] for z in (0, 1) for y in (0, 1) for x in (0, 1)],
                   dtype=np.float64)
    xpts = []
    for _ in range(n):
        X = ref + 0.12 * rng.standard_normal((8, 3))
        Q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        if np.linalg.det(Q) < 0:
            Q[:, 0] *= -1
        xpts.append(X @ Q.T * (0.5 + rng.random()))
    xpts = np.concatenate(xpts)
    conn = np.arange(8 * n).reshape(n, 8)
    th = 0.1 + 0.9 * rng.random(n)
    return _base(HEX, xpts, conn, th, np.arange(n), (2700.0, 70e9, 0.3, 2.7e8))


def concat(probs):
    """Independent meshes of one element type batched into one problem.

    Nodes and elements are numbered mesh after mesh, so mesh g owns the
    contiguous ranges ``seg_node_ptr[g]:seg_node_ptr[g+1]`` and
    ``seg_elem_ptr[g]:seg_elem_ptr[g+1]`` and the Jacobian is block
    diagonal.  Material constants are those of the first mesh.
    """
    et = probs[0]["elem_type"]
    vpn = 6 if et == SHELL else 3
    npe = 4 if et == SHELL else 8
    node_ptr = np.cumsum([0] + [p["nnodes"] for p in probs])
    elem_ptr = np.cumsum([0] + [p["nelem"] for p in probs])
    cat = lambda k, dt: np.concatenate(  # noqa: E731
        [np.asarray(p[k], dt).ravel() for p in probs])
    conn = np.concatenate([np.asarray(p["conn"]).reshape(-1, npe) + node_ptr[g]
                           for g, p in enumerate(probs)])
    out = _base(et, cat("xpts", np.float64).reshape(-1, 3), conn,
                cat("thick", np.float64),
                np.concatenate([np.asarray(p["dvnum"]) + elem_ptr[g]
                                for g, p in enumerate(probs)]),
                probs[0]["mat"])
    out["bc_nodes"] = np.concatenate(
        [np.asarray(p["bc_nodes"], np.int64) + node_ptr[g]
         for g, p in enumerate(probs)]).astype(np.int32)
    out["bc_masks"] = cat("bc_masks", np.int32)
    out["pres_elems"] = np.concatenate(
        [np.asarray(p["pres_elems"], np.int64) + elem_ptr[g]
         for g, p in enumerate(probs)]).astype(np.int32)
    out["pres_vals"] = cat("pres_vals", np.float64)
    out["force"] = cat("force", np.float64)
    out["seg_node_ptr"] = node_ptr.astype(np.int32)
    out["seg_elem_ptr"] = elem_ptr.astype(np.int32)
    assert len(out["force"]) == vpn * out["nnodes"]
    return out


def clamped_plate(n, L=1.0, thick=None, pressure=1e3, t=0.01):
    """n x n MITC4 plate on an L x L square, all edges clamped (mask 0x3F),
    uniform pressure on every element."""
    p = plate(n, n, Lx=L, Ly=L, t=t, thick=thick)
    edges = plate_edges(n, n)
    p["bc_nodes"] = edges.astype(np.int32)
    p["bc_masks"] = np.full(len(edges), 0x3F, np.int32)
    p["pres_elems"] = np.arange(n * n, dtype=np.int32)
    p["pres_vals"] = np.full(4 * n * n, float(pressure))
    return p


def plate_c2(n=512, L=2.0, seed=2):
    """Simply supported MITC4 plate: n x n elements on an L x L square,
    per-element thickness ~ U[0.005, 0.02] (numpy default_rng(seed)),
    E 70e9, nu 0.3, rho 2700, ys 2.7e8; edge nodes hold u, v, w (mask 0x07);
    nodal pressure p(x, y) = 1e3 (1 + 0.5 sin(pi x) sin(pi y)) with x, y in
    metres on every element."""
    rng = np.random.default_rng(seed)
    p = plate(n, n, L, L, t=0.01, E=70e9, nu=0.3, rho=2700.0, ys=2.7e8,
              thick=rng.uniform(0.005, 0.02, n * n))
    e = plate_edges(n, n).astype(np.int32)
    p["bc_nodes"], p["bc_masks"] = e, np.full(len(e), 0x07, np.int32)
    xyz = p["xpts"].reshape(-1, 3)
    pn = 1e3 * (1.0 + 0.5 * np.sin(np.pi * xyz[:, 0])
                * np.sin(np.pi * xyz[:, 1]))
    conn = p["conn"].reshape(-1, 4)
    p["pres_elems"] = np.arange(n * n, dtype=np.int32)
    p["pres_vals"] = pn[conn].ravel()
    return p


def batch_plates(count=48, seed=4, nmin=16, nmax=256, L=1.0, tmin=0.004,
                 tmax=0.02, pressure=1e3, point_load=1e3):
    """Independent clamped MITC4 plates of seeded uneven sizes in one problem.

    Plate g is N_g x N_g elements on an L x L square with
    N_g = round(nmin * (nmax / nmin)**u_g), u_g ~ U[0, 1]; per-element
    thickness ~ U[tmin, tmax]; all edges clamped; uniform pressure on every
    element.  Four load cases per plate: the pressure, and three point loads
    of point_load in the w direction at seeded distinct interior nodes (one
    per case).  Draws, in order, from numpy.random.default_rng(seed): the
    count u's, then per plate its thicknesses and its three load nodes.
    Returns the concatenated problem with ``plate_n`` and ``point_nodes``
    (count x 3 global node ids) added.
    """
    rng = np.random.default_rng(seed)
    u = rng.random(count)
    sizes = np.rint(nmin * (nmax / nmin) ** u).astype(int)
    probs, pts = [], []
    for n in sizes:
        th = rng.uniform(tmin, tmax, n * n)
        p = clamped_plate(int(n), L=L, thick=th, pressure=pressure)
        ids = np.arange((n + 1) ** 2).reshape(n + 1, n + 1)
        interior = ids[1:-1, 1:-1].ravel()
        pts.append(rng.choice(interior, 3, replace=False))
        probs.append(p)
    out = concat(probs)
    out["plate_n"] = sizes
    out["point_nodes"] = np.stack(
        [pts[g] + out["seg_node_ptr"][g] for g in range(count)]).astype(
            np.int64)
    out["point_load"] = float(point_load)
    return out


def hex_c3(nx=128, ny=128, nz=64, seed=3, traction=-1e4, half=0.1):
    """Topology-style solid block: nx x ny x nz hex8 on a 2 x 2 x 1 m block,
    per-element density rho ~ U[0.1, 1] (numpy default_rng(seed)) with SIMP
    stiffness E rho^3 carried as the element scale t = rho^3; the x = 0 face
    clamped; a traction (0, 0, traction) Pa on the x = 2 face of the elements
    whose face centroid lies within |y - 1| <= half, |z - 0.5| <= half.
    ``rho`` holds the densities."""
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.1, 1.0, nx * ny * nz)
    p = hex_block(nx, ny, nz, 2.0, 2.0, 1.0, thick=rho ** 3)
    xyz = p["xpts"].reshape(-1, 3)
    bcn = np.nonzero(xyz[:, 0] == 0.0)[0].astype(np.int32)
    p["bc_nodes"], p["bc_masks"] = bcn, np.full(len(bcn), 0x7, np.int32)
    ijk = p["elem_ijk"]
    yc = (ijk[:, 1] + 0.5) * 2.0 / ny
    zc = (ijk[:, 2] + 0.5) * 1.0 / nz
    te = np.nonzero((ijk[:, 0] == nx - 1) & (np.abs(yc - 1.0) <= half)
                    & (np.abs(zc - 0.5) <= half))[0]
    p["trac_elems"] = te.astype(np.int32)
    p["trac_faces"] = np.full(len(te), 1, np.int32)
    p["trac_vals"] = np.tile([0.0, 0.0, float(traction)], len(te))
    p["rho"] = rho
    return p


def cylinder_c5(nc=384, nz=256, R=1.0, L=3.0, t=0.005, axial=1e5,
                pressure=5e3):
    """Cylindrical shell, z = 0 ring clamped; at z = L an axial compressive
    edge load of ``axial`` N/m as nodal forces -axial * 2 pi R / nc (z
    direction) per ring node; internal pressure on every element (the
    element normal of this connectivity points outward, +pressure pushes
    outward).  One design variable (thickness) per element."""
    p = cylinder(nc, nz, R=R, L=L, t=t)
    ring0 = np.arange(nc)
    p["bc_nodes"] = ring0.astype(np.int32)
    p["bc_masks"] = np.full(nc, 0x3F, np.int32)
    ne = nc * nz
    p["pres_elems"] = np.arange(ne, dtype=np.int32)
    p["pres_vals"] = np.full(4 * ne, float(pressure))
    f = np.zeros((p["nnodes"], 6))
    f[nc * nz + np.arange(nc), 2] = -axial * 2.0 * np.pi * R / nc
    p["force"] = f.ravel()
    return p
