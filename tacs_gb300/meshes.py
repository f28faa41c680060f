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
understood by :mod:`tacs_gb300.assembler` and by the golden-vector tooling):

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
