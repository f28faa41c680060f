"""Regenerate the golden fixtures in this directory from the reference TACS.

Each case is a seeded synthetic problem (tacs_gb300.meshes).  It is written
as a problem file, run through the reference library's own assembler,
solver and adjoint code by ``oracle/_ref/gen_golden`` (built from the
reference sources by ``oracle/ref/Makefile``), and the inputs plus every
reference output are stored together as ``<case>.npz``.

Run here (where the reference sources are present):

    make -C oracle/ref REF=<path to tacs>
    python tests/golden/make_golden.py

The node-coordinate sensitivities come from the reference's complex build
(``make -C oracle/ref REF=<path to tacs> cplx``), whose shell and load
elements form them by complex step and so exactly; they are added to the
stored fixtures with

    python tests/golden/make_golden.py --xpt [case ...]

and the ILU(1) / ILU(2) applies of the real build with ``--iluk``.

The fixtures are committed; the GPU machine never needs the reference.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tacs_gb300 import meshes  # noqa: E402

GEN = os.path.join(ROOT, "oracle", "_ref", "gen_golden")
GEN_CPLX = os.path.join(ROOT, "oracle", "_ref", "gen_golden_cplx")
XPT_KEYS = ("dfdX_test_comp", "dfdX_test_ks", "adjxpt_test", "grad_xpt_comp",
            "grad_xpt_ks")

INT_KEYS = {"elem_type", "nnodes", "nelem", "conn", "dvnum", "transform",
            "bc_nodes", "bc_masks", "pres_elems", "trac_elems", "trac_faces",
            "gmres_m", "gmres_restart"}


def write_tgarr(path, prob):
    with open(path, "wb") as fp:
        for k, v in prob.items():
            if k in INT_KEYS:
                a = np.ascontiguousarray(np.atleast_1d(v), dtype="<i4")
                dt = 1
            else:
                try:
                    a = np.ascontiguousarray(np.atleast_1d(v), dtype="<f8")
                except (TypeError, ValueError):
                    continue
                dt = 0
            name = k.encode()[:31].ljust(32, b"\0")
            fp.write(name)
            fp.write(np.int32(dt).tobytes())
            fp.write(np.int64(a.size).tobytes())
            fp.write(a.tobytes())


def read_tgarr(path):
    out = {}
    with open(path, "rb") as fp:
        while True:
            name = fp.read(32)
            if len(name) < 32:
                break
            dt = int(np.frombuffer(fp.read(4), "<i4")[0])
            n = int(np.frombuffer(fp.read(8), "<i8")[0])
            if dt == 0:
                a = np.frombuffer(fp.read(8 * n), "<f8").copy()
            else:
                a = np.frombuffer(fp.read(4 * n), "<i4").copy()
            out[name.rstrip(b"\0").decode()] = a
    return out


def run_reference(prob, gen=GEN):
    with tempfile.TemporaryDirectory() as td:
        pin, pout = os.path.join(td, "p.bin"), os.path.join(td, "o.bin")
        write_tgarr(pin, prob)
        subprocess.run([gen, pin, pout], check=True)
        return read_tgarr(pout)


def add_tests_vectors(p, seed, scale=1e-3):
    rng = np.random.default_rng(seed)
    vpn = 6 if p["elem_type"] == meshes.SHELL else 3
    n = p["nnodes"] * vpn
    p["u_test"] = scale * rng.standard_normal(n)
    p["psi_test"] = rng.standard_normal(n)
    p["x_test"] = rng.standard_normal(n)


def case_shell_rand():
    p = meshes.random_shell_elements(6, seed=11)
    # Clamp node 0 of every element so that each element block is solvable
    p["bc_nodes"] = np.arange(0, 24, 4, dtype=np.int32)
    p["bc_masks"] = np.full(6, 0x3F, np.int32)
    add_tests_vectors(p, 12)
    rng = np.random.default_rng(13)
    p["pres_elems"] = np.arange(6, dtype=np.int32)
    p["pres_vals"] = 1e3 * (1 + rng.random(24))
    p["force"] = 10.0 * rng.standard_normal(p["nnodes"] * 6)
    p["ks_weight"] = 100.0
    return p


def case_shell_rand_refaxis():
    p = case_shell_rand()
    p["transform"] = 1
    p["ref_axis"] = np.array([0.3, 1.0, -0.2])
    return p


def case_shell_beam():
    """tests/integration_tests/test_shell_beam_quad.py:12-160 (KS weight 10,
    Qx = 5e6 tip shear, t = 0.1 as one shared DV)."""
    nx, ny, Lx, Ly = 10, 10, 10.0, 1.0
    x = np.linspace(0, Lx, nx + 1)
    y = np.linspace(0, Ly, ny + 1)
    xyz = np.zeros((nx + 1, ny + 1, 3))
    xyz[:, :, 0], xyz[:, :, 1] = np.meshgrid(x, y, indexing="ij")
    ids = np.arange((nx + 1) * (ny + 1)).reshape(nx + 1, ny + 1)
    conn = []
    for i in range(nx):
        for j in range(ny):
            conn.append([ids[i, j], ids[i + 1, j], ids[i, j + 1],
                         ids[i + 1, j + 1]])
    ne = nx * ny
    p = meshes._base(meshes.SHELL, xyz.reshape(-1, 3), np.array(conn),
                     np.full(ne, 0.1), np.zeros(ne, np.int32),
                     (2570.0, 70e9, 0.3, 350e6))
    p["bc_nodes"] = ids[0, :].astype(np.int32)
    p["bc_masks"] = np.full(ny + 1, 0x3F, np.int32)
    f = np.zeros(((nx + 1) * (ny + 1), 6))
    f[ids[-1, :], 2] += 5e6 * Ly / ny
    p["force"] = f.ravel()
    p["ks_weight"] = 10.0
    p["gmres_m"], p["gmres_restart"], p["rtol"] = 100, 2, 1e-12
    p["func_refs"] = np.array([1.70202700e09, 8.47336988e01])
    return p


def case_hex_cube():
    """tests/integration_tests/test_elast_linhexa_element_3d.py:10-160
    (3x3x3 cube, 1e8 on every dof, x = 0 face clamped, KS weight 10)."""
    p = meshes.hex_block(3, 3, 3, 10.0, 10.0, 10.0, E=70e9, nu=0.3, rho=2570.0,
                         ys=350e6, node_order="ijk")
    p["dvnum"] = np.zeros(p["nelem"], np.int32)
    x = p["xpts"].reshape(-1, 3)[:, 0]
    bcn = np.nonzero(x == 0.0)[0].astype(np.int32)
    p["bc_nodes"], p["bc_masks"] = bcn, np.full(len(bcn), 0x7, np.int32)
    p["force"] = np.full(p["nnodes"] * 3, 1e8)
    p["ks_weight"] = 10.0
    p["gmres_m"], p["gmres_restart"], p["rtol"] = 100, 2, 1e-12
    p["func_refs"] = np.array([178995399.11928475, 1.1074017881777185])
    return p


def case_shell_plate8():
    rng = np.random.default_rng(21)
    p = meshes.plate(8, 8, 1.0, 1.0,
                     zfun=lambda X, Y: 0.05 * np.sin(2 * X + 1) * np.cos(Y),
                     thick=0.005 + 0.015 * rng.random(64))
    e = meshes.plate_edges(8, 8).astype(np.int32)
    p["bc_nodes"], p["bc_masks"] = e, np.full(len(e), 0x3F, np.int32)
    p["pres_elems"] = np.arange(64, dtype=np.int32)
    p["pres_vals"] = 1e3 * (1 + 0.5 * rng.random(256))
    add_tests_vectors(p, 22)
    p["gmres_m"], p["gmres_restart"], p["rtol"] = 200, 5, 1e-12
    return p


def case_shell_plate8_refaxis():
    p = case_shell_plate8()
    p["transform"], p["ref_axis"] = 1, np.array([1.0, 0.2, 0.0])
    p["bc_masks"] = np.full(len(p["bc_nodes"]), 0x07, np.int32)
    return p


def case_shell_c1():
    """The 32x32 clamped flat plate under 1e3 Pa (E 70e9, nu 0.3, rho 2700,
    t 0.01), one thickness DV per element, GMRES + ILU(0) to 1e-12."""
    p = meshes.plate(32, 32, 1.0, 1.0, t=0.01)
    e = meshes.plate_edges(32, 32).astype(np.int32)
    p["bc_nodes"], p["bc_masks"] = e, np.full(len(e), 0x3F, np.int32)
    p["pres_elems"] = np.arange(1024, dtype=np.int32)
    p["pres_vals"] = np.full(4096, 1e3)
    add_tests_vectors(p, 31)
    p["gmres_m"], p["gmres_restart"], p["rtol"] = 300, 10, 1e-12
    return p


def case_shell_cyl():
    p = meshes.cylinder(16, 6, R=1.0, L=3.0, t=0.005)
    rng = np.random.default_rng(41)
    p["thick"] = 0.004 + 0.004 * rng.random(p["nelem"])
    nc, nz = 16, 6
    bot = np.arange(nc, dtype=np.int32)
    p["bc_nodes"], p["bc_masks"] = bot, np.full(nc, 0x3F, np.int32)
    p["pres_elems"] = np.arange(p["nelem"], dtype=np.int32)
    p["pres_vals"] = np.full(4 * p["nelem"], -5e3)
    f = np.zeros((p["nnodes"], 6))
    f[nc * nz + np.arange(nc), 2] = -1e5 * 2 * np.pi / nc
    p["force"] = f.ravel()
    add_tests_vectors(p, 42)
    p["gmres_m"], p["gmres_restart"], p["rtol"] = 200, 10, 1e-12
    return p


def case_hex_block():
    rng = np.random.default_rng(51)
    nx, ny, nz = 4, 4, 3
    rho = 0.1 + 0.9 * rng.random(nx * ny * nz)
    p = meshes.hex_block(nx, ny, nz, 2.0, 2.0, 1.0, thick=rho ** 3)
    xyz = p["xpts"].reshape(-1, 3)
    bcn = np.nonzero(xyz[:, 0] == 0.0)[0].astype(np.int32)
    p["bc_nodes"], p["bc_masks"] = bcn, np.full(len(bcn), 0x7, np.int32)
    ijk = p["elem_ijk"]
    te = np.nonzero((ijk[:, 0] == nx - 1) & (np.abs(ijk[:, 1] - 1.5) < 1.0))[0]
    p["trac_elems"] = te.astype(np.int32)
    p["trac_faces"] = np.full(len(te), 1, np.int32)
    p["trac_vals"] = np.tile([0.0, 0.0, -1e4], len(te))
    add_tests_vectors(p, 52)
    p["ks_weight"] = 100.0
    p["gmres_m"], p["gmres_restart"], p["rtol"] = 200, 5, 1e-12
    return p


def case_hex_rand():
    p = meshes.random_hex_elements(5, seed=61)
    # Clamp the four z = -1 face nodes of every element (no rigid modes)
    p["bc_nodes"] = (8 * np.arange(5)[:, None] + np.arange(4)).ravel().astype(
        np.int32)
    p["bc_masks"] = np.full(20, 0x7, np.int32)
    rng = np.random.default_rng(62)
    p["force"] = 1e3 * rng.standard_normal(p["nnodes"] * 3)
    add_tests_vectors(p, 63)
    p["gmres_m"], p["gmres_restart"], p["rtol"] = 100, 5, 1e-12
    return p


CASES = {
    "shell_rand": case_shell_rand,
    "shell_rand_refaxis": case_shell_rand_refaxis,
    "shell_beam": case_shell_beam,
    "shell_plate8": case_shell_plate8,
    "shell_plate8_refaxis": case_shell_plate8_refaxis,
    "shell_c1": case_shell_c1,
    "shell_cyl": case_shell_cyl,
    "hex_cube": case_hex_cube,
    "hex_block": case_hex_block,
    "hex_rand": case_hex_rand,
}

# Large reference arrays that are not stored for the bigger cases (their
# content is covered by the smaller ones); scalars and vectors always are.
DROP_LARGE = {"shell_c1": {"jac_nobc_vals"}}


def main(names=None):
    for name in (names or CASES):
        prob = CASES[name]()
        ref = run_reference(prob)
        rec = {}
        for k, v in prob.items():
            if isinstance(v, np.ndarray) or np.isscalar(v):
                rec["in_" + k] = np.asarray(v)
        for k, v in ref.items():
            if k in DROP_LARGE.get(name, ()):
                rec["sum_" + k] = np.array([np.sum(v), np.sum(np.abs(v))])
                continue
            rec["ref_" + k] = v
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **rec)
        print(f"{name}: funcs={ref.get('funcs')} iters={ref.get('gmres_iters')}"
              f" size={os.path.getsize(path)}")


ILUK_KEYS = ("ilu1_apply", "ilu2_apply")


def add_keys(names, gen, keys):
    """Run a reference build on each stored fixture's inputs and add the
    given outputs as ref_<key> (the stored inputs and outputs stay)."""
    for name in (names or CASES):
        path = os.path.join(HERE, name + ".npz")
        rec = dict(np.load(path))
        prob = {k[3:]: v for k, v in rec.items() if k.startswith("in_")}
        ref = run_reference(prob, gen)
        for k in keys:
            if k in ref:
                rec["ref_" + k] = ref[k]
        np.savez_compressed(path, **rec)
        print(name, {k: float(np.abs(ref[k]).max()) for k in keys
                     if k in ref})


if __name__ == "__main__":
    if sys.argv[1:2] == ["--xpt"]:
        add_keys(sys.argv[2:], GEN_CPLX, XPT_KEYS)
    elif sys.argv[1:2] == ["--iluk"]:
        add_keys(sys.argv[2:], GEN, ILUK_KEYS)
    elif sys.argv[1:2] == ["--keys"]:
        # --keys k1,k2 case...: add the named reference outputs
        add_keys(sys.argv[3:], GEN, tuple(sys.argv[2].split(",")))
    else:
        main(sys.argv[1:] or None)
