"""Small stand-alone runs of single kernels of the path, for profilers.

    python -m tacs_gb300.workloads gmres [--n 64] [--m 30] [--mixed]
    python -m tacs_gb300.workloads hex [--n 64]
    python -m tacs_gb300.workloads spmv [--n 512]
    python -m tacs_gb300.workloads assemble [--n 256]

gmres: one restart cycle of GMRES(m) + natural-order ILU(0) on an n x n
clamped MITC4 plate (random right-hand side); hex: three residual +
Jacobian assemblies of an n x n x n/2 hex8 SIMP block; spmv: five BCSR
mat-vecs on an n x n clamped plate; assemble: three MITC4 assemblies of an
n x n plate.  Each prints one line and exits 0 on success.
"""
from __future__ import annotations

import argparse

import torch

from . import meshes, problem


def gmres(n=64, m=30, mixed=False):
    M = problem.GpuModel(meshes.clamped_plate(n))
    mat = M.new_mat()
    M.assemble_jacobian(M.vec(), mat, M.vec())
    pc = problem.Pc(mat, 0, 1 if mixed else 0)
    pc.factor()
    ksm = problem.Ksm(mat, pc, m, 0, mixed)
    ksm.set_tolerances(1e-14)
    b = torch.randn(M.ndof, dtype=torch.float64, device="cuda",
                    generator=torch.Generator("cuda").manual_seed(0))
    M.apply_bcs(b)
    ksm.solve(b)
    torch.cuda.synchronize()
    return f"gmres n={n} m={m} iterations={ksm.iters} schedule={pc.schedule()}"


def hex_block(n=64):
    p = meshes.hex_c3(n, n, n // 2)
    M = problem.GpuModel(p)
    u, res, mat = M.vec(), M.vec(), M.new_mat()
    for _ in range(3):
        M.assemble_jacobian(u, mat, res)
    torch.cuda.synchronize()
    return f"hex elements={p['nelem']} colours={M.ncolors}"


def spmv(n=512):
    M = problem.GpuModel(meshes.clamped_plate(n))
    mat = M.new_mat()
    M.assemble_jacobian(M.vec(), mat, M.vec())
    x = torch.randn(M.ndof, dtype=torch.float64, device="cuda")
    for _ in range(5):
        mat.mult(x)
    torch.cuda.synchronize()
    return f"spmv blocks={mat.nnz}"


def assemble(n=256):
    M = problem.GpuModel(meshes.clamped_plate(n))
    u, res, mat = M.vec(), M.vec(), M.new_mat()
    for _ in range(3):
        M.assemble_jacobian(u, mat, res)
    torch.cuda.synchronize()
    return f"assemble elements={n * n} colours={M.ncolors}"


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["gmres", "hex", "spmv", "assemble"])
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--m", type=int, default=30)
    ap.add_argument("--mixed", action="store_true")
    a = ap.parse_args(argv)
    if a.case == "gmres":
        print(gmres(a.n or 64, a.m, a.mixed))
    elif a.case == "hex":
        print(hex_block(a.n or 64))
    elif a.case == "spmv":
        print(spmv(a.n or 512))
    else:
        print(assemble(a.n or 256))


if __name__ == "__main__":
    main()
