"""Small stand-alone runs of single kernels of the path, for profilers.

    python -m tacs_gb300.workloads gmres [--n 64] [--m 30] [--mixed]
    python -m tacs_gb300.workloads hex [--n 64]
    python -m tacs_gb300.workloads spmv [--n 512]
    python -m tacs_gb300.workloads assemble [--n 256]
    python -m tacs_gb300.workloads direct [--n 512]
    python -m tacs_gb300.workloads batch [--count 48] [--nmax 256]

gmres: one restart cycle of GMRES(m) + natural-order ILU(0) on an n x n
clamped MITC4 plate (random right-hand side); hex: three residual +
Jacobian assemblies of an n x n x n/2 hex8 SIMP block; spmv: five BCSR
mat-vecs on an n x n clamped plate; assemble: three MITC4 assemblies of an
n x n plate; direct: the complete factorisation of the simply supported
n x n plate (2 m at 512 x 512) in FP64 and in FP32, one factorisation and
one solve each; batch: the factorisation of the batch of clamped plates
(N log-uniform in [16, nmax]) in FP32 and in FP64, then one 4-load-case
solve of each (the FP32 one as one refinement step).  Each prints one line
and exits 0 on success.
"""
from __future__ import annotations

import argparse

import numpy as np

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


def direct(n=512):
    from . import _lib
    p = meshes.plate_c2(n, 2.0 * n / 512)
    M = problem.GpuModel(p)
    mat = M.new_mat()
    r0 = M.vec()
    M.assemble_jacobian(M.vec(), mat, r0)
    out = []
    for prec in (_lib.PREC_FP64, _lib.PREC_FP32):
        d = problem.Direct(mat, precision=prec)
        d.factor()
        b = -r0 if prec == _lib.PREC_FP64 else (-r0).float()
        d.solve(b)
        torch.cuda.synchronize()
        out.append(f"prec={prec} supernodes={d.stats()['supernodes']}")
        del d
    return "direct " + " ".join(out)


def batch(count=48, nmax=256):
    from . import _lib
    bp = meshes.batch_plates(count=count, nmax=nmax)
    M = problem.GpuModel(bp)
    M.set_fixed_geometry(True)
    F = problem.batch_loads(M)
    mat = M.new_mat()
    M.assemble_jacobian(M.vec(), mat, M.vec())
    for prec in (_lib.PREC_FP32, _lib.PREC_FP64):
        d = problem.Direct(mat, precision=prec)
        d.factor()
        # FP32: one refinement step = one 4-right-hand-side FP32 solve
        if prec == _lib.PREC_FP32:
            d.solve(F, steps=1, tol=1.0)
        else:
            d.solve(F)
        del d
    torch.cuda.synchronize()
    return f"batch plates={count} elements={bp['nelem']}"


def functions(nc=384, nz=256, reps=5):
    """The compliance value, its df/du and its total derivative with
    respect to the thicknesses (adjoint = df/du) on the 384 x 256 MITC4
    cylinder at a seeded state, `reps` times; prints the time per
    repetition of each call (host clock, each behind a synchronisation)."""
    import time
    c = meshes.cylinder_c5(nc, nz)
    M = problem.GpuModel(c)
    rng = np.random.default_rng(5)
    u = M.vec(1e-4 * rng.standard_normal(M.ndof))
    M.apply_bcs(u)
    ms = {"eval_functions": 0.0, "add_sv_sens": 0.0,
          "add_total_derivative": 0.0}

    def lap(name, t0):
        torch.cuda.synchronize()
        ms[name] += (time.perf_counter() - t0) * 1e3 / reps

    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        M.eval_functions(u, (0,))
        lap("eval_functions", t0)
        t0 = time.perf_counter()
        dfdu = M.vec()
        M.add_sv_sens(u, [0], [dfdu])
        lap("add_sv_sens", t0)
        t0 = time.perf_counter()
        g = M.dv_vec()
        M.add_total_derivative(u, 0, dfdu, g, 1.0, -1.0)
        lap("add_total_derivative", t0)
    return (f"functions elements={c['nelem']} ms per call: " +
            " ".join(f"{k}={v:.2f}" for k, v in ms.items()))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["gmres", "hex", "spmv", "assemble",
                                     "direct", "batch", "functions"])
    ap.add_argument("--count", type=int, default=48)
    ap.add_argument("--nmax", type=int, default=256)
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
    elif a.case == "direct":
        print(direct(a.n or 512))
    elif a.case == "batch":
        print(batch(a.count, a.nmax))
    elif a.case == "functions":
        print(functions())
    else:
        print(assemble(a.n or 256))


if __name__ == "__main__":
    main()
