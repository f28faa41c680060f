"""Benchmark: MITC4 residual + Jacobian assembly (elements/s) on a GB300.

Workload (the configuration the headline metric is quoted on): a 2.0 m
square flat plate of 512 x 512 MITC4 shell elements (262,144 elements,
263,169 nodes, 1,579,014 dof, 2,362,369 6x6 blocks), per-element thickness
seeded uniform in [0.005, 0.02] (numpy default_rng(2)), E = 70e9, nu = 0.3,
nodal pressure p(x, y) = 1e3 (1 + 0.5 sin(pi x) sin(pi y)) (x, y in metres),
simply-supported edges (u, v, w fixed).  Synthetic data; the BCSR matrix
(680 MB) and the state exceed the 129 MB L2, so no flush is needed between
steps.

One step = TACSAssembler::assembleJacobian(1, 0, 0, res, mat) semantics:
zero, element residual + Jacobian for every element, scatter into BCSR,
row-zero Dirichlet conditions.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  --impl reference times the CPU restatement
of the reference path (oracle/, all host threads) on a bounded sample of the
same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "elements/s res+Jacobian assembly; adjoint grad s/solve, FP32-precond vs FP64"
UNIT = "elements/s"


def c2_problem(n=512, L=2.0, seed=2):
    from tacs_gb300 import meshes
    return meshes.plate_c2(n, L, seed)


def clamped_plate(n, seed=5):
    """C1-type clamped 1 m plate (E 70e9, nu 0.3, rho 2700), per-element
    thickness U[0.008, 0.012], uniform 1e3 Pa: the adjoint-gradient workload
    (GMRES + ILU(0) converges on it, unlike the simply-supported 512 x 512
    plate, where the reference's own GMRES(80) + ILU(0) stalls)."""
    from tacs_gb300 import meshes
    rng = np.random.default_rng(seed)
    p = meshes.plate(n, n, 1.0, 1.0, t=0.01,
                     thick=rng.uniform(0.008, 0.012, n * n))
    e = meshes.plate_edges(n, n).astype(np.int32)
    p["bc_nodes"], p["bc_masks"] = e, np.full(len(e), 0x3F, np.int32)
    p["pres_elems"] = np.arange(n * n, dtype=np.int32)
    p["pres_vals"] = np.full(4 * n * n, 1e3)
    return p


def adjoint_section(n, torch, colored=False):
    """Seconds per adjoint gradient of compliance and KS failure: Jacobian
    assembly, factorisation, forward GMRES solve, both functions, two adjoint
    solves and the fused total derivatives, for three solver set-ups."""
    from tacs_gb300 import _lib, problem
    p = clamped_plate(n)
    M = problem.GpuModel(p)
    f0 = np.zeros(M.ndof)
    # (label, pc type, mixed, fill level); ILU(5) is what the reference's
    # Python Pc builds for an assembler matrix (TACSAdditiveSchwarz(mat, 5))
    runs = [("fp64_ilu0_natural", _lib.PC_ILU0, False, 0),
            ("mixed_ilu0_natural", _lib.PC_ILU0, True, 0),
            ("fp64_ilu3_natural", _lib.PC_ILU0, False, 3),
            ("mixed_ilu3_natural", _lib.PC_ILU0, True, 3),
            ("fp64_ilu5_natural", _lib.PC_ILU0, False, 5)]
    if colored:
        runs += [("fp64_ilu0_colored", _lib.PC_ILU0_COLORED, False, 0),
                 ("mixed_ilu0_colored", _lib.PC_ILU0_COLORED, True, 0)]
    out, grads = {"workload": f"clamped MITC4 plate {n}x{n}, GMRES(100) "
                              "to 1e-10, compliance + KS(100) gradients",
                  "elements": n * n, "dof": int(M.ndof)}, {}
    for label, kind, mixed, lev in runs:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = problem.static_adjoint(M, f0, 100, 400, 1e-10, pc_kind=kind,
                                   mixed=mixed, lev_fill=lev)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        grads[label] = [g.cpu().numpy() for g in r["grads"]]
        out[label] = {"s_per_gradient": dt, "iters": r["iters"],
                      "converged": [int(f) for f in r["flags"]],
                      "ilu_schedule": r["pc"].schedule(),
                      "launch": r["ksm"].graph_info()}
        if label == "fp64_ilu0_natural":
            out["shape_derivative"] = guarded(
                lambda: xpt_timing(M, r, torch))
    ref = grads["fp64_ilu0_natural"]
    for label in [r[0] for r in runs[1:]]:
        out[label]["grad_rel_err_vs_fp64_natural"] = [
            float(np.abs(a - b).max() / np.abs(b).max())
            for a, b in zip(grads[label], ref)]
    out["mixed_speedup_vs_fp64_natural"] = (
        out["fp64_ilu0_natural"]["s_per_gradient"]
        / out["mixed_ilu0_natural"]["s_per_gradient"])
    out["ilu3_speedup_vs_ilu0_fp64"] = (
        out["fp64_ilu0_natural"]["s_per_gradient"]
        / out["fp64_ilu3_natural"]["s_per_gradient"])
    return out, p


def xpt_timing(M, r, torch, reps=3):
    """Node-coordinate total derivative df/dX - psi^T dR/dX of compliance
    and KS from a solved state and its adjoints (the fused addXptSens +
    addAdjointResXptSensProducts pass), CUDA-event time per function, for
    both exact forms of the shell derivative: dual numbers per coordinate
    and the reverse sweep per element (the default); their largest
    relative difference is reported beside the times."""
    u, psis = r["u"], r["psis"]
    out = {}
    res = {}
    try:
        for label, reverse in (("forward_dual", False),
                               ("reverse_sweep", True)):
            M.set_xpt_mode(reverse)
            ms, grads = [], []
            for fn in (0, 1):
                M.eval_functions(u, [fn])
                gX = M.node_vec()
                M.add_total_xpt_derivative(u, fn, psis[fn], gX)  # warm-up
                grads.append(gX.clone())
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    M.add_total_xpt_derivative(u, fn, psis[fn], gX)
                e1.record()
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1) / reps)
            res[label] = grads
            out[label] = {"ms_per_function": ms,
                          "elements_per_s": [M.nelem / (t / 1e3)
                                             for t in ms]}
    finally:
        M.set_xpt_mode(True)
    out["reverse_vs_forward_max_rel_diff"] = max(
        float((a - b).abs().max() / b.abs().max())
        for a, b in zip(res["reverse_sweep"], res["forward_dual"]))
    out["reverse_speedup"] = (sum(out["forward_dual"]["ms_per_function"]) /
                              sum(out["reverse_sweep"]["ms_per_function"]))
    return out


def c2_adjoint_section(torch, n=512):
    """The 512 x 512 simply supported plate (per-element thickness, nodal
    pressure field): compliance and its gradient with respect to the
    262,144 thicknesses through torch.autograd, both solves by the complete
    multifrontal factorisation (GMRES(80) + ILU(0) does not converge on
    this plate), refined to the 1e-10 relative residual of the stated
    GMRES tolerance (or the FP64 floor).  Times the analysis, the
    factorisation, one solve and the whole gradient, and the whole gradient
    with the FP32 factorisation and FP64 refinement (`mixed`, with its
    error against the FP64 gradient)."""
    from tacs_gb300 import autograd as ag
    from tacs_gb300 import problem
    p = c2_problem(n=n)
    M = problem.GpuModel(p)
    M.set_fixed_geometry(True)  # thicknesses change, the nodes do not
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    solver = ag.StaticSolver(M, np.zeros(M.ndof), rtol=1e-10, direct=True)
    torch.cuda.synchronize()
    t_analysis = time.perf_counter() - t0
    x = torch.as_tensor(np.asarray(p["thick"]), device="cuda")
    out = {"workload": f"simply supported MITC4 plate {n}x{n}, compliance "
                       "gradient through torch.autograd, direct solves",
           "elements": n * n, "dof": int(M.ndof),
           "analysis_s": t_analysis, "factor": solver.direct.stats()}
    # the last pass is timed: the first one factors once, the second
    # factorisation also tunes the solves' launch shapes
    for rep in range(3):
        xr = x.clone().requires_grad_(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f = ag.static_functional(xr, solver, 0)
        f.sum().backward()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    out["s_per_gradient"] = dt
    out["compliance"] = float(f.item())
    g64 = xr.grad.clone()
    # the same gradient with the FP32 factorisation and FP64 refinement
    solver32 = ag.StaticSolver(M, np.zeros(M.ndof), rtol=1e-10,
                               direct="mixed")
    for rep in range(3):
        xr = x.clone().requires_grad_(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f32 = ag.static_functional(xr, solver32, 0)
        f32.sum().backward()
        torch.cuda.synchronize()
        dt32 = time.perf_counter() - t0
    st32 = solver32.direct.stats()
    out["mixed"] = {
        "s_per_gradient": dt32,
        "speedup_vs_fp64": dt / dt32,
        "grad_rel_err_vs_fp64": float((xr.grad - g64).abs().max()
                                      / g64.abs().max()),
        "fp32_mode": st32["fp32_mode"],
        "refinement_steps": st32["last_refinement_steps"],
        "gmres_ir_iters": st32["last_gmres_iters"],
        "gmres_ir_fp64_factor": st32["gmres_ir_fp64_factor"],
        "fell_back_to_fp64": st32["fell_back_to_fp64"]}
    del solver32
    b = M.vec()
    M.assemble_res(M.vec(), res=b)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    solver.direct.factor()
    e1.record()
    torch.cuda.synchronize()
    out["factor_ms"] = e0.elapsed_time(e1)
    e0.record()
    u = solver.direct.solve(b)
    e1.record()
    torch.cuda.synchronize()
    out["solve_ms"] = e0.elapsed_time(e1)
    r = solver.mat.mult(u) - b
    out["true_residual_rel"] = float(r.abs().max() / b.abs().max())
    return out


def hex_section(torch, steps=5):
    """Hex8 SIMP block (128 x 128 x 64 elements, 3.24M dof, 28.6M 3x3
    blocks): residual + Jacobian assembly throughput."""
    from tacs_gb300 import meshes, problem
    p = meshes.hex_c3()
    M = problem.GpuModel(p)
    u, res, mat = M.vec(), M.vec(), M.new_mat()
    for _ in range(2):
        M.assemble_jacobian(u, mat, res)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        M.assemble_jacobian(u, mat, res)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    nnzb = mat.nnz
    algo = (p["nnodes"] * 6 * 8 + p["nelem"] * (8 * 4 + 8) + p["nnodes"] * 3 * 8
            + nnzb * 9 * 8)
    out = {"workload": "hex8 SIMP block 128x128x64 (2x2x1 m), clamped x=0, "
                       "traction patch on x=2; assembleRes+assembleJacobian",
           "elements": int(p["nelem"]), "dof": int(M.ndof),
           "bcsr_blocks": int(nnzb), "ms_per_step": ms,
           "elements_per_s": p["nelem"] / (ms / 1e3),
           "hbm_gbs_algorithmic": algo / (ms / 1e3) / 1e9,
           "algorithmic_bytes": int(algo),
           "fp64": fp64_roofline("hex", p["nelem"] / (ms / 1e3))}
    # node-coordinate total derivatives at a seeded state and adjoint (the
    # kernels' cost does not depend on the values)
    g = torch.Generator(device="cuda").manual_seed(11)
    us = 1e-5 * torch.randn(M.ndof, dtype=torch.float64, device="cuda",
                            generator=g)
    ps = torch.randn(M.ndof, dtype=torch.float64, device="cuda", generator=g)
    out["shape_derivative"] = xpt_timing(M, {"u": us, "psis": [ps, ps]},
                                         torch, reps=2)
    out["shape_derivative"]["workload"] = (
        "hex8 block 128x128x64: df/dX - psi^T dR/dX of compliance and KS")
    del M, mat, u, res
    torch.cuda.empty_cache()
    return out


def c3_solve_section(torch, pc_kind=0, h=1e-6, direct=None):
    """The 128 x 128 x 64 SIMP block solved and differentiated: FP64 GMRES
    with ILU(0) (pc_kind: natural or colour-reordered), or with
    direct="mixed" the complete factorisation in FP32 with FP64 refinement
    (GMRES-IR where refinement stagnates), compliance and its
    gradient with respect to the 1,048,576 densities through the autograd
    backward (dC/drho = 3 rho^2 dC/dt), checked by
      * a central difference with h along a seeded positive direction
        (seed 34) over all densities, two compliances subtracted (a single
        density moves the compliance by ~1e-12 of itself at h = 1e-6, below
        FP64 resolution; the per-element central differences on 32 seeded
        elements run on a reduced block in tests/test_autograd.py);
      * the oracle's addDVSens + addAdjointResProducts at the GPU's state
        and adjoint (psi = 2 u for compliance) against the GPU's."""
    import oracle
    from tacs_gb300 import autograd as ag
    from tacs_gb300 import meshes, problem
    p = meshes.hex_c3()
    M = problem.GpuModel(p)
    M.set_fixed_geometry(True)
    t0 = time.perf_counter()
    solver = ag.StaticSolver(M, np.zeros(M.ndof), m=200, nrestart=40,
                             rtol=1e-10, pc_kind=pc_kind,
                             direct=direct or False)
    torch.cuda.synchronize()
    s_setup = time.perf_counter() - t0  # the direct analysis, once
    rho0 = torch.as_tensor(p["rho"], device="cuda")
    x = rho0.clone().requires_grad_(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    c = ag.static_functional(x ** 3, solver, 0).sum()
    c.backward()
    torch.cuda.synchronize()
    s_grad = time.perf_counter() - t0
    g = x.grad.detach()
    u = solver.u[0].clone()
    out = {"workload": "hex8 SIMP block 128x128x64, compliance gradient wrt "
                       "densities, " + ("complete factorisation in FP32, "
                                        "FP64 refinement / GMRES-IR"
                                        if direct else "GMRES(200) + ILU(0)")
                       + " to 1e-10",
           "elements": int(p["nelem"]), "dof": int(M.ndof),
           "preconditioner": ("complete factorisation (FP32)" if direct
                              else "natural ILU(0)" if pc_kind == 0
                              else "colour-reordered ILU(0)"),
           "s_per_gradient": s_grad, "compliance": float(c.detach()),
           "iters": [int(np.max(i)) for i in solver.iters]}
    if direct:
        st = solver.direct.stats()
        out["direct"] = {"analysis_s": s_setup, **{
            k: st[k] for k in ("supernodes", "levels", "factor_bytes",
                               "pool_bytes", "flops", "max_front",
                               "fp32_mode", "last_gmres_iters",
                               "fell_back_to_fp64")}}
        # the FP32 factorisation alone, once more (no launch-shape tuning)
        solver.direct.autotune = False
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        solver.direct.factor()
        e1.record()
        torch.cuda.synchronize()
        fms = e0.elapsed_time(e1)
        out["direct"]["factor_ms"] = fms
        out["direct"]["factor_tflops"] = st["flops"] / (fms * 1e-3) / 1e12
    # directional central difference, warm-started solves (with the
    # factorisation: GMRES preconditioned by the unperturbed FP32 factor)
    zero = M.vec()
    mat_p = M.new_mat()
    if direct:
        pc_p = problem.Pc.from_direct(solver.direct)
        pc_p.factor()
        ksm_p = problem.Ksm(mat_p, pc_p, 30, 20)
    else:
        ksm_p = problem.Ksm(mat_p, solver.pc, 200, 40)
    ksm_p.set_tolerances(1e-9, 1e-30)
    d = torch.as_tensor(np.random.default_rng(34).random(int(p["nelem"])),
                        device="cuda")
    t0 = time.perf_counter()
    cs = []
    for sgn in (1.0, -1.0):
        M.set_design_vars((rho0 + sgn * h * d) ** 3)
        r0 = M.vec()
        M.assemble_jacobian(zero, mat_p, r0)
        xs, fl = ksm_p.solve(-r0, x=u.clone(), zero_guess=False)
        cs.append(float(M.eval_functions(xs, [0])[0]))
    M.set_design_vars(rho0 ** 3)
    fd_dir = (cs[0] - cs[1]) / (2.0 * h)
    adj_dir = float((g * d).sum())
    out["fd_direction"] = {"h": h, "seed": 34, "fd": fd_dir,
                           "adjoint": adj_dir,
                           "rel_err": abs(fd_dir - adj_dir) / abs(adj_dir),
                           "s": time.perf_counter() - t0}
    # oracle: addDVSens + addAdjointResProducts at the GPU state
    psi = 2.0 * u
    gt = M.dv_vec()
    M.eval_functions(u, [0])
    M.add_total_derivative(u, 0, psi, gt, 1.0, -1.0)
    o = oracle.Oracle(p, nthreads=os.cpu_count() or 1)
    uh, ph = u.cpu().numpy(), psi.cpu().numpy()
    t0 = time.perf_counter()
    go = o.dv_sens(uh, 0) + o.adj_res_product(uh, ph, -1.0)
    gth = gt.cpu().numpy()
    out["oracle_dv_adjres"] = {
        "rel_err": float(np.abs(gth - go).max() / np.abs(go).max()),
        "chain_rule_rel_err": float(
            (3.0 * rho0 ** 2 * gt - g).abs().max() / g.abs().max()),
        "oracle_s": time.perf_counter() - t0}
    del M, solver, mat_p, ksm_p
    torch.cuda.empty_cache()
    return out


def fixed_geometry_section(torch, p, steps=20, label="", bs=6):
    """Fixed-geometry assembly (tg_assembler_set_fixed_geometry) of the same
    workload: the residual and Jacobian from per-geometry coefficient
    matrices, each BCSR block summed from its contributions and written
    once.  Times the one-off build (classes, coefficient table, loads) and
    the steady-state assembly (CUDA events, inputs larger than L2), and
    checks the result against the element kernels on the same state."""
    from tacs_gb300 import problem
    M = problem.GpuModel(p)
    g = torch.Generator(device="cuda").manual_seed(5)
    u = 1e-4 * torch.randn(M.ndof, dtype=torch.float64, device="cuda",
                           generator=g)
    mat0, res0 = M.new_mat(), M.vec()
    M.assemble_jacobian(u, mat0, res0)  # element kernels
    M.set_fixed_geometry(True)
    mat, res = M.new_mat(), M.vec()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    M.assemble_jacobian(u, mat, res)  # builds the cache
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    dv = float((mat.vals - mat0.vals).abs().max() / mat0.vals.abs().max())
    dr = float((res - res0).abs().max() / res0.abs().max())
    del mat0, res0
    for _ in range(3):
        M.assemble_jacobian(u, mat, res)
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        M.assemble_jacobian(u, mat, res)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    nn, ne = p["nnodes"], p["nelem"]
    npe = 4 if bs == 6 else 8
    algo = (nn * (3 + bs) * 8 + ne * (4 * npe + 8) + nn * bs * 8
            + mat.nnz * bs * bs * 8)
    peak, src = measured_peaks()
    info = M.fixed_geometry_info()
    ach = algo / (ms / 1e3) / 1e9
    out = {"workload": label, "elements": int(ne), "bcsr_blocks": int(mat.nnz),
           "build_s": build_s, "ms_per_step": ms,
           "elements_per_s": ne / (ms / 1e3), "geometry_classes":
           info["classes"], "table_bytes": info["table_bytes"],
           "plan_bytes": info["plan_bytes"],
           "rel_diff_vs_element_kernels": {"K": dv, "R": dr},
           "roofline": {"bound": "hbm", "achieved": ach, "peak": peak,
                        "unit": "GB/s", "frac": ach / peak,
                        "peak_source": src, "kernel": "geo_assembly_kernel",
                        "algorithmic_bytes": int(algo)},
           "gpu_launches_per_step": 1}
    del M, mat, res, u
    torch.cuda.empty_cache()
    return out


def cylinder_section(torch, nc=384, nz=256):
    """Cylinder (384 x 256 MITC4, 592k dof): static solve and compliance
    adjoint gradient, all-FP64 against mixed precision (FP32 factor and
    mat-vec inside FP64 GMRES with true-residual refinement), both with the
    colour-reordered ILU(0) (the natural order of a closed cylinder is one
    sequential chain of 98,688 rows); beside them the complete
    factorisation in FP64 and in FP32 with FP64 refinement.  Each
    gradient's error is against the FP64 ILU(0) arm."""
    from tacs_gb300 import _lib, meshes, problem
    c = meshes.cylinder_c5(nc, nz)
    M = problem.GpuModel(c)
    out = {"workload": f"cylinder R=1 L=3 t=0.005, {nc}x{nz} MITC4, clamped "
                       "z=0, axial 1e5 N/m + 5e3 Pa; GMRES(200) to 1e-10, "
                       "compliance adjoint gradient",
           "elements": int(c["nelem"]), "dof": int(M.ndof)}
    g = {}
    # the configured solver (FP32 / FP64 ILU(0) inside FP64 GMRES), then the
    # complete factorisation in FP64 and in FP32 with FP64 refinement, all
    # to the same 1e-10 relative residual
    arms = (("fp64_ilu0_colored", dict(pc_kind=_lib.PC_ILU0_COLORED)),
            ("mixed_ilu0_colored", dict(pc_kind=_lib.PC_ILU0_COLORED,
                                        mixed=True)),
            ("fp64_direct", dict(direct="fp64")),
            ("mixed_direct", dict(direct="mixed")))
    for label, kw in arms:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = problem.static_adjoint(M, c["force"], 200, 30, 1e-10,
                                   funcs=(0,), **kw)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        g[label] = (r["grads"][0].cpu().numpy(), r["funcs"][0])
        out[label] = {"s_per_gradient": dt, "iters": r["iters"],
                      "converged": [int(f) for f in r["flags"]],
                      "compliance": float(r["funcs"][0])}
        if r.get("direct") is not None:
            out[label]["direct"] = {
                k: r["direct"].stats()[k]
                for k in ("flops", "factor_bytes", "fell_back_to_fp64",
                          "fp32_mode", "last_gmres_iters")}
    b = g["fp64_ilu0_colored"]
    for label in ("mixed_ilu0_colored", "fp64_direct", "mixed_direct"):
        a = g[label]
        out[label]["grad_rel_err_vs_fp64"] = float(
            np.abs(a[0] - b[0]).max() / np.abs(b[0]).max())
        out[label]["compliance_rel_err_vs_fp64"] = float(
            abs(a[1] - b[1]) / abs(b[1]))
    out["mixed_speedup_vs_fp64"] = (out["fp64_ilu0_colored"]["s_per_gradient"]
                                    / out["mixed_ilu0_colored"]["s_per_gradient"])
    out["mixed_direct_speedup_vs_fp64_direct"] = (
        out["fp64_direct"]["s_per_gradient"]
        / out["mixed_direct"]["s_per_gradient"])
    a, b = g["mixed_direct"], g["fp64_direct"]
    out["mixed_direct"]["grad_rel_err_vs_fp64_direct"] = float(
        np.abs(a[0] - b[0]).max() / np.abs(b[0]).max())
    # where a one-off direct arm's time goes (outside the timed arms): the
    # steps of problem.static_adjoint one by one, each behind a
    # synchronisation
    for label, prec in (("fp64_direct", _lib.PREC_FP64),
                        ("mixed_direct", _lib.PREC_FP32)):
        bd = {}
        t = [time.perf_counter()]

        def lap(name):
            torch.cuda.synchronize()
            t.append(time.perf_counter())
            bd[name] = bd.get(name, 0.0) + t[-1] - t[-2]

        torch.cuda.synchronize()
        t[0] = time.perf_counter()
        mat = M.new_mat()
        res = M.vec()
        M.assemble_jacobian(M.vec(), mat, res)
        lap("assemble")
        d = problem.Direct(mat, precision=prec)
        lap("create")
        d.factor()
        lap("factor")
        f = torch.as_tensor(np.asarray(c["force"], np.float64),
                            device="cuda").clone()
        M.apply_bcs(f)
        res -= f
        lap("load")
        u = -d.solve(res, rtol=1e-10)
        lap("solve")
        M.eval_functions(u, (0,))
        dfdu = M.vec()
        M.add_sv_sens(u, [0], [dfdu])
        M.apply_bcs(dfdu)
        lap("functions_and_dfdu")
        psi = d.solve(dfdu, rtol=1e-10)
        lap("solve")
        gr = M.dv_vec()
        M.add_total_derivative(u, 0, psi, gr, 1.0, -1.0)
        lap("total_derivative")
        bd["solve_steps"] = d.last_steps
        bd["sum"] = t[-1] - t[0]
        out[label]["breakdown_s"] = bd
        del d, mat, res, f, u, dfdu, psi, gr
    del M
    torch.cuda.empty_cache()
    return out


def batch_section(torch, count=48, nmax=256, m=100, nrestart=100, pc_kind=0,
                  lev_fill=0, direct=False):
    """Independent clamped plates of seeded uneven sizes (N log-uniform in
    [16, nmax]) in one assembler: 4 load cases per plate, one batched
    GMRES for all forward solves and one for all adjoint solves, KS failure
    (weight 100, yield 2.7e8) gradient per plate and load case; FP64 and
    mixed precision."""
    from tacs_gb300 import _lib, meshes, problem
    bp = meshes.batch_plates(count=count, nmax=nmax)
    M = problem.GpuModel(bp)
    # the meshes do not move: assembly, functions and sensitivities from
    # the per-geometry tables (one class per plate size here)
    M.set_fixed_geometry(True)
    F = problem.batch_loads(M)
    out = {"workload": f"{count} clamped MITC4 plates N~logU[16,{nmax}] "
                       "(seed 4), 4 load cases each, KS(100) adjoint "
                       f"gradients, GMRES({m}) to 1e-10, "
                       + ("complete multifrontal factorisation" if direct
                          else ("natural" if pc_kind == 0
                                else "colour-reordered")
                          + f" ILU({lev_fill})"),
           "plates": count, "elements": int(bp["nelem"]),
           "dof": int(M.ndof), "systems": 4 * count}
    g = {}
    for label, mixed in (("fp64", False), ("mixed", True)):
        kw = dict(m=m, nrestart=nrestart, rtol=1e-10, pc_kind=pc_kind,
                  mixed=mixed, func=_lib.FUNC_KS_FAILURE, lev_fill=lev_fill,
                  direct=("mixed" if mixed else "fp64") if direct else False)
        first = None
        if direct:
            # the first design of an optimisation loop also runs the
            # factorisation's analysis; the next ones reuse it
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r0 = problem.batched_adjoint(M, F, **kw)
            torch.cuda.synchronize()
            first = time.perf_counter() - t0
            kw.update(direct_solver=r0["direct"], mat=r0["mat"])
            # the second design's factorisation tunes the solves' launch
            # shapes (tg_direct_autotune); the third one is timed
            problem.batched_adjoint(M, F, **kw)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = problem.batched_adjoint(M, F, **kw)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        g[label] = r["grads"].cpu().numpy()
        out[label] = {"s_per_batch": dt,
                      "first_design_s": first,
                      "s_per_gradient": dt / (4 * count),
                      "max_iters_fwd": int(r["iters_fwd"].max()),
                      "max_iters_adj": int(r["iters_adj"].max()),
                      "converged_fwd": int(r["flags_fwd"].sum()),
                      "converged_adj": int(r["flags_adj"].sum())}
        if r.get("ksm") is not None:
            out[label]["launch"] = r["ksm"].graph_info()
        if r.get("direct") is not None:
            dsol = r["direct"]
            st = dsol.stats()
            out[label]["direct"] = {
                k: st[k] for k in ("supernodes", "levels", "factor_bytes",
                                   "flops", "fell_back_to_fp64",
                                   "fp32_mode", "last_refinement_steps",
                                   "last_gmres_iters",
                                   "last_backward_error")}
            # one factorisation and one solve of the first load case alone
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            dsol.factor()
            e1.record()
            torch.cuda.synchronize()
            fms = e0.elapsed_time(e1)
            b = F[0].clone()
            t0 = time.perf_counter()
            dsol.solve(b)
            torch.cuda.synchronize()
            out[label]["direct"]["factor_ms"] = fms
            out[label]["direct"]["factor_tflops"] = st["flops"] / fms / 1e9
            out[label]["direct"]["solve_ms"] = (time.perf_counter() - t0) * 1e3
    d = g["mixed"] - g["fp64"]
    out["mixed"]["grad_rel_err_vs_fp64"] = float(
        np.abs(d).max() / np.abs(g["fp64"]).max())
    out["mixed_speedup_vs_fp64"] = out["fp64"]["s_per_batch"] / \
        out["mixed"]["s_per_batch"]
    del M
    torch.cuda.empty_cache()
    return out


def replica_time(ms, dist=None, device=None):
    """Replicas only: every rank runs the whole workload on its own GPU;
    the job's step time is the slowest rank's (max over ranks)."""
    if dist is None or not dist.is_initialized():
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# Figures carried over from the committed ncu capture of one colour launch
# (16,384 elements) of the 256 x 256 plate
# (profiles/shell_team_assembly_mitc4_256_full.md); the bench line labels
# them as such, beside the CUDA-event timings it measures itself.
SHELL_PROFILE = {
    "source": "profiles/shell_team_assembly_mitc4_256_full.md (ncu --set "
              "full, one colour launch, 256x256 plate)",
    "dram_bytes_per_launch": 100.64e6 + 36.31e6,
    "elements_per_launch": 16384,
    "fp64_pipe_active": 0.872,
}


def traffic_per_step(nelem):
    """DRAM bytes (read + write) of the assembly kernel per step, scaled
    from the capture by elements (the per-element traffic is size
    independent: colour-by-colour block read-modify-write)."""
    return int(SHELL_PROFILE["dram_bytes_per_launch"]
               / SHELL_PROFILE["elements_per_launch"] * nelem)


# FP64 work per element of one residual + Jacobian assembly (flops: add,
# sub, mul, div, sqrt; a fused multiply-add is two).
#  - reference: the reference element's addJacobian(alpha=1, beta=gamma=0),
#    counted by the operation-counting build of its sources
#    (oracle/ref/opcount.h, `make -C oracle/ref opc && oracle/_ref/op_count`)
#  - executed: this repository's kernels, from ncu's executed DFMA / DADD /
#    DMUL thread instructions over one colour launch of 16,384 elements
#    (shell: 256 x 256 plate; hex: 64 x 64 x 32 block)
FP64_FLOPS_PER_ELEMENT = {
    "shell": {"reference": 153602, "executed": 37745},
    "hex": {"reference": 149808, "executed": 14204},
}
# nominal FP64 peak: 152 SMs x 2 FMA lanes per clock x 2 flops x 2.07 GHz
FP64_PEAK_TFLOPS = 1.259


def fp64_roofline(kind, elements_per_s):
    """The kernel's FP64 throughput (executed flops) against the nominal
    FP64 peak, and the reference-equivalent rate: the reference element's
    flops for the same elements per second (above the peak when this
    formulation needs fewer flops than the reference's)."""
    f = FP64_FLOPS_PER_ELEMENT[kind]
    ach = elements_per_s * f["executed"] / 1e12
    ref = elements_per_s * f["reference"] / 1e12
    return {"unit": "TFLOP/s", "peak": FP64_PEAK_TFLOPS,
            "peak_source": "nominal (152 SMs x 2 FP64 FMA/clk x 2.07 GHz)",
            "executed_flops_per_element": f["executed"],
            "achieved": ach, "frac": ach / FP64_PEAK_TFLOPS,
            "reference_flops_per_element": f["reference"],
            "reference_equivalent": ref,
            "reference_equivalent_frac": ref / FP64_PEAK_TFLOPS}


def algorithmic_bytes(p):
    """Assembly traffic a perfect implementation moves once: node coords and
    state read, connectivity + thickness read, residual write, BCSR write."""
    nn, ne = p["nnodes"], p["nelem"]
    n = int(np.sqrt(ne))
    nnzb = (3 * (n + 1) - 2) ** 2
    return nn * (3 + 6) * 8 + ne * (4 * 4 + 8) + nn * 6 * 8 + nnzb * 36 * 8


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def guarded(fn):
    """Run one optional section of the bench line; a failure is recorded
    as {"error": ...} in that section so the line itself still prints."""
    try:
        return fn()
    except Exception as e:  # noqa: BLE001 - reported in the JSON line
        return {"error": f"{type(e).__name__}: {e}"[:500]}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fp:
            d = json.load(fp)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_baseline(p_full, seconds=12.0):
    """The oracle's threaded CPU assembly on a bounded sample (a 128 x 128
    sub-plate of the same workload), elements/s."""
    import oracle
    n = 128
    sub = c2_problem(n=n, L=2.0 * n / 512, seed=2)
    threads = os.cpu_count() or 1
    o = oracle.Oracle(sub, nthreads=threads)
    u = np.zeros(o.ndof)
    A = o.new_bcsr()
    o.assemble_jac(u, A)  # warm-up
    reps, t0 = 0, time.perf_counter()
    while True:
        o.assemble_jac(u, A)
        reps += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    o.free(A)
    return {"value": reps * sub["nelem"] / dt, "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": f"{reps} x assembleJacobian of a {n}x{n} sub-plate "
                      f"({sub['nelem']} elements), {dt:.1f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    p = c2_problem()
    steps, warm = args.steps, args.warmup
    import oracle
    n = 128
    sub = c2_problem(n=n, L=2.0 * n / 512, seed=2)
    threads = os.cpu_count() or 1
    o = oracle.Oracle(sub, nthreads=threads)
    u = np.zeros(o.ndof)
    A = o.new_bcsr()
    for _ in range(warm):
        o.assemble_jac(u, A)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.assemble_jac(u, A)
    dt = time.perf_counter() - t0
    value = steps * sub["nelem"] / dt
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": steps, "warmup": warm,
            "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "MITC4 plate 512x512 (sampled 128x128)",
                       "elements": int(p["nelem"]), "sample_elements": n * n},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads,
                             "kind": "port",
                             "sample": f"{steps} x assembleJacobian of a "
                                       f"{n}x{n} sub-plate"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--adj-size", type=int, default=64)
    ap.add_argument("--no-hex", action="store_true")
    ap.add_argument("--c3-solve", action="store_true",
                    help="solve and differentiate the 128x128x64 hex block")
    ap.add_argument("--c3-pc", type=int, default=0,
                    help="its ILU(0): 0 natural order, 2 colour-reordered")
    ap.add_argument("--no-c3", action="store_true",
                    help="skip the hex block's gradient by the FP32 complete "
                         "factorisation (c3_direct, ~40 s)")
    ap.add_argument("--no-fixed", action="store_true",
                    help="skip the fixed-geometry assembly section")
    ap.add_argument("--no-cylinder", action="store_true")
    ap.add_argument("--no-c2-adjoint", action="store_true",
                    help="skip the 512 x 512 plate's autograd gradient "
                         "(direct solves)")
    ap.add_argument("--batch", type=int, default=48)
    ap.add_argument("--batch-nmax", type=int, default=256)
    ap.add_argument("--batch-pc", type=int, default=0)
    ap.add_argument("--batch-fill", type=int, default=0,
                    help="ILU fill level of the batched solves")
    ap.add_argument("--batch-ilu", action="store_true",
                    help="batched solves by GMRES + ILU instead of the "
                         "complete factorisation")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from tacs_gb300 import problem
    p = c2_problem(n=args.size)
    M = problem.GpuModel(p)
    u = M.vec()
    res = M.vec()
    mat = M.new_mat()
    stream = torch.cuda.current_stream()

    def step():
        M.assemble_jacobian(u, mat, res)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    ms = replica_time(ms, dist, "cuda")

    # end to end through the public API with host buffers: design variables
    # and state in (pinned), residual out.
    thick_h = torch.as_tensor(np.asarray(p["thick"]), dtype=torch.float64).pin_memory()
    u_h = torch.zeros(M.ndof, dtype=torch.float64).pin_memory()
    res_h = torch.empty(M.ndof, dtype=torch.float64).pin_memory()
    dv_d = M.dv_vec()
    for _ in range(2):
        dv_d.copy_(thick_h, non_blocking=True)
        u.copy_(u_h, non_blocking=True)
        M.set_design_vars(dv_d)
        step()
        res_h.copy_(res, non_blocking=True)
    torch.cuda.synchronize()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    for _ in range(args.steps):
        dv_d.copy_(thick_h, non_blocking=True)
        u.copy_(u_h, non_blocking=True)
        M.set_design_vars(dv_d)
        step()
        res_h.copy_(res, non_blocking=True)
    e3.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e2.elapsed_time(e3) / args.steps

    nelem = p["nelem"]
    value = world * nelem / (ms / 1e3)
    peak, peak_src = measured_peaks()
    algo = algorithmic_bytes(p)
    # the step is kernels only: the colours' assembly launches (the first
    # writer of each block stores, so there is no zero fill) and the two
    # boundary-condition launches
    kern_ms = ms
    achieved = algo / (kern_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"MITC4 plate {args.size}x{args.size}, "
                               "assembleRes+assembleJacobian",
                   "elements": int(nelem), "nodes": int(p["nnodes"]),
                   "dof": int(M.ndof), "bcsr_blocks": int(mat.nnz),
                   "l2": "inputs larger than L2 (680 MB BCSR), no flush",
                   "colors": M.ncolors},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic_per_step(nelem),
                     "traffic_unit": "bytes per step (ncu, scaled)",
                     # the kernel's binding resource: ncu's
                     # sm__pipe_fp64_cycles_active on one colour launch
                     "fp64_pipe_active": SHELL_PROFILE["fp64_pipe_active"],
                     "carried_from_profile": {
                         "fields": ["traffic", "fp64_pipe_active",
                                    "fp64.executed_flops_per_element"],
                         "source": SHELL_PROFILE["source"]},
                     "peak_source": peak_src,
                     "kernel": "shell_team_assembly_kernel",
                     "kernel_ms": kern_ms, "algorithmic_bytes": algo,
                     "fp64": fp64_roofline("shell",
                                           nelem / (kern_ms / 1e3))},
        "e2e": {"value": world * nelem / (ms_e2e / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": int(8 * (M.ndv + M.ndof)),
                "d2h_bytes_per_step": int(8 * M.ndof)},
        "gpu_launches": M.ncolors * args.steps + 2 * args.steps,
        "clocks": clk,
    }
    padj = None
    if rank == 0:
        def shape_derivative():
            # node-coordinate total derivatives on the same plate at a
            # seeded state and adjoint (the kernels' cost does not depend
            # on the values)
            g = torch.Generator(device="cuda").manual_seed(7)
            us = 1e-4 * torch.randn(M.ndof, dtype=torch.float64,
                                    device="cuda", generator=g)
            ps = torch.randn(M.ndof, dtype=torch.float64, device="cuda",
                             generator=g)
            out = xpt_timing(M, {"u": us, "psis": [ps, ps]}, torch)
            out["workload"] = (f"MITC4 plate {args.size}x{args.size}: "
                               "df/dX - psi^T dR/dX of compliance and KS")
            return out
        line["shape_derivative"] = guarded(shape_derivative)
    if rank == 0 and args.adj_size > 0:
        res = guarded(lambda: adjoint_section(args.adj_size, torch))
        if isinstance(res, tuple):
            line["adjoint"], padj = res
        else:
            line["adjoint"] = res
    if rank == 0 and not args.no_fixed:
        line["fixed_geometry"] = guarded(lambda: fixed_geometry_section(
            torch, p, args.steps, f"MITC4 plate {args.size}x{args.size}, "
            "assembleRes+assembleJacobian with the fixed-geometry cache"))
        if not args.no_hex:
            from tacs_gb300 import meshes
            line["fixed_geometry_hex"] = guarded(
                lambda: fixed_geometry_section(
                    torch, meshes.hex_c3(), 5, "hex8 SIMP block 128x128x64, "
                    "assembleRes+assembleJacobian with the fixed-geometry "
                    "cache", bs=3))
    if rank == 0 and not args.no_hex:
        line["hex_c3"] = guarded(lambda: hex_section(torch))
    if rank == 0 and args.c3_solve:
        line["c3_solve"] = guarded(lambda: c3_solve_section(
            torch, pc_kind=args.c3_pc))
    if rank == 0 and not args.no_c3:
        line["c3_direct"] = guarded(lambda: c3_solve_section(
            torch, direct="mixed"))
    if rank == 0 and not args.no_c2_adjoint:
        line["c2_adjoint"] = guarded(
            lambda: c2_adjoint_section(torch, args.size))
    if rank == 0 and not args.no_cylinder:
        line["cylinder_c5"] = guarded(lambda: cylinder_section(torch))
    if rank == 0 and args.batch > 0:
        line["batch_c4"] = guarded(lambda: batch_section(
            torch, count=args.batch, nmax=args.batch_nmax,
            pc_kind=args.batch_pc, lev_fill=args.batch_fill,
            direct=not args.batch_ilu))
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = guarded(lambda: cpu_baseline(p))
        if padj is not None and "error" not in line["cpu_baseline"]:
            import oracle
            o = oracle.Oracle(padj, nthreads=os.cpu_count() or 1)
            t0 = time.perf_counter()
            r = o.static_adjoint(np.zeros(o.ndof), 100, 400, 1e-10)
            line["cpu_baseline"]["adjoint_s_per_gradient"] = \
                time.perf_counter() - t0
            line["cpu_baseline"]["adjoint_iters"] = r["iters"]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
