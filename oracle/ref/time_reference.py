"""Times the reference TACS library on this machine's host cores against the
oracle port on the same problems -- test infrastructure, run where the
reference sources are (it needs oracle/_ref built from them):

    make -C oracle/ref REF=<path to tacs> OPT=-O3 OUT=$PWD/oracle/_ref/o3
    python oracle/ref/time_reference.py [--full]

Problems: the bench's 512 x 512 plate workload sampled as its 128 x 128
sub-plate (bench.c2_problem; --full adds the whole 512 x 512 plate) and the
bench's 64 x 64 clamped adjoint plate for the node-coordinate products.
Each reference call is timed by oracle/ref/ref_bench.cpp (best of 3 after a
warm-up, 1 thread and all threads); the port's assembly by the oracle with
the same thread counts.  The ratio of the two on the same cores is what
turns the port's number on another machine (the bench's cpu_baseline)
into an estimate of the reference there.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

import bench  # noqa: E402
import oracle  # noqa: E402
from make_golden import write_tgarr  # noqa: E402


def ref_bench_exe():
    for sub in ("o3", "."):
        exe = os.path.join(ROOT, "oracle", "_ref", sub, "ref_bench")
        if os.path.exists(exe):
            return exe, sub
    raise SystemExit("build oracle/_ref first (oracle/ref/Makefile)")


def run_ref(exe, prob, threads, reps=3, xpt=False):
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "p.bin")
        write_tgarr(path, prob)
        cmd = [exe, path, str(threads), str(reps)] + (["xpt"] if xpt else [])
        out = subprocess.run(cmd, check=True, capture_output=True, text=True)
    return json.loads(out.stdout.strip().splitlines()[-1])


def run_port(prob, threads, reps=3):
    o = oracle.Oracle(prob, nthreads=threads)
    u = np.zeros(o.ndof)
    A = o.new_bcsr()
    o.assemble_jac(u, A)
    best = 1e30
    for _ in range(reps):
        t0 = time.perf_counter()
        o.assemble_jac(u, A)
        best = min(best, time.perf_counter() - t0)
    o.free(A)
    return {"threads": threads, "assemble_jacobian_ms": 1e3 * best,
            "elements_per_s": prob["nelem"] / best}


def main():
    exe, build = ref_bench_exe()
    nproc = os.cpu_count() or 1
    cases = [("plate 128x128 (bench sample)",
              bench.c2_problem(n=128, L=0.5, seed=2))]
    if "--full" in sys.argv:
        cases.append(("plate 512x512 (bench workload)", bench.c2_problem()))
    report = {"host_cores": nproc, "reference_build": build, "cases": []}
    for label, prob in cases:
        for th in sorted({1, nproc}):
            r = run_ref(exe, prob, th)
            q = run_port(prob, th)
            report["cases"].append({
                "case": label, "threads": th,
                "reference_elements_per_s": r["elements_per_s"],
                "reference_res_ms": r["assemble_res_ms"],
                "port_elements_per_s": q["elements_per_s"],
                "reference_over_port": r["elements_per_s"]
                / q["elements_per_s"]})
            print(json.dumps(report["cases"][-1]), flush=True)
    r = run_ref(exe, bench.clamped_plate(64), 1, reps=1, xpt=True)
    report["xpt_64x64"] = {k: r[k] for k in ("add_xpt_sens_ms",
                                             "add_adjoint_res_xpt_ms")}
    print(json.dumps(report["xpt_64x64"]), flush=True)
    print(json.dumps(report))


if __name__ == "__main__":
    main()
