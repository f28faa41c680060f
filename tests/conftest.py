"""Shared test helpers.  GPU tests are marked ``gpu``; everything else runs on
the CPU (the oracle against the golden fixtures, host logic, the C-ABI
library's exports)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
CASES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line(
        "markers", "direct: uses the direct (multifrontal) factorisation")
    config.addinivalue_line(
        "markers", "late: a newer kernel, run after the established tests")


def _late(item):
    return bool(item.get_closest_marker("direct")
                or item.get_closest_marker("late"))


def _last(item):
    return os.path.basename(str(item.fspath)) == "test_zz_no_alloc.py"


def pytest_collection_modifyitems(session, config, items):
    """Tests of the direct factorisation and of other newer kernels run
    after the others (stable order otherwise): the established parity tests
    come first, so that under -x a failure in a newer path cannot stop
    them.  The allocation-free entry point's tests run last of all."""
    items[:] = ([i for i in items if not _late(i) and not _last(i)]
                + [i for i in items if _late(i) and not _last(i)]
                + [i for i in items if _last(i)])


def load_case(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    prob = {k[3:]: d[k] for k in d.files if k.startswith("in_")}
    for k in ("elem_type", "nnodes", "nelem", "transform", "gmres_m",
              "gmres_restart"):
        if k in prob:
            prob[k] = int(prob[k])
    for k in ("ks_weight", "rtol"):
        if k in prob:
            prob[k] = float(prob[k])
    ref = {k[4:]: d[k] for k in d.files if k.startswith("ref_")}
    return prob, ref


def rel(a, b):
    """Norm-wise relative difference max|a-b| / max|b|."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.max(np.abs(b)) if b.size else 0.0
    return float(np.max(np.abs(a - b)) / den) if den > 0 else float(
        np.max(np.abs(a - b)) if a.size else 0.0)


def exact_solve(K, b, prob, spec="COLAMD"):
    """Sparse direct solution on the host for checking: the constrained
    dofs (prob's bc_nodes / bc_masks) are removed, the remaining symmetric
    positive definite matrix is scaled to a unit diagonal and factored in
    SuperLU's symmetric mode without pivoting (elimination order `spec`).
    The row-zeroed, unit-diagonal constraint rows of the assembled matrix
    mix entries of 1 with stiffnesses of 1e9 and more; a pivoting LU of that
    matrix loses digits the problem itself does not lose (two elimination
    orders then differ by 1e-5 on thin shells, against 1e-11 here).
    Returns x with zeros in the constrained dofs."""
    from scipy import sparse
    from scipy.sparse.linalg import splu
    vpn = 6 if int(prob["elem_type"]) == 0 else 3
    fixed = np.zeros(K.shape[0], bool)
    for node, mask in zip(prob["bc_nodes"], prob["bc_masks"]):
        for k in range(vpn):
            if (int(mask) >> k) & 1:
                fixed[vpn * int(node) + k] = True
    free = np.nonzero(~fixed)[0]
    K = sparse.csr_matrix(K)
    Kr = K[free][:, free].tocsc()
    d = 1.0 / np.sqrt(Kr.diagonal())
    S = sparse.diags(d)
    lu = splu((S @ Kr @ S).tocsc(), permc_spec=spec, diag_pivot_thresh=0.0,
              options=dict(SymmetricMode=True))
    x = np.zeros(K.shape[0])
    x[free] = d * lu.solve(d * np.asarray(b)[free])
    return x


def exact_and_spread(K, b, prob):
    """exact_solve and its rounding spread: the relative distance between
    the solutions of two elimination orders, for the solution (max norm)
    and for the compliance b^T x."""
    x1 = exact_solve(K, b, prob, "COLAMD")
    x2 = exact_solve(K, b, prob, "MMD_ATA")
    return x1, rel(x2, x1), abs(b @ x2 - b @ x1) / abs(b @ x1)

