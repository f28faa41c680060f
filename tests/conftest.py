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
