"""Build tests/golden/known/plate_bdf.npz: the reference's 100-element plate
model (tests/integration_tests/input_files/plate.bdf of the reference) read
by tacs_gb300.bdf.read_bdf, with the element data of the reference test's
call-back (tests/integration_tests/test_shell_plate_quad.py:96-116:
t = 0.005, E = 70e9, nu = 0.3, rho = 2500, ys = 464e6), and the known
answers that test pins for the 100 kPa pressure and the 10 kN point force
at GRID 81 with KS weight 10 (test_shell_plate_quad.py:37-38, 51-52).

    python tests/golden/make_bdf_golden.py <path to tacs>
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tacs_gb300 import bdf  # noqa: E402

KNOWN = {  # test_shell_plate_quad.py FUNC_REFS
    "pressure_compliance": 4679.345460332448,
    "pressure_ks_vmfailure": 1.2938623156883402,
    "point_load_compliance": 683.8571611645635,
    "point_load_ks_vmfailure": 0.5757488025912149,
}


def main(ref_root):
    path = os.path.join(ref_root, "tests", "integration_tests", "input_files",
                        "plate.bdf")
    p = bdf.read_bdf(path, thickness=0.005, E=70e9, nu=0.3, rho=2500.0,
                     ys=464e6)
    k = int(np.nonzero(p["grid_ids"] == 81)[0][0])
    point = np.zeros(6 * p["nnodes"])
    point[6 * k + 2] = 1e4
    out = {f"in_{key}": np.asarray(p[key]) for key in (
        "xpts", "conn", "thick", "dvnum", "mat", "bc_nodes", "bc_masks",
        "grid_ids", "elem_ids")}
    out["in_nnodes"] = np.asarray(p["nnodes"])
    out["in_nelem"] = np.asarray(p["nelem"])
    out["in_point_force"] = point
    for key, v in KNOWN.items():
        out[f"ref_{key}"] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "known", "plate_bdf.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1])
