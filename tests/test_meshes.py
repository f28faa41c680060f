"""Host-side checks of the synthetic workload builders (no GPU)."""
import numpy as np

from tacs_gb300 import meshes


def test_concat_offsets_and_block_diagonal_connectivity():
    a = meshes.clamped_plate(3)
    b = meshes.clamped_plate(2)
    c = meshes.concat([a, b])
    assert c["nnodes"] == a["nnodes"] + b["nnodes"]
    assert c["nelem"] == a["nelem"] + b["nelem"]
    assert list(c["seg_node_ptr"]) == [0, 16, 25]
    assert list(c["seg_elem_ptr"]) == [0, 9, 13]
    conn = c["conn"].reshape(-1, 4)
    for g in range(2):
        e0, e1 = c["seg_elem_ptr"][g], c["seg_elem_ptr"][g + 1]
        n0, n1 = c["seg_node_ptr"][g], c["seg_node_ptr"][g + 1]
        assert conn[e0:e1].min() >= n0 and conn[e0:e1].max() < n1
    assert np.all(c["bc_nodes"][len(a["bc_nodes"]):] >= 16)
    assert np.all(c["pres_elems"][a["nelem"]:] >= 9)
    assert list(c["dvnum"]) == list(range(13))


def test_batch_plates_seeded_sizes_and_loads():
    b1 = meshes.batch_plates(count=48)
    b2 = meshes.batch_plates(count=48)
    n = b1["plate_n"]
    assert np.array_equal(n, b2["plate_n"])
    assert n.min() >= 16 and n.max() <= 256
    assert np.array_equal(b1["thick"], b2["thick"])
    assert b1["thick"].min() >= 0.004 and b1["thick"].max() <= 0.02
    pn = b1["point_nodes"]
    assert pn.shape == (48, 3)
    for g in range(48):
        lo, hi = b1["seg_node_ptr"][g], b1["seg_node_ptr"][g + 1]
        assert np.all((pn[g] >= lo) & (pn[g] < hi))
        assert len(set(pn[g])) == 3
        # interior nodes: not clamped
        assert not np.isin(pn[g], b1["bc_nodes"]).any()


def test_hex_c3_patch_and_clamp():
    p = meshes.hex_c3()
    assert p["nelem"] == 128 * 128 * 64
    assert p["nnodes"] == 129 * 129 * 65
    # |y - 1| <= 0.1 and |z - 0.5| <= 0.1 on a 1/64 x 1/64 face grid:
    # 12 x 12 face centroids
    assert len(p["trac_elems"]) == 144
    xyz = p["xpts"].reshape(-1, 3)
    assert np.all(xyz[p["bc_nodes"], 0] == 0.0)
    assert np.allclose(p["thick"], p["rho"] ** 3)


def test_cylinder_c5_loads():
    c = meshes.cylinder_c5(48, 16)
    f = c["force"].reshape(-1, 6)
    top = 48 * 16 + np.arange(48)
    assert np.allclose(f[top, 2], -1e5 * 2 * np.pi / 48)
    assert np.allclose(np.delete(f, top, axis=0), 0.0)
    assert len(c["bc_nodes"]) == 48 and np.all(c["bc_masks"] == 0x3F)
