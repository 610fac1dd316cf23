"""Golden vectors taken from the reference's own tests and code (tests/golden/make_golden.py)."""
import os

import numpy as np

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_convert_triangles_golden():
    """receive_horn.ply -> triangle records (lyceanem/tests/test_ray_functions.py:9-24)."""
    from lyceanem_gb300.geometry import read_ply, triangles_of
    d = np.load(os.path.join(GOLD, "convert_triangles.npz"))
    mesh = read_ply(d["ply"].tobytes())
    v, f = triangles_of(mesh)
    got = np.concatenate([v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]], axis=1)
    assert got.shape == d["triangles"].shape
    assert np.array_equal(got, d["triangles"])
    # the oracle's packing keeps v0 and forms the FP32 edges from the same vertices
    t = O.pack_triangles(v, f)
    assert np.array_equal(t[:, 0:3], d["triangles"][:, 0:3])
    assert np.array_equal(t[:, 4:7], d["triangles"][:, 3:6] - d["triangles"][:, 0:3])


def test_vector_mapping_golden():
    """Known answers of lyceanem/tests/test_empropagation.py:8-95."""
    from lyceanem_gb300.geometry import vector_mapping
    d = np.load(os.path.join(GOLD, "vector_mapping.npz"))
    for i in range(len(d["names"])):
        got = vector_mapping(d["desired"][i], d["normal"][i], d["rotation"][i])
        np.testing.assert_allclose(got, d["expected"][i], atol=1e-12, err_msg=str(d["names"][i]))


def test_tile_structure_geometry_golden():
    """Bounds / tile size / cell counts of Tile_acceleration_structure.__init__."""
    from lyceanem_gb300.models.acceleration_structures import tile_geometry
    d = np.load(os.path.join(GOLD, "tile_structure.npz"))
    keys = ["max_x", "min_x", "max_y", "min_y", "max_z", "min_z", "tile_size", "y_cells_count", "z_cells_count"]
    for pts, n_cells, vals in zip(d["points"], d["n_cells"], d["values"]):
        g = tile_geometry(pts, int(n_cells))
        got = np.array([g[k] for k in keys], np.float64)
        assert np.array_equal(got, vals), (got, vals)
