"""Host-side logic on CPU: scene recipes, chunking, steering weights, sink grids."""
import numpy as np
import pytest

from lyceanem_gb300 import scenes


def test_direct_scene_shapes():
    s = scenes.direct_scene()
    assert s.src.shape == (64, 3) and s.snk.shape == (2664, 3) and s.faces.shape == (1024, 3)
    assert np.allclose(np.linalg.norm(s.snk, axis=1), 10.0, rtol=1e-6)
    assert np.allclose(s.snk_n, -s.snk / 10.0, atol=1e-6)
    c = s.verts.reshape(-1, 3, 3).mean(axis=1)
    assert c[:, :2].min() > -1.06 and c[:, :2].max() < 1.06 and c[:, 2].min() > 0.44 and c[:, 2].max() < 1.56
    pitch = np.diff(np.unique(s.src[:, 0]))
    assert np.allclose(pitch, 0.029979 / 2, rtol=1e-5)


def test_bounce_scene_shapes():
    s = scenes.bounce_scene()
    assert s.src.shape == (1024, 3)
    assert s.faces.shape == (120000, 3)
    assert s.scat.shape == (50000, 3)
    assert s.snk.shape == (65341, 3)
    assert np.isclose(s.wavelength, 299792458.0 / 28e9)
    # ground triangles face +z
    v = s.verts.astype(np.float64)
    f = s.faces[:80000]
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    assert (n[:, 2] > 0).all()


def test_chunks_follow_reference_loop():
    from lyceanem_gb300.models.acceleration_structures import _chunks
    assert _chunks(10, 1) == [(0, 10)]
    assert _chunks(10, 3) == [(0, 3), (3, 6), (6, 10)]
    assert _chunks(7, 7) == [(i, i + 1) for i in range(7)]


def test_steering_weights_match_far_point_formula():
    """WavefrontWeights (beamforming.py:81-120): phase k (|p - 1e9 s| - min)."""
    rng = np.random.default_rng(0)
    src, _ = scenes.planar_array(8, 8, 0.0107)
    d = rng.normal(size=(5, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    W = scenes.steering_weights(src, d, 0.0107)
    for k in range(5):
        far = d[k] * 1e9
        dist = np.sqrt(((src.astype(np.float64) - far) ** 2).sum(axis=1))
        ref = np.exp(1j * 2 * np.pi / 0.0107 * (dist - dist.min()))
        assert np.abs(W[k] - ref).max() < 2e-3   # the 1e9 far point itself costs ~1e-7 m of path
    assert np.allclose(np.abs(W), 1.0)


def test_spherical_field():
    from lyceanem_gb300.geometry import spherical_field
    m = spherical_field(np.linspace(-180, 180, 7), np.linspace(-90, 90, 5), field_radius=3.0)
    assert m.points.shape == (35, 3)
    assert np.allclose(np.linalg.norm(m.points, axis=1), 3.0, rtol=1e-6)
    assert np.allclose(m.point_data["Normals"] * 3.0, -m.points, atol=1e-5)
    th = m.point_data["theta_(Radians)"]
    assert np.allclose(np.cos(th) * 3.0, m.points[:, 2], atol=1e-5)


def test_sweep_and_batched_recipes_small():
    s = scenes.sweep_scene(n_side=8, n_clutter=100, n_beams=16, el_n=5, az_n=7, n_ground=10)
    assert s.weights.shape == (16, 64) and s.faces.shape == (200 + 100, 3)
    assert (s.directions[:, 2] >= 0).all()
    sc, snk, snk_n, freqs = scenes.batched_scenes(n_scenes=3, elem_range=(16, 64), tri_range=(1000, 2000),
                                                  n_sinks=100, n_freqs=4)
    assert len(sc) == 3 and snk.shape == (100, 3) and freqs.shape == (4,)
    for s in sc:
        assert 900 <= s.faces.shape[0] <= 2100


def _stl_bytes_binary(tri, normals):
    import struct
    out = bytearray(b"\0" * 80) + struct.pack("<I", tri.shape[0])
    for t, n in zip(tri, normals):
        out += struct.pack("<12fH", *n, *t.ravel(), 0)
    return bytes(out)


def _stl_bytes_ascii(tri, normals):
    lines = ["solid test"]
    for t, n in zip(tri, normals):
        lines.append(f"facet normal {n[0]:.9g} {n[1]:.9g} {n[2]:.9g}")
        lines.append("outer loop")
        lines += [f"vertex {v[0]:.9g} {v[1]:.9g} {v[2]:.9g}" for v in t]
        lines += ["endloop", "endfacet"]
    lines.append("endsolid test")
    return "\n".join(lines).encode()


def test_read_stl_binary_and_ascii():
    """STL scenes (the format of the reference's test scenes) read to the same triangles either way."""
    from lyceanem_gb300.geometry import read_stl, triangles_of
    rng = np.random.default_rng(0)
    # a closed cube (shared vertices) plus a few loose triangles
    c = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], np.float32)
    f = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4], [1, 2, 6], [1, 6, 5],
                  [2, 3, 7], [2, 7, 6], [3, 0, 4], [3, 4, 7]])
    tri = np.concatenate([c[f], rng.uniform(-1, 1, (5, 3, 3)).astype(np.float32)])
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]).astype(np.float32)
    for raw in (_stl_bytes_binary(tri, nrm), _stl_bytes_ascii(tri, nrm)):
        m = read_stl(raw)
        v, fc = triangles_of(m)
        assert fc.shape == (tri.shape[0], 3)
        assert np.allclose(v[fc], tri, atol=1e-6)
        assert np.allclose(m.cell_data["Normals"][0], nrm, atol=1e-5)
        assert v.shape[0] == 8 + 15  # cube vertices shared, loose triangles' vertices distinct


def test_mesh_conversion_records():
    """mesh_conversion of a mesh, a list and a structures-like object (geometryfunctions.py:473-510)."""
    from lyceanem_gb300.geometry import Mesh, mesh_conversion
    rng = np.random.default_rng(1)
    a = Mesh(rng.normal(size=(6, 3)), [("triangle", [[0, 1, 2], [3, 4, 5]])])
    b = Mesh(rng.normal(size=(3, 3)), [("triangle", [[0, 1, 2]])])
    ra, rb = mesh_conversion(a), mesh_conversion(b)
    assert ra.shape == (2,) and np.isclose(ra["v1y"][1], np.float32(a.points[4, 1]))
    both = mesh_conversion([a, b])
    assert both.shape == (3,) and np.array_equal(both[2:], rb)

    class Structures:
        def triangles_base_raycaster(self):
            return mesh_conversion([a, b])

    assert np.array_equal(mesh_conversion(Structures()), both)
    assert mesh_conversion(object()).shape == (0,)


@pytest.mark.parametrize("limit_div,spread", [(1.0, 1e-12), (3.5, 1e-12), (3.5, 3e-9), (7.2, 3e-9)])
def test_time_map_source_chunks_vs_oracle(limit_div, spread):
    """Wake times of the time map, single and split into source chunks (TimeDomainv3 splits a float64 map of
    more than 1e9 bytes; here the limit is lowered to split a small map), against the oracle's loop over the
    reference's chunk sequence: chunk wakes within one sample (no shift) and chunks whose wakes differ by
    several samples (shifted into alignment).  Host-side: the map is built from CPU tensors."""
    import torch

    from lyceanem_gb300.empropagation import time_map
    from oracle import oracle as O
    rng = np.random.default_rng(int(limit_div * 10))
    n_src, n_snk, S, R = 9, 5, 300, 400
    pair = np.stack([rng.integers(0, n_src, R), rng.integers(0, n_snk, R)], 1).astype(np.int32)
    # later sources arrive earlier by up to `spread` seconds, so the chunks' wakes differ
    arrival = 3e-8 + rng.uniform(0, 2e-9, R) - spread * pair[:, 0] / n_src
    amp = rng.normal(size=(R, 3))
    exc = np.sin(np.linspace(0, 5 * np.pi, 30))
    limit = n_src * n_snk * S * 3 * 8 / limit_div
    fs = 20e9
    tm, wake = time_map(torch.from_numpy(amp), torch.from_numpy(arrival), torch.from_numpy(pair), n_src, n_snk, exc,
                        fs, S, map_bytes_limit=limit)
    otm, owake = O.time_map(amp, arrival, pair, n_src, n_snk, exc, fs, S, map_bytes_limit=limit)
    assert wake == owake
    assert np.abs(tm.numpy() - otm).max() <= 1e-12 * np.abs(otm).max()
