"""Acceleration structures with the interface of lyceanem/models/acceleration_structures.py.

Tile_acceleration_structure(blocking_mesh, n_cells) keeps the reference's
attributes (bounds with the 0.1 % margin, tile_size, y/z cell counts,
bin_counts, binned_triangles from the y-z binning) and adds a device-resident
uniform 3-D grid that the traversal actually uses; it is built once and reused
by every calculate_scattering call.  Brute_Force_acceleration_structure keeps
the packed triangles on the device.

calculate_scattering(source_mesh, sink_mesh, alpha, beta, wavelength,
self_to_self, chunk_count=1) returns the complex64 [N, M, 3] network like the
reference (lyceanem/models/acceleration_structures.py:72-115).
sink_field(...) returns the source-summed complex64 [M, 3] field without
forming the network.
"""
import collections
import hashlib

import numpy as np
import torch

from .. import em as _em
from .. import propagation as P
from ..geometry import triangles_of


def _cvec_from_point_data(mesh):
    pd = mesh.point_data
    return np.stack([np.asarray(pd["ex"]), np.asarray(pd["ey"]), np.asarray(pd["ez"])], axis=1).astype(np.complex64)


def _chunks(n, chunk_count):
    """Source ranges of the reference's chunk loop (acceleration_structures.py:74-113)."""
    assert chunk_count > 0, "chunk_count must be greater than 0"
    out, start, step = [], 0, int(np.floor(n / chunk_count))
    end = step
    for i in range(chunk_count):
        if i == chunk_count - 1:
            end = n
        out.append((start, end))
        start = end
        end = end + step
    return [(a, b) for a, b in out if b > a]


def tile_geometry(points, n_cells):
    """Bounds (0.1 % margin on each bound's magnitude), tile size and y/z cell
    counts of the reference's tile structure (acceleration_structures.py:55-68)."""
    pts = np.asarray(points)
    mx, mn = np.max(pts, axis=0), np.min(pts, axis=0)
    g = {}
    for k, ax in enumerate("xyz"):
        g["max_" + ax] = mx[k] + abs(mx[k] * 0.001)
        g["min_" + ax] = mn[k] - abs(mn[k] * 0.001)
    diff_y = g["max_y"] - g["min_y"]
    diff_z = g["max_z"] - g["min_z"]
    g["tile_size"] = min(diff_y, diff_z) / n_cells
    g["y_cells_count"] = int(np.ceil(diff_y / g["tile_size"]))
    g["z_cells_count"] = int(np.ceil(diff_z / g["tile_size"]))
    return g


def em_float(x):
    """A scalar as the reference's compiled em module receives it: its bindings take alpha and beta as
    C++ float (lyceanem/src/frequency_domain_models.cu:44-47, 190-195), so they arrive rounded to float32."""
    return float(np.float32(x))


class _DeviceScene:
    """Packed triangles on the device plus an optional uniform grid."""

    def __init__(self, vertices, faces, grid_cell=None, use_grid=True):
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float32)
        self.faces = np.ascontiguousarray(faces, dtype=np.int32)
        if self.faces.shape[0]:
            self.tris = P.pack_triangles(torch.from_numpy(self.vertices), torch.from_numpy(self.faces))
        else:
            self.tris = torch.zeros((0, 12), dtype=torch.float32, device="cuda")
        self.grid = P.UniformGrid(self.tris, cell=grid_cell) if (use_grid and self.faces.shape[0]) else None

    def stage(self, src, E, snk, snk_n, alpha, beta, self_to_self, **kw):
        return P.pair_stage(src, E, snk, snk_n, beta=beta, alpha=alpha, tris=self.tris, grid=self.grid,
                            self_to_self=self_to_self, **kw)

    def network(self, source_mesh, sink_mesh, alpha, beta, self_to_self, chunk_count):
        src = np.asarray(source_mesh.points, dtype=np.float32)
        snk = torch.as_tensor(np.asarray(sink_mesh.points, dtype=np.float32)).cuda()
        snk_n = torch.as_tensor(np.asarray(sink_mesh.point_data["Normals"], dtype=np.float32)).cuda()
        E = _cvec_from_point_data(source_mesh)
        out = np.zeros((src.shape[0], snk.shape[0], 3), dtype=np.complex64)
        for a, b in _chunks(src.shape[0], chunk_count):
            r = self.stage(src[a:b], E[a:b], snk, snk_n, alpha, beta, self_to_self, want_pairs=True)
            out[a:b] = r.pairs.cpu().numpy()
        return out

    def sink_field(self, source_mesh, sink_mesh, alpha, beta, self_to_self=False):
        src = np.asarray(source_mesh.points, dtype=np.float32)
        snk = np.asarray(sink_mesh.points, dtype=np.float32)
        snk_n = np.asarray(sink_mesh.point_data["Normals"], dtype=np.float32)
        r = self.stage(src, _cvec_from_point_data(source_mesh), snk, snk_n, alpha, beta, self_to_self)
        return r.sink.cpu().numpy()


class Tile_acceleration_structure:
    """Tile structure of the reference (y-z bins over an x slab) plus this package's 3-D grid.

    grid_cell: edge of the traversal grid's cubic cells in metres (None picks
    about one cell per triangle; the reference's tile_size is kept only as an
    attribute because the traversal result does not depend on the cells)."""

    def __init__(self, blocking_mesh, n_cells, grid_cell=None):
        pts = np.asarray(blocking_mesh.points)
        self.triangle_verticies = np.ascontiguousarray(pts)
        self.__dict__.update(tile_geometry(pts, n_cells))
        verts, faces = triangles_of(blocking_mesh)
        self.bin_counts = _em.bin_counts_to_numpy(pts, faces, self.y_cells_count, self.z_cells_count, self.min_y,
                                                  self.tile_size, self.min_z)
        self.binned_triangles_count = int(np.sum(self.bin_counts))
        self.binned_triangles = _em.bin_triangles_to_numpy(pts, faces, self.y_cells_count, self.z_cells_count,
                                                           self.min_y, self.tile_size, self.min_z, self.bin_counts,
                                                           self.binned_triangles_count)
        self.device = _DeviceScene(verts, faces, grid_cell=grid_cell, use_grid=True)

    def calculate_scattering(self, source_mesh, sink_mesh, alpha, beta, wavelength, self_to_self, chunk_count=1):
        del wavelength  # unused by the field formula, as in the reference
        alpha, beta = em_float(alpha), em_float(beta)
        return self.device.network(source_mesh, sink_mesh, alpha, beta, self_to_self, chunk_count)

    def sink_field(self, source_mesh, sink_mesh, alpha, beta, wavelength=None, self_to_self=False):
        return self.device.sink_field(source_mesh, sink_mesh, alpha, beta, self_to_self)


# Scene cache: the last few tile structures, keyed by a fingerprint of the geometry and the grid
# cell, so that repeated model calls on the same solid reuse its device triangles and grid.
_CACHE = collections.OrderedDict()
CACHE_SIZE = 4
cache_stats = {"hits": 0, "misses": 0}


def clear_cache():
    """Drops every cached structure (the next model call uploads and grids its solid again)."""
    _CACHE.clear()


def cached_structure(verts, faces, grid_cell=None):
    """Tile_acceleration_structure of (verts, faces) from the scene cache, built on a miss."""
    v = np.ascontiguousarray(verts, dtype=np.float32)
    f = np.ascontiguousarray(faces, dtype=np.int32)
    h = hashlib.sha1()
    h.update(v.tobytes())
    h.update(f.tobytes())
    key = (h.hexdigest(), v.shape, f.shape, None if grid_cell is None else float(grid_cell),
           torch.cuda.current_device())
    if key in _CACHE:
        cache_stats["hits"] += 1
        _CACHE.move_to_end(key)
        return _CACHE[key]
    cache_stats["misses"] += 1
    from ..geometry import Mesh
    acc = Tile_acceleration_structure(Mesh(v, [("triangle", f)]), 1, grid_cell=grid_cell)
    _CACHE[key] = acc
    while len(_CACHE) > CACHE_SIZE:
        _CACHE.popitem(last=False)
    return acc


class Brute_Force_acceleration_structure:
    """Brute-force structure of the reference; calculate_scattering returns the network
    (the reference's binding leaves it on the device, frequency_domain_models.cu:159-171)."""

    def __init__(self, blocking_mesh):
        self.triangle_verticies = np.ascontiguousarray(np.asarray(blocking_mesh.points))
        verts, faces = triangles_of(blocking_mesh)
        self.triangles = faces
        self.device = _DeviceScene(verts, faces, use_grid=False)

    def calculate_scattering(self, source_mesh, sink_mesh, alpha, beta, wavelength, self_to_self, chunk_count=1):
        del wavelength
        alpha, beta = em_float(alpha), em_float(beta)
        return self.device.network(source_mesh, sink_mesh, alpha, beta, self_to_self, chunk_count)

    def sink_field(self, source_mesh, sink_mesh, alpha, beta, wavelength=None, self_to_self=False):
        return self.device.sink_field(source_mesh, sink_mesh, alpha, beta, self_to_self)
