"""Numba-engine raycasting entry points with the call shape of lyceanem/raycasting/rayfunctions.py.

The reference's numba engine casts one ray per (origin, target) pair on the
GPU through numba (hit without back-face culling, EPSILON 1e-7,
lyceanem/raycasting/rayfunctions.py:19, 37-104) and lists the unblocked paths
as rows of 1-based indices into [sources, sinks, scatter points].  Here the
visibility comes from this package's kernels (the same test in the cull = 0
mode, every pair tested) and the rows are assembled on the device.
"""
import numpy as np
import torch

from . import propagation as P

# triangle_t of lyceanem/base_types.py (numpy record layout, no numba needed)
triangle_t = np.dtype([(f"v{i}{c}", "f4") for i in range(3) for c in "xyz"], align=True)


def convertTriangles(triangle_object):
    """meshio-like mesh (points + a "triangle" cell block) -> triangle_t records
    (lyceanem/raycasting/rayfunctions.py:531-557)."""
    if triangle_object is None:
        return np.empty(0, dtype=triangle_t)
    from .geometry import triangles_of
    verts, faces = triangles_of(triangle_object)
    v = np.asarray(verts)[np.asarray(faces)].astype(np.float32)  # [T, 3, 3]
    out = np.empty(v.shape[0], dtype=triangle_t)
    for i in range(3):
        for k, c in enumerate("xyz"):
            out[f"v{i}{c}"] = v[:, i, k]
    return out


def _packed(environment):
    """triangle_t records, (verts, faces), or packed [T, 12] -> packed device triangles."""
    if isinstance(environment, tuple):
        return P.pack_triangles(environment[0], environment[1])
    env = np.asarray(environment) if not isinstance(environment, torch.Tensor) else environment
    if isinstance(env, np.ndarray) and env.dtype.names:
        v = np.stack([np.stack([env[f"v{i}{c}"] for c in "xyz"], 1) for i in range(3)], 1).astype(np.float32)
        verts = v.reshape(-1, 3)
        faces = np.arange(verts.shape[0], dtype=np.int32).reshape(-1, 3)
        return P.pack_triangles(verts, faces)
    return P._dev(env, torch.float32).reshape(-1, 12).contiguous()


def numba_masks(sources, sinks, scattering_points, environment, need_scatter_scatter=False, grid_cell=None):
    """Device visibility (bool tensors) of the numba engine's ray sets: sources->sinks,
    sources->scatter, scatter->sinks and (optionally) scatter->scatter."""
    tris = _packed(environment)
    src, snk, scat = P._points(sources), P._points(sinks), P._points(scattering_points)
    kw = dict(beta=1.0, self_to_self=True, cull=False, eps=P.NUMBA_EPSILON, want_mask=True)
    if tris.shape[0]:
        kw["grid"] = P.UniformGrid(tris, cell=grid_cell)
    else:
        kw["tris"] = tris
    ones = lambda n: torch.ones((n, 3), dtype=torch.complex64, device=src.device)  # noqa: E731
    z = lambda a, b: torch.zeros((a, b), dtype=torch.bool, device=src.device)  # noqa: E731
    N, M, Pn = src.shape[0], snk.shape[0], scat.shape[0]
    nrm = lambda n: torch.ones((n, 3), dtype=torch.float32, device=src.device)  # noqa: E731
    m0 = P.pair_stage(src, ones(N), snk, nrm(M), **kw).mask() if N and M else z(N, M)
    m1 = P.pair_stage(src, ones(N), scat, nrm(Pn), **kw).mask() if N and Pn else z(N, Pn)
    m2 = P.pair_stage(scat, ones(Pn), snk, nrm(M), **kw).mask() if Pn and M else z(Pn, M)
    m3 = None
    if need_scatter_scatter:
        m3 = P.pair_stage(scat, ones(Pn), scat, nrm(Pn), **kw).mask() if Pn else z(0, 0)
    return m0, m1, m2, m3


def workchunkingv2(sources, sinks, scattering_points, environment, max_scatter, line_of_sight=True):
    """(full_index, RAYS_CAST) of lyceanem/raycasting/rayfunctions.py:2681-2955.

    full_index rows are 1-based indices into [sources, sinks, scatter points]:
    max_scatter 1: [n, m]; 2: [n, m, 0] then [n, p, m]; 3: per source chunk
    [n, m, 0, 0], [n, p, m, 0], [n, p, q, m] (q != p).  Rows follow the
    reference's order (its extra splitting when the rays exceed 80 % of the
    GPU memory is not reproduced; that only regroups rows).  RAYS_CAST counts
    the rays cast as the reference does (for max_scatter 3, the last source
    chunk's count, as the reference overwrites it per chunk)."""
    src = P._points(sources)
    snk = P._points(sinks)
    scat = P._points(scattering_points) if scattering_points is not None else P._points(np.zeros((0, 3)))
    N, M, Pn = src.shape[0], snk.shape[0], scat.shape[0]
    m0, m1, m2, m3 = numba_masks(src, snk, scat, environment, need_scatter_scatter=(max_scatter == 3))
    dev = src.device
    snk0, sc0 = N + 1, N + M + 1
    if max_scatter == 1:
        nm = torch.nonzero(m0)
        out = torch.stack([nm[:, 0] + 1, nm[:, 1] + snk0], 1)
        return out.to(torch.int32).cpu().numpy(), N * (M + Pn)
    if max_scatter == 2:
        rows = []
        if line_of_sight:
            nm = torch.nonzero(m0)
            rows.append(torch.stack([nm[:, 0] + 1, nm[:, 1] + snk0, torch.zeros_like(nm[:, 0])], 1))
        np_ = torch.nonzero(m1)
        km = torch.nonzero(m2[np_[:, 1]])
        rows.append(torch.stack([np_[km[:, 0], 0] + 1, np_[km[:, 0], 1] + sc0, km[:, 1] + snk0], 1))
        rays = N * ((M if line_of_sight else 0) + Pn) + np_.shape[0] * M
        out = torch.cat(rows, 0) if rows else torch.zeros((0, 3), dtype=torch.int64, device=dev)
        return out.to(torch.int32).cpu().numpy().reshape(-1, 3), rays
    if max_scatter != 3:
        raise ValueError("max_scatter must be 1, 2 or 3")
    ray_estimate = N * (M + Pn) + N * (Pn * M * max_scatter)
    chunknum = max(2, min(N, int(np.ceil(ray_estimate / 2e8))))
    bounds = np.linspace(0, N, chunknum, dtype=np.int32)
    out, rays = [], 0
    eye = torch.eye(Pn, dtype=torch.bool, device=dev)
    m3 = m3 & ~eye
    for c in range(bounds.size - 1):
        s0, s1 = int(bounds[c]), int(bounds[c + 1])
        rows = []
        if line_of_sight:
            nm = torch.nonzero(m0[s0:s1])
            z = torch.zeros_like(nm[:, 0])
            rows.append(torch.stack([nm[:, 0] + s0 + 1, nm[:, 1] + snk0, z, z], 1))
        np_ = torch.nonzero(m1[s0:s1])
        n1, p1 = np_[:, 0] + s0, np_[:, 1]
        km = torch.nonzero(m2[p1])
        rows.append(torch.stack([n1[km[:, 0]] + 1, p1[km[:, 0]] + sc0, km[:, 1] + snk0, torch.zeros_like(km[:, 0])], 1))
        kq = torch.nonzero(m3[p1])
        n2, p2, q2 = n1[kq[:, 0]], p1[kq[:, 0]], kq[:, 1]
        k3 = torch.nonzero(m2[q2])
        rows.append(torch.stack([n2[k3[:, 0]] + 1, p2[k3[:, 0]] + sc0, q2[k3[:, 0]] + sc0, k3[:, 1] + snk0], 1))
        out.append(torch.cat(rows, 0))
        rays = (s1 - s0) * ((M if line_of_sight else 0) + Pn) + n1.shape[0] * (M + Pn - 1) + n2.shape[0] * M
    return torch.cat(out, 0).to(torch.int32).cpu().numpy().reshape(-1, 4), rays


def visiblespace(source_coords, source_normals, environment, vertex_area=0, az_range=None, elev_range=None,
                 shell_range=0.5):
    """(visible_patterns float32 [len(elev_range), len(az_range)], sample_shell) of
    lyceanem/raycasting/rayfunctions.py:316-427: for each point of a shell of radius shell_range
    (spherical_field, outward normals), the summed projected area of the sources that see it.

    A source n sees shell point m when the numba engine's ray n -> m is unblocked (workchunkingv2 with
    max_scatter 1, this package's kernels); it contributes area_n |cos angle| where angle is the angle
    between the ray direction and the source normal (unit vectors, float32 as the reference), and nothing
    when the angle exceeds pi / 2.  vertex_area: one value per source, or a single value (0, the default,
    counts every visible pair as 1); NaN areas count as 0 (the reference sets them to 0 in the caller's
    array and raises for a plain scalar; here the caller's array is left as it is and a scalar is taken
    as a single value).  The angle's sign, which the reference takes from a 2 x 2 minor, is not formed:
    only |cos angle| and |angle| are used.  Shell points are in this package's spherical_field order
    (elevation-major), so the patterns reshape to [elevation, azimuth]; sample_shell.point_data
    ["Projected_Area"] holds them as a column."""
    from .geometry import spherical_field
    if az_range is None:
        az_range = np.linspace(-180.0, 180.0, 19)
    if elev_range is None:
        elev_range = np.linspace(-90.0, 90.0, 19)
    pts = np.asarray(getattr(source_coords, "points", source_coords), dtype=np.float32).reshape(-1, 3)
    n_src = pts.shape[0]
    shell = spherical_field(az_range, elev_range, outward_normals=True, field_radius=shell_range)
    sinks = np.asarray(shell.points, dtype=np.float32)
    n_snk = sinks.shape[0]
    hit_index, _ = workchunkingv2(pts, sinks, np.empty((0, 3), np.float32), environment, 1)
    src_t = P._points(pts)
    dev = src_t.device
    hi = torch.as_tensor(hit_index, device=dev).long().reshape(-1, 2)
    si, mi = hi[:, 0] - 1, hi[:, 1] - 1 - n_src
    # calc_dv_norm (lyceanem/utility/math_functions.py:149-156): float32, nothing fused
    r = P._points(sinks)[mi] - src_t[si]
    length = torch.sqrt((r[:, 0] * r[:, 0] + r[:, 1] * r[:, 1]) + r[:, 2] * r[:, 2])
    d = r / length[:, None]
    nrm = P._dev(np.asarray(source_normals, dtype=np.float32).reshape(-1, 3), torch.float32)[si]
    u1 = d / torch.linalg.vector_norm(d, dim=1, keepdim=True)
    u2 = nrm / torch.linalg.vector_norm(nrm, dim=1, keepdim=True)
    # angle(): arccos of the dot product clamped to [-1, 1] in FP64, stored as float32 (rayfunctions.py:436-448)
    ang = torch.arccos((u1 * u2).sum(1).double().clamp(-1.0, 1.0)).float()
    area = np.nan_to_num(np.asarray(vertex_area, dtype=np.float64).reshape(-1), nan=0.0)
    if area.size == 1:
        portion = torch.ones_like(ang, dtype=torch.float64) if area[0] == 0 else \
            area[0] * torch.cos(ang).abs().double()
    else:
        portion = torch.as_tensor(area, device=dev)[si] * torch.cos(ang).abs().double()
    portion = torch.where(ang.abs().double() > np.pi / 2, torch.zeros_like(portion), portion)
    # patternsort (rayfunctions.py:462-468): the sum over each shell point's visible sources
    total = torch.zeros(n_snk, dtype=torch.float64, device=dev).index_add_(0, mi, portion)
    visible = total.float().cpu().numpy().reshape(len(elev_range), len(az_range))
    shell.point_data["Projected_Area"] = visible.reshape(-1, 1)
    return visible, shell
