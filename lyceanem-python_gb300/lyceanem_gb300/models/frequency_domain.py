"""Frequency-domain models with the call shape of lyceanem/models/frequency_domain.py.

calculate_scattering / calculate_farfield / calculate_scattering_cuda take the
same arguments as the reference's CUDA branch (lyceanem/models/frequency_domain.py:94-264,
719-926) and return the same arrays.  With elements=False the source sum is
fused into the device kernels, so the [N, M, 3] network (and, with one
bounce, the [P, M, 3] scatter network) is never formed:
    E[m, c] = sum_n S0[n, m, c] + sum_p e_p[c] * S2[p, m, c],   e_p = sum_n S1[n, p, :]
which is 1^T (S0 + S1 @ S2) of the reference's composition (:230-260, :847-849).
"""
import copy

import numpy as np
import torch

from .. import propagation as P
from ..geometry import Mesh, calculate_conformal_vectors, spherical_field, triangles_of
from . import acceleration_structures


def _as_structure(antenna_solid, acceleration_structure, grid_cell=None):
    if acceleration_structure is not None:
        return acceleration_structure
    verts, faces = triangles_of(antenna_solid)
    mesh = Mesh(verts, [("triangle", faces)])
    return acceleration_structures.Tile_acceleration_structure(mesh, 1, grid_cell=grid_cell)


def _excitation(desired_E_axis, aperture_coords, project_vectors, antenna_axes):
    """Source E-vectors of the CUDA branch (frequency_domain.py:729-773), times the point areas."""
    normals = np.asarray(aperture_coords.point_data["Normals"])
    n = normals.shape[0]
    desired = np.asarray(desired_E_axis)
    if project_vectors:
        E = calculate_conformal_vectors(desired, normals, antenna_axes)
    elif desired.shape[0] == n and desired.ndim == 2:
        E = copy.deepcopy(desired)
    else:
        E = np.repeat(desired.reshape(1, 3).astype(np.complex64), n, axis=0)
    area = np.asarray(aperture_coords.point_data.get("Area", np.ones(n))).reshape(-1, 1)
    return (E * area).astype(np.complex64)


def sink_field(structure, src, E, snk, snk_n, alpha, beta, scat=None, scat_n=None, scattering=0, counters=None,
               cull=True, eps=P.EPSILON):
    """Fused source-summed sink field (complex64 [M,3] CUDA tensor) of the direct path and,
    with scattering=1, the one-bounce path, on the current stream."""
    dev = structure.device
    kw = dict(tris=dev.tris, grid=dev.grid, alpha=alpha, beta=beta, self_to_self=False, counters=counters, cull=cull,
              eps=eps)
    # Processing order: scatter points (unstructured) are traced in Morton
    # order; sources and sinks keep the caller's order, which for arrays and
    # elevation-major far-field grids already puts rays of similar cost in a warp.
    out = P.pair_stage(src, E, snk, snk_n, **kw).sink
    if scattering >= 1 and scat is not None and len(scat):
        scat = P._points(scat)
        o_scat = P.spatial_order(scat)
        e_p = P.pair_stage(src, E, scat, scat_n, snk_order=o_scat, **kw).sink
        P.pair_stage(scat, e_p, snk, snk_n, src_W=e_p, sink_out=out, accumulate=True, src_order=o_scat, **kw)
    return out


def calculate_scattering_cuda(alpha, beta, wavelength, acceleration_structure, scatter_depth, source_mesh, sink_mesh,
                              scatter_mesh=None, chunks=1):
    """Per-element network total = S0 (+ S1 @ S2 per component), complex64 [N, M, 3]
    (lyceanem/models/frequency_domain.py:195-264)."""
    acc = acceleration_structure
    total = acc.calculate_scattering(source_mesh, sink_mesh, alpha, beta, wavelength, chunk_count=chunks,
                                     self_to_self=False)
    if scatter_depth == 0:
        return total
    S1 = acc.calculate_scattering(source_mesh, scatter_mesh, alpha, beta, wavelength, chunk_count=chunks,
                                  self_to_self=False)
    scatter_mesh.point_data["ex"] = S1[:, :, 0].sum(axis=0)
    scatter_mesh.point_data["ey"] = S1[:, :, 1].sum(axis=0)
    scatter_mesh.point_data["ez"] = S1[:, :, 2].sum(axis=0)
    S2 = acc.calculate_scattering(scatter_mesh, sink_mesh, alpha, beta, wavelength, chunk_count=chunks,
                                  self_to_self=False)
    if scatter_depth == 1:
        a = torch.from_numpy(np.ascontiguousarray(S1)).cuda()
        b = torch.from_numpy(np.ascontiguousarray(S2)).cuda()
        t = torch.from_numpy(total).cuda()
        for c in range(3):
            t[:, :, c] += a[:, :, c] @ b[:, :, c]
        return t.cpu().numpy()
    return total


def calculate_scattering(aperture_coords, sink_coords, antenna_solid, desired_E_axis, scatter_points=None,
                         wavelength=1.0, scattering=0, elements=False, los=True, project_vectors=False,
                         antenna_axes=np.eye(3), multiE=False, alpha=0.0, beta=(np.pi * 2) / 1.0, cuda=True,
                         acceleration_structure=None, chunks=1, permittivity=8.8541878176e-12,
                         permeability=1.25663706212e-6, grid_cell=None):
    """Ex, Ey, Ez at the sinks (elements=False: complex64 [M] each, summed over
    sources) or per element (elements=True: [N, M] each), like the reference.

    cuda=False selects the numba engine's visibility rule (no back-face cull,
    eps 1e-7, lyceanem/raycasting/rayfunctions.py:37-104) on the same kernels."""
    del los, permittivity, permeability
    cull, eps = (True, P.EPSILON) if cuda else (False, P.NUMBA_EPSILON)
    acc = _as_structure(antenna_solid, acceleration_structure, grid_cell)
    src = np.asarray(aperture_coords.points, dtype=np.float32)
    snk = np.asarray(sink_coords.points, dtype=np.float32)
    snk_n = np.asarray(sink_coords.point_data["Normals"], dtype=np.float32)
    scat = scat_n = None
    if scattering > 0 and scatter_points is not None:
        scat = np.asarray(scatter_points.points, dtype=np.float32)
        scat_n = np.asarray(scatter_points.point_data["Normals"], dtype=np.float32)
    N = src.shape[0]

    def fused(E):
        f = sink_field(acc, src, E, snk, snk_n, alpha, beta, scat, scat_n, scattering, cull=cull, eps=eps)
        f = f.cpu().numpy()
        return f[:, 0], f[:, 1], f[:, 2]

    def per_element(E):
        aperture_coords.point_data["ex"] = E[:, 0]
        aperture_coords.point_data["ey"] = E[:, 1]
        aperture_coords.point_data["ez"] = E[:, 2]
        S = calculate_scattering_cuda(alpha, beta, wavelength, acc, scattering, aperture_coords, sink_coords,
                                      scatter_points, chunks)
        return S

    if not multiE:
        E = _excitation(desired_E_axis, aperture_coords, project_vectors, antenna_axes)
        if not elements:
            return fused(E)
        S = per_element(E)
        return S[:, :, 0], S[:, :, 1], S[:, :, 2]
    # multiE: one excitation per row of desired_E_axis (frequency_domain.py:858-921)
    desired = np.asarray(desired_E_axis)
    normals = np.asarray(aperture_coords.point_data["Normals"]).astype(np.float32)
    if not elements:
        K = desired.shape[0]
        Ex = np.zeros((K, snk.shape[0]), np.complex64)
        Ey, Ez = Ex.copy(), Ex.copy()
        for k in range(K):
            E = calculate_conformal_vectors(desired[k, :], normals, antenna_axes)
            Ex[k], Ey[k], Ez[k] = fused(E)
        return Ex, Ey, Ez
    K = desired.shape[1]
    Ex = np.zeros((N, snk.shape[0], K), np.complex64)
    Ey, Ez = Ex.copy(), Ex.copy()
    for k in range(K):
        E = calculate_conformal_vectors(desired[k, :], normals, antenna_axes)
        for e in range(N):
            Ee = np.zeros_like(E)
            Ee[e] = E[e]
            Ex[e, :, k], Ey[e, :, k], Ez[e, :, k] = fused(Ee)
    return Ex, Ey, Ez


def calculate_farfield(aperture_coords, antenna_solid, desired_E_axis, az_range=None, el_range=None,
                       scatter_points=None, wavelength=1.0, farfield_distance=2.0, scattering=0, elements=False,
                       los=True, project_vectors=False, cuda=True, antenna_axes=np.eye(3), alpha=0.0,
                       beta=(np.pi * 2) / 1.0, grid_cell=None):
    """E_theta, E_phi on a far-field sphere (lyceanem/models/frequency_domain.py:94-192)."""
    if az_range is None:
        az_range = np.linspace(-180.0, 180.0, 19)
    if el_range is None:
        el_range = np.linspace(-90.0, 90.0, 19)
    sink_coords = spherical_field(az_range, el_range, field_radius=farfield_distance)
    Ex, Ey, Ez = calculate_scattering(aperture_coords, sink_coords, antenna_solid, desired_E_axis,
                                      scatter_points=scatter_points, wavelength=wavelength, scattering=scattering,
                                      elements=elements, los=los, project_vectors=project_vectors,
                                      antenna_axes=antenna_axes, multiE=False, cuda=cuda, alpha=alpha, beta=beta,
                                      grid_cell=grid_cell)
    th = sink_coords.point_data["theta_(Radians)"]
    ph = sink_coords.point_data["phi_(Radians)"]
    etheta = Ex * np.cos(ph) * np.cos(th) + Ey * np.sin(ph) * np.cos(th) - Ez * np.sin(th)
    ephi = -Ex * np.sin(ph) + Ey * np.cos(ph)
    return etheta, ephi
