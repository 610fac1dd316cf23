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
from ..geometry import calculate_conformal_vectors, spherical_field, triangles_of
from . import acceleration_structures


def _as_structure(antenna_solid, acceleration_structure, grid_cell=None):
    """The caller's structure, or the device scene of antenna_solid from the scene cache
    (packed triangles and grid stay on the device across calls with the same geometry)."""
    if acceleration_structure is not None:
        return acceleration_structure
    verts, faces = triangles_of(antenna_solid)
    return acceleration_structures.cached_structure(verts, faces, grid_cell)


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


def _sink_order(dev, snk):
    """Sinks in direction order seen from the grid's centre (rays of a warp then share a direction and
    walk similar cells); natural order for brute force."""
    return P.direction_order(snk, dev.grid.centre) if dev.grid is not None else None


def sink_field(structure, src, E, snk, snk_n, alpha, beta, scat=None, scat_n=None, scattering=0, counters=None,
               cull=True, eps=P.EPSILON, skip_unlit=False):
    """Fused source-summed sink field (complex64 [M,3] CUDA tensor) of the direct path and,
    with scattering=1, the one-bounce path, on the current stream.

    skip_unlit: trace the scatter->sink rays only from the scattering points that
    at least one source sees.  A point no source sees has a source->scatter field
    of exactly zero, so every one-bounce path through it contributes exactly zero
    (the reference forms those paths in S1 @ S2, lyceanem/models/frequency_domain.py:
    230-260, and their products vanish); the field is the same up to the FP32
    rounding of the regrouped source sums.  Costs one device->host read (the
    number of lit points)."""
    dev = structure.device
    kw = dict(tris=dev.tris, grid=dev.grid, alpha=alpha, beta=beta, self_to_self=False, counters=counters, cull=cull,
              eps=eps)
    # Processing order: scatter points (unstructured) are traced in Morton
    # order, sinks in direction order from the scene; sources keep the
    # caller's order.
    snk = P._points(snk)
    o_snk = _sink_order(dev, snk)
    # the stages that start at the sources take the transposed schedule when the sources are compact (an array)
    ts = P.source_schedule(src, dev.grid)
    out = P.pair_stage(src, E, snk, snk_n, snk_order=o_snk, traversal=ts, **kw).sink
    if scattering >= 1 and scat is not None and len(scat):
        scat = P._points(scat)
        o_scat = P.spatial_order(scat)
        if not skip_unlit:
            e_p = P.pair_stage(src, E, scat, scat_n, snk_order=o_scat, traversal=ts, **kw).sink
            P.pair_stage(scat, e_p, snk, snk_n, src_W=e_p, sink_out=out, accumulate=True, src_order=o_scat,
                         snk_order=o_snk, **kw)
            return out
        seen = torch.zeros(scat.shape[0], dtype=torch.int32, device=scat.device)
        e_p = P.pair_stage(src, E, scat, scat_n, snk_order=o_scat, traversal=ts, snk_visible=seen, **kw).sink
        # the lit points in Morton order, passed as a subset order (each keeps its row, so the reference's
        # untested pair of equal source and sink index stays the same pair)
        lit = o_scat[seen[o_scat.long()] > 0].contiguous()
        if lit.numel():
            P.pair_stage(scat, e_p, snk, snk_n, src_W=e_p, sink_out=out, accumulate=True, src_order=lit,
                         snk_order=o_snk, **kw)
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


# ------------------------------------------------------------ numba engine (cuda=False)

def _numba_excitation(desired_E_axis, aperture_coords, project_vectors, antenna_axes, scattering, multiE):
    """Source E-vectors of the numba branch (lyceanem/models/frequency_domain.py:337-485): with
    scattering 0 the CUDA branch's rule times the point areas; with scattering > 0 the first row of
    desired_E_axis (real part, as the reference casts it to float32) repeated, or its conformal
    vectors, without areas."""
    if scattering == 0:
        return _excitation(desired_E_axis, aperture_coords, project_vectors, antenna_axes)
    normals = np.asarray(aperture_coords.point_data["Normals"]).astype(np.float32)
    n = normals.shape[0]
    desired = np.atleast_2d(np.asarray(desired_E_axis))
    if project_vectors:
        return np.asarray(calculate_conformal_vectors(desired[0, :].reshape(1, 3), normals), np.complex64)
    if multiE and desired.size != 3:
        return desired.reshape(n, 3).astype(np.complex64)
    return np.repeat(desired[0, :].astype(np.float32).reshape(1, 3), n, axis=0).astype(np.complex64)


def _unit(t):
    return t / torch.linalg.norm(t, dim=-1, keepdim=True)


def numba_sink_field(structure, src, E, snk, snk_n, alpha, beta, scat=None, scat_n=None, scattering=0, los=True):
    """Source-summed sink field of the numba engine (complex64 [M,3] CUDA tensor), scattering 0 or 1.

    The engine sums, over workchunkingv2's unblocked paths, the products of
    freqdomainkernal (lyceanem/electromagnetics/empropagation.py:1083-1265).  With
    P(x) f = f - (f.x^) x^ and S the em_wave pair field, that sum factors as
      scattering 0:  sum_n S0[n, m]
      scattering 1:  P(n_m) sum_n S0[n, m] (line of sight)  +  sum_p S2(p, m; P(n_p) e_p),
                     e_p = sum_n S1[n, p]
    (a 3-column path index projects the direct paths at the sink too), so it runs as
    three pair stages and two projections.  Visibility: no back-face cull, EPSILON
    1e-7, every pair tested."""
    from ..empropagation import tangential_project
    dev = structure.device
    kw = dict(tris=dev.tris, grid=dev.grid, alpha=alpha, beta=beta, self_to_self=True, cull=False,
              eps=P.NUMBA_EPSILON)
    snk_n_t = P._points(snk_n)
    snk = P._points(snk)
    o_snk = _sink_order(dev, snk)
    if scattering == 0 or los:
        out = P.pair_stage(src, E, snk, snk_n_t, snk_order=o_snk, **kw).sink
    else:
        out = torch.zeros((snk_n_t.shape[0], 3), dtype=torch.complex64, device=snk_n_t.device)
    if scattering >= 1:
        tangential_project(out, snk_n_t)
        if scat is not None and len(scat):
            scat_t = P._points(scat)
            o = P.spatial_order(scat_t)
            e_p = P.pair_stage(src, E, scat_t, scat_n, snk_order=o, **kw).sink
            tangential_project(e_p, scat_n)
            P.pair_stage(scat_t, e_p, snk, snk_n_t, sink_out=out, accumulate=True, src_order=o, snk_order=o_snk, **kw)
    return out


def numba_per_element(structure, src, E, snk, snk_n, alpha, beta, scat=None, scat_n=None, scattering=0, los=True):
    """Per-element network of the numba engine (complex64 [N,M,3] CUDA tensor), scattering 0 or 1:
    the direct network (projected at the sinks when scattering is on) plus
    sum_p sum_k U[n,p,k] T_k[p,m,:], U = P(n_p) S1[n,p] and T_k the scatter->sink network
    of a unit excitation along axis k."""
    dev = structure.device
    kw = dict(tris=dev.tris, grid=dev.grid, alpha=alpha, beta=beta, self_to_self=True, cull=False,
              eps=P.NUMBA_EPSILON, want_pairs=True)
    src_t, snk_t, snk_n_t = P._points(src), P._points(snk), P._points(snk_n)
    N, M = src_t.shape[0], snk_t.shape[0]
    if scattering == 0 or los:
        S = P.pair_stage(src_t, E, snk_t, snk_n_t, **kw).pairs
    else:
        S = torch.zeros((N, M, 3), dtype=torch.complex64, device=src_t.device)
    if scattering >= 1:
        u = _unit(snk_n_t).to(torch.complex64)[None]
        S = S - (S * u).sum(-1, keepdim=True) * u
        if scat is not None and len(scat):
            scat_t, scat_n_t = P._points(scat), P._points(scat_n)
            Pn = scat_t.shape[0]
            U = P.pair_stage(src_t, E, scat_t, scat_n_t, **kw).pairs
            up = _unit(scat_n_t).to(torch.complex64)[None]
            U = U - (U * up).sum(-1, keepdim=True) * up
            for k in range(3):
                ek = torch.zeros((Pn, 3), dtype=torch.complex64, device=src_t.device)
                ek[:, k] = 1.0
                T = P.pair_stage(scat_t, ek, snk_t, snk_n_t, **kw).pairs
                S = S + (U[:, :, k].contiguous() @ T.reshape(Pn, M * 3)).reshape(N, M, 3)
    return S


def _numba_paths_network(acc, src, src_n, E, snk, snk_n, scat, scat_n, alpha, beta, max_scatter, los):
    """Per-element network through the explicit path list (workchunkingv2 + EMGPUFreqDomain)."""
    from .. import raycasting as RC
    from ..empropagation import path_network
    dev = acc.device
    env = dev.tris
    scat = np.zeros((0, 3), np.float32) if scat is None else scat
    scat_n = np.zeros((0, 3), np.float32) if scat_n is None else scat_n
    idx, _ = RC.workchunkingv2(src, snk, scat, env, max_scatter, line_of_sight=los)
    N, M = src.shape[0], snk.shape[0]
    pos = np.concatenate([src, snk, scat]).astype(np.float32)
    nrm = np.concatenate([src_n, snk_n, scat_n]).astype(np.float32)
    w = np.ones((pos.shape[0], 3), np.complex64)
    w[:N] = E
    if idx.shape[0] == 0:
        return torch.zeros((N, M, 3), dtype=torch.complex64, device="cuda")
    return path_network(idx, pos, nrm, w, N, M, alpha, beta).to(torch.complex64)


def _numba_branch(aperture_coords, sink_coords, antenna_solid, desired_E_axis, scatter_points, scattering, elements,
                  los, project_vectors, antenna_axes, multiE, alpha, beta, acceleration_structure, grid_cell):
    """calculate_scattering(..., cuda=False) (lyceanem/models/frequency_domain.py:333-718)."""
    acc = _as_structure(antenna_solid, acceleration_structure, grid_cell)
    src = np.asarray(aperture_coords.points, dtype=np.float32)
    src_n = np.asarray(aperture_coords.point_data["Normals"], dtype=np.float32)
    snk = np.asarray(sink_coords.points, dtype=np.float32)
    snk_n = np.asarray(sink_coords.point_data["Normals"], dtype=np.float32)
    scat = scat_n = None
    if scattering > 0 and scatter_points is not None:
        scat = np.asarray(scatter_points.points, dtype=np.float32)
        scat_n = np.asarray(scatter_points.point_data["Normals"], dtype=np.float32)
    N = src.shape[0]

    def network(E):
        if scattering >= 2:
            return _numba_paths_network(acc, src, src_n, E, snk, snk_n, scat, scat_n, alpha, beta, scattering + 1,
                                        los)
        return numba_per_element(acc, src, E, snk, snk_n, alpha, beta, scat, scat_n, scattering, los)

    def summed(E):
        if scattering >= 2:
            return network(E).sum(0)
        return numba_sink_field(acc, src, E, snk, snk_n, alpha, beta, scat, scat_n, scattering, los)

    if not multiE:
        E = _numba_excitation(desired_E_axis, aperture_coords, project_vectors, antenna_axes, scattering, multiE)
        if not elements:
            f = summed(E).cpu().numpy()
            return f[:, 0], f[:, 1], f[:, 2]
        S = network(E).cpu().numpy()
        return S[:, :, 0], S[:, :, 1], S[:, :, 2]
    desired = np.asarray(desired_E_axis)
    normals = src_n
    if not elements:
        K = desired.shape[0]
        Ex = np.zeros((K, snk.shape[0]), np.complex64)
        Ey, Ez = Ex.copy(), Ex.copy()
        for k in range(K):
            E = calculate_conformal_vectors(desired[k, :], normals)
            f = summed(np.asarray(E, np.complex64)).cpu().numpy()
            Ex[k], Ey[k], Ez[k] = f[:, 0], f[:, 1], f[:, 2]
        return Ex, Ey, Ez
    K = desired.shape[1]
    Ex = np.zeros((N, snk.shape[0], K), np.complex64)
    Ey, Ez = Ex.copy(), Ex.copy()
    for k in range(K):
        E = np.asarray(calculate_conformal_vectors(desired[k, :], normals), np.complex64)
        for e in range(N):
            Ee = np.zeros_like(E)
            Ee[e] = E[e]
            f = summed(Ee).cpu().numpy()
            Ex[e, :, k], Ey[e, :, k], Ez[e, :, k] = f[:, 0], f[:, 1], f[:, 2]
    return Ex, Ey, Ez


def calculate_scattering(aperture_coords, sink_coords, antenna_solid, desired_E_axis, scatter_points=None,
                         wavelength=1.0, scattering=0, elements=False, los=True, project_vectors=False,
                         antenna_axes=np.eye(3), multiE=False, alpha=0.0, beta=(np.pi * 2) / 1.0, cuda=False,
                         acceleration_structure=None, chunks=1, permittivity=8.8541878176e-12,
                         permeability=1.25663706212e-6, grid_cell=None, skip_unlit=False):
    """Ex, Ey, Ez at the sinks (elements=False: complex64 [M] each, summed over
    sources) or per element (elements=True: [N, M] each), like the reference.

    cuda=False reproduces the numba engine's branch on this package's kernels:
    its visibility rule (no back-face cull, EPSILON 1e-7, every pair tested,
    lyceanem/raycasting/rayfunctions.py:37-104, 2624-2680), its path product with
    tangential projection at scatter points and sinks
    (lyceanem/electromagnetics/empropagation.py:1083-1265) and its excitation
    rules; scattering=2 goes through the explicit path list.

    skip_unlit (not in the reference; CUDA branch, source-summed fields): the
    one-bounce stage traces only from the scattering points that some source
    sees, as sink_field describes; off by default."""
    del permittivity, permeability
    if not cuda:
        return _numba_branch(aperture_coords, sink_coords, antenna_solid, desired_E_axis, scatter_points, scattering,
                             elements, los, project_vectors, antenna_axes, multiE, alpha, beta, acceleration_structure,
                             grid_cell)
    del los
    cull, eps = True, P.EPSILON
    alpha, beta = acceleration_structures.em_float(alpha), acceleration_structures.em_float(beta)
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
        f = sink_field(acc, src, E, snk, snk_n, alpha, beta, scat, scat_n, scattering, cull=cull, eps=eps,
                       skip_unlit=skip_unlit)
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
                       los=True, project_vectors=False, cuda=False, antenna_axes=np.eye(3), alpha=0.0,
                       beta=(np.pi * 2) / 1.0, grid_cell=None):
    """E_theta, E_phi on a far-field sphere (lyceanem/models/frequency_domain.py:94-192).  As in the
    reference, farfield_distance reaches spherical_field as its third positional argument, outward_normals
    (:159): the sinks lie on the unit sphere, with outward normals unless farfield_distance is 0."""
    if az_range is None:
        az_range = np.linspace(-180.0, 180.0, 19)
    if el_range is None:
        el_range = np.linspace(-90.0, 90.0, 19)
    sink_coords = spherical_field(az_range, el_range, farfield_distance)
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
