"""Time-domain model with the call shape of lyceanem/models/time_domain.py.

calculate_scattering reuses the numba engine's path list (raycasting.workchunkingv2,
visibility resolved once) and, per row, a real magnitude vector and an arrival
time (lyem_path_time); the sink signals are the excitation placed at each row's
arrival relative to the earliest one, built as an amplitude histogram of
arrival samples convolved with the excitation (empropagation.time_map).
"""
import numpy as np

from .. import raycasting as RC
from ..empropagation import path_times, time_map
from ..geometry import calculate_conformal_vectors
from .frequency_domain import _as_structure


def _weights(desired_E_axis, aperture_coords, project_vectors, antenna_axes):
    """Source E-vectors of lyceanem/models/time_domain.py:75-118 (times the point areas)."""
    normals = np.asarray(aperture_coords.point_data["Normals"])
    n = normals.shape[0]
    desired = np.asarray(desired_E_axis)
    if project_vectors:
        E = np.asarray(calculate_conformal_vectors(desired, normals, antenna_axes), np.complex64)
    elif desired.ndim == 2 and desired.shape[0] == n:
        E = desired.astype(np.complex64)
    else:
        E = np.repeat(desired.reshape(1, 3).astype(np.complex64), n, axis=0)
    area = np.asarray(aperture_coords.point_data.get("Area", np.ones(n))).reshape(-1, 1)
    return (E * area).astype(np.complex64)


def calculate_scattering(aperture_coords, sink_coords, excitation_function, antenna_solid, desired_E_axis,
                         scatter_points=None, wavelength=1.0, scattering=0, elements=False, sampling_freq=1e9,
                         los=False, num_samples=10000, antenna_axes=np.eye(3), project_vectors=True, alpha=0.0,
                         beta=(np.pi * 2) / 1.0, grid_cell=None):
    """(Ex, Ey, Ez, WakeTimes) of lyceanem/models/time_domain.py:14-525.

    elements=False: float64 [num_samples] per component, the sum over all sources and sinks,
    starting at the sample of the earliest arrival (np.digitize of the wake time on
    linspace(0, num_samples / sampling_freq, num_samples)).  elements=True: the reference's
    per-element loop -- element e excited alone with E_e / N -- whose result, summed over
    sources and sinks, it assigns to every sink: float64 [N, M, num_samples] per component."""
    acc = _as_structure(antenna_solid, None, grid_cell)
    S = int(num_samples)
    time_index = np.linspace(0, S / sampling_freq, S)
    src = np.asarray(aperture_coords.points, np.float32)
    src_n = np.asarray(aperture_coords.point_data["Normals"], np.float32)
    snk = np.asarray(sink_coords.points, np.float32)
    snk_n = np.asarray(sink_coords.point_data["Normals"], np.float32)
    if scattering > 0 and scatter_points is not None:
        scat = np.asarray(scatter_points.points, np.float32)
        scat_n = np.asarray(scatter_points.point_data["Normals"], np.float32)
    else:
        scat = np.zeros((0, 3), np.float32)
        scat_n = np.zeros((0, 3), np.float32)
    N, M = src.shape[0], snk.shape[0]
    E = _weights(desired_E_axis, aperture_coords, project_vectors, antenna_axes)
    idx, _ = RC.workchunkingv2(src, snk, scat, acc.device.tris, scattering + 1, line_of_sight=los)
    pos = np.concatenate([src, snk, scat])
    nrm = np.concatenate([src_n, snk_n, scat_n])
    w = np.ones((pos.shape[0], 3), np.complex64)

    def run(weights):
        w[:N] = weights
        amp, arrival, pair = path_times(idx, pos, nrm, w, N, M, alpha, beta)
        return time_map(amp, arrival, pair, N, M, excitation_function, sampling_freq, S)

    if not elements:
        tm, wake = run(E)
        total = tm.sum(dim=(0, 1)).cpu().numpy()  # [S, 3]
        wake_index = int(np.digitize(wake, time_index))
        out = np.zeros((S, 3), np.float64)
        out[wake_index:] = total[:S - wake_index]
        return out[:, 0], out[:, 1], out[:, 2], np.array([wake])
    Ex = np.zeros((N, M, S), np.float64)
    Ey, Ez = Ex.copy(), Ex.copy()
    wake = 1.0
    for e in range(N):
        We = np.zeros_like(E)
        We[e] = E[e] / N
        tm, wake = run(We)
        total = tm.sum(dim=(0, 1)).cpu().numpy()
        Ex[e], Ey[e], Ez[e] = total[:, 0], total[:, 1], total[:, 2]
    return Ex, Ey, Ez, np.array([wake])
