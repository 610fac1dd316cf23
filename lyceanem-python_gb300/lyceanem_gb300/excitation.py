"""Source excitation weights: the inputs of the propagation path, with the interface of the reference's
excitation_function (lyceanem/electromagnetics/emfunctions.py:9-82) and its helpers WavefrontWeights and
ArbitaryCoherenceWeights (lyceanem/electromagnetics/beamforming.py:81-152) and discrete_transmit_power
(lyceanem/utility/math_functions.py:79-121).  Host numpy, evaluated once per excitation.

The reference's own known-answer tests of excitation_function (lyceanem/tests/test_base_classes.py:70-152)
state unit E-vectors; the function they call scales its result to the requested transmit power (one
point of the default area (wavelength / 2)^2 at 1 W over 120 pi ohms gives |E| = sqrt(4 * 120 pi)), so
those answers hold for the direction of the result, and the magnitude follows discrete_transmit_power.
"""
import numpy as np

from .geometry import calculate_conformal_vectors

SPEED_OF_LIGHT = 299792458.0  # scipy.constants.speed_of_light
FREE_SPACE_IMPEDANCE = np.pi * 120.0  # the reference's default impedance


def wavefront_weights(source_coords, steering_vector, wavelength):
    """Unit-amplitude weights steering toward a direction: phases from the distances of the elements to
    a point 1e9 m along the steering vector, less the smallest (WavefrontWeights, complex64 (N,))."""
    s = np.asarray(source_coords)
    v = np.asarray(steering_vector, dtype=np.float64).ravel()
    dist = np.sqrt(np.abs((s[:, 0] - v[0] * 1e9) ** 2 + (s[:, 1] - v[1] * 1e9) ** 2 + (s[:, 2] - v[2] * 1e9) ** 2))
    dist = dist - np.min(dist)
    delays = dist / SPEED_OF_LIGHT
    w = np.zeros(s.shape[0], dtype=np.complex64)
    w[:] = np.exp(1j * 2 * np.pi * (SPEED_OF_LIGHT / wavelength) * delays)
    return w


def coherence_weights(source_coords, target_coord, wavelength):
    """Weights focusing on a target point: phases from the element-to-target distances less the smallest
    (ArbitaryCoherenceWeights, complex64 (N, 1))."""
    s = np.asarray(source_coords, dtype=np.float64)
    t = np.asarray(target_coord, dtype=np.float64).reshape(-1, 3)
    dist = np.sqrt(((s[:, None, :] - t[None, :, :]) ** 2).sum(-1))
    dist = dist - np.min(dist)
    delays = dist / SPEED_OF_LIGHT
    w = np.zeros((s.shape[0], 1), dtype=np.complex64)
    w[:] = np.exp(1j * 2 * np.pi * (SPEED_OF_LIGHT / wavelength) * delays)
    return w


def discrete_transmit_power(weights, element_area, transmit_power=100.0, impedance=FREE_SPACE_IMPEDANCE):
    """Per-point complex amplitudes (V/m) with the directions and phases of `weights` whose power,
    |weights| x area summed over the aperture, is normalised to `transmit_power` watts."""
    w = np.asarray(weights)
    area = np.asarray(element_area).reshape(-1, 1)
    power_at_point = np.linalg.norm(w, axis=1).reshape(-1, 1) * area
    power_normalisation = transmit_power / np.sum(power_at_point)
    density = (power_at_point * power_normalisation) / area
    amplitude = (density * impedance) ** 0.5
    return (w / np.linalg.norm(w, axis=1).reshape(-1, 1)) * amplitude


def excitation_function(aperture_points, desired_e_vector, phase_shift="none", wavelength=1.0,
                        steering_vector=np.zeros((1, 3)), transmit_power=1.0, local_projection=True):
    """Calibrated E-vector weights (N, 3) of an aperture point cloud (`.points`, `.point_data["Normals"]`,
    optionally `.point_data["Area"]`, else (wavelength / 2)^2 per point) for a desired E-vector:
    projected onto each point's local (u, v, n) axes when local_projection, phase-steered by
    phase_shift "wavefront" (toward a direction) or "coherence" (onto a point), and scaled to the total
    transmit power.  A 1-D desired vector with local_projection=False is taken as one row (the reference
    repeats it into a flat array there, which its power normalisation cannot take)."""
    pts = np.asarray(aperture_points.points)
    n = pts.shape[0]
    if local_projection:
        w = calculate_conformal_vectors(desired_e_vector, np.asarray(aperture_points.point_data["Normals"]),
                                        np.eye(3))
    else:
        d = np.asarray(desired_e_vector)
        w = np.repeat(d.reshape(1, -1) if d.ndim == 1 else d, n, axis=0)
    if phase_shift == "wavefront":
        w = w * wavefront_weights(pts, steering_vector, wavelength).reshape(-1, 1)
    if phase_shift == "coherence":
        w = w * coherence_weights(pts, steering_vector, wavelength).reshape(-1, 1)
    if "Area" in aperture_points.point_data:
        areas = np.asarray(aperture_points.point_data["Area"])
    else:
        areas = np.zeros(n)
        areas[:] = (wavelength * 0.5) ** 2
    return discrete_transmit_power(w, areas, transmit_power)
