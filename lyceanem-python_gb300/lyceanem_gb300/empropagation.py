"""Numba-engine field products with the call shape of lyceanem/electromagnetics/empropagation.py.

EMGPUFreqDomain evaluates every path row of the numba engine's index (see
raycasting.workchunkingv2) on the GPU (lyem_path_field) and sums the fields
per (source, sink), as freqdomainkernal does
(lyceanem/electromagnetics/empropagation.py:1083-1265, 2197-2410).
"""
import ctypes

import numpy as np
import torch

from . import propagation as P
from ._native import LyemError, check, lib

# scattering_point of lyceanem/base_types.py (numpy record layout, no numba needed)
scattering_point = np.dtype([("px", "f4"), ("py", "f4"), ("pz", "f4"), ("vx", "f4"), ("vy", "f4"), ("vz", "f4"),
                             ("nx", "f4"), ("ny", "f4"), ("nz", "f4"), ("ex", "c8"), ("ey", "c8"), ("ez", "c8"),
                             ("permittivity", "c8"), ("permeability", "c8"), ("Electric", "?")], align=True)


def _vp(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def path_network(full_index, pos, nrm, weights, n_src, n_snk, alpha, beta, magnetic=None, impedance=None):
    """complex128 [n_src, n_snk, 3] on the device: the path rows' fields summed per (source, sink)."""
    dev = torch.device("cuda", torch.cuda.current_device())
    idx = torch.as_tensor(np.ascontiguousarray(np.asarray(full_index), dtype=np.int32), device=dev)
    pos = P._points(pos)
    nrm = P._points(nrm)
    w = torch.view_as_real(P._cvec(weights, pos.shape[0])).reshape(-1, 6).contiguous()
    mag = imp = None
    if magnetic is not None and np.any(np.asarray(magnetic)):
        mag = torch.as_tensor(np.asarray(magnetic, dtype=np.uint8), device=dev)
        imp = torch.as_tensor(np.asarray(impedance, dtype=np.float32), device=dev)
    out = torch.zeros((n_src, n_snk, 3, 2), dtype=torch.float64, device=dev)
    rows, cols = (idx.shape[0], idx.shape[1]) if idx.dim() == 2 else (0, 2)
    check(lib.lyem_path_field(_vp(idx), rows, cols, _vp(pos), _vp(nrm), _vp(w), _vp(mag), _vp(imp), pos.shape[0],
                              n_src, n_snk, float(alpha), float(beta), _vp(out), P._stream()), "path_field")
    st, flags = P.device_errors()
    if st != 0 or flags != 0:
        raise LyemError(st or 1, f"path_field: device error word {flags:#x} (an index out of range)")
    return torch.view_as_complex(out)


def EMGPUFreqDomain(source_num, sink_num, full_index, point_information, wavelength, alpha, beta):
    """Scattering network complex128 [source_num, sink_num, 3] of the paths in full_index
    (lyceanem/electromagnetics/empropagation.py:2197-2410); point_information is an array
    of scattering_point records ([sources, sinks, scatter points])."""
    del wavelength  # the reference's kernel takes alpha and beta; wavelength is unused there
    pts = np.asarray(point_information)
    pos = np.stack([pts["px"], pts["py"], pts["pz"]], 1).astype(np.float32)
    nrm = np.stack([pts["nx"], pts["ny"], pts["nz"]], 1).astype(np.float32)
    w = np.stack([pts["ex"], pts["ey"], pts["ez"]], 1).astype(np.complex64)
    magnetic = impedance = None
    if "Electric" in pts.dtype.names and not np.all(pts["Electric"]):
        magnetic = ~pts["Electric"].astype(bool)
        impedance = np.sqrt(np.real(pts["permeability"]).astype(np.float64)
                            / np.real(pts["permittivity"]).astype(np.float64)).astype(np.float32)
    idx = np.asarray(full_index)
    if idx.size == 0:
        return np.zeros((source_num, sink_num, 3), np.complex128)
    net = path_network(idx, pos, nrm, w, int(source_num), int(sink_num), alpha, beta, magnetic, impedance)
    return net.cpu().numpy()


def tangential_project(vec, normals):
    """In place on a complex64 [n, 3] CUDA tensor: f - (f . n^) n^ (sourcelaunchtransformGPU
    with a surface normal, lyceanem/electromagnetics/empropagation.py:179-258)."""
    nrm = P._points(normals)
    v = torch.view_as_real(vec)
    check(lib.lyem_tangential_project(_vp(v), _vp(nrm), vec.shape[0], P._stream()), "tangential_project")
    return vec


def path_times(full_index, pos, nrm, weights, n_src, n_snk, alpha, beta, magnetic=None, impedance=None):
    """Per path row (CUDA tensors): real magnitude vector float64 [R,3], arrival time float64 [R] (s)
    and (source, sink) int32 [R,2] -- the per-row part of timedomainkernal."""
    dev = torch.device("cuda", torch.cuda.current_device())
    idx = torch.as_tensor(np.ascontiguousarray(np.asarray(full_index), dtype=np.int32), device=dev)
    pos = P._points(pos)
    nrm = P._points(nrm)
    w = torch.view_as_real(P._cvec(weights, pos.shape[0])).reshape(-1, 6).contiguous()
    mag = imp = None
    if magnetic is not None and np.any(np.asarray(magnetic)):
        mag = torch.as_tensor(np.asarray(magnetic, dtype=np.uint8), device=dev)
        imp = torch.as_tensor(np.asarray(impedance, dtype=np.float32), device=dev)
    R, K = (idx.shape[0], idx.shape[1]) if idx.dim() == 2 else (0, 2)
    amp = torch.zeros((R, 3), dtype=torch.float64, device=dev)
    arrival = torch.zeros(R, dtype=torch.float64, device=dev)
    pair = torch.zeros((R, 2), dtype=torch.int32, device=dev)
    check(lib.lyem_path_time(_vp(idx), R, K, _vp(pos), _vp(nrm), _vp(w), _vp(mag), _vp(imp), pos.shape[0], n_src,
                             n_snk, float(alpha), float(beta), _vp(amp), _vp(arrival), _vp(pair), P._stream()),
          "path_time")
    st, flags = P.device_errors()
    if st != 0 or flags != 0:
        raise LyemError(st or 1, f"path_time: device error word {flags:#x} (an index out of range)")
    return amp, arrival, pair


MAP_BYTES_LIMIT = 1e9  # TimeDomainv3 splits the sources into chunks when its float64 map exceeds this


def start_samples(arrival, src_of_row, n_src, n_snk, num_samples, sampling_freq, map_bytes_limit=MAP_BYTES_LIMIT):
    """(start sample of each row's excitation, int64 [R]; the reported wake time) as TimeDomainv3 sets them
    (lyceanem/electromagnetics/empropagation.py:2955-3170), with the wake times taken before any row is
    placed (there an atomic minimum synchronised only within a thread block):
    - a map (n_src x n_snk x num_samples x 3 float64) of at most map_bytes_limit bytes has one wake time,
      min(1 s, the arrivals); a row starts floor((arrival - wake) / step) samples in;
    - a larger map splits the sources into ceil(bytes / limit) chunks (np.linspace bounds): chunk 0's wake
      is min(1 s, its arrivals), chunk n's min(chunk 0's wake, its arrivals), and a row starts relative to
      its chunk's wake.  When the chunk wakes differ by a sample or more the reference shifts each chunk by
      round((wake_n - min wake) / step) samples to align them (its copy for the chunk at the minimum uses the
      empty slice :-0, so there the reference raises); here that shift is applied.  The reported wake is
      chunk 0's."""
    dev = arrival.device
    step = 1.0 / sampling_freq
    nbytes = float(n_src) * n_snk * num_samples * 3 * 8
    step_t = torch.tensor(step, dtype=torch.float64, device=dev)
    if nbytes <= map_bytes_limit:
        wake = min(1.0, float(arrival.min().item())) if arrival.numel() else 1.0
        return torch.div(arrival - wake, step_t, rounding_mode="floor").to(torch.int64), wake
    n_chunks = int(np.ceil(nbytes / map_bytes_limit))
    bounds = np.linspace(0, n_src, n_chunks + 1).astype(np.int32)
    chunk = torch.bucketize(src_of_row.to(torch.int64), torch.as_tensor(bounds[1:-1], dtype=torch.int64, device=dev),
                            right=True)
    first = torch.full((n_chunks,), float("inf"), dtype=torch.float64, device=dev)
    first = first.scatter_reduce(0, chunk, arrival, reduce="amin").cpu().numpy()
    wakes = np.empty(n_chunks)
    wakes[0] = min(1.0, first[0])
    wakes[1:] = np.minimum(wakes[0], first[1:])
    shift = np.zeros(n_chunks, np.int64)
    if np.max((wakes - np.min(wakes)) / step) >= 1.0:
        shift = np.round((wakes - np.min(wakes)) / step).astype(np.int64)
    w_row = torch.as_tensor(wakes, device=dev)[chunk]
    s_row = torch.as_tensor(shift, device=dev)[chunk]
    return torch.div(arrival - w_row, step_t, rounding_mode="floor").to(torch.int64) + s_row, float(wakes[0])


def time_map(amp, arrival, pair, n_src, n_snk, excitation, sampling_freq, num_samples, map_bytes_limit=MAP_BYTES_LIMIT):
    """float64 [n_src, n_snk, num_samples, 3]: each row's excitation, scaled by its magnitudes, starting at
    the sample start_samples gives it and cut at num_samples (timedomainkernal adds the whole excitation
    where it fits and the part before the end where it does not,
    lyceanem/electromagnetics/empropagation.py:1509-1578); returned with the reported wake time.  Built
    as an amplitude histogram of start samples per (source, sink) convolved with the excitation (FFT)."""
    dev = amp.device
    S = int(num_samples)
    exc = torch.as_tensor(np.asarray(excitation, np.float64), device=dev).reshape(-1)
    if arrival.numel() == 0:
        return torch.zeros((n_src, n_snk, S, 3), dtype=torch.float64, device=dev), 1.0
    t0, wake = start_samples(arrival, pair[:, 0], n_src, n_snk, S, sampling_freq, map_bytes_limit)
    keep = t0 < S
    h = torch.zeros((n_src * n_snk * S, 3), dtype=torch.float64, device=dev)
    flat = (pair[:, 0].long() * n_snk + pair[:, 1].long()) * S + t0
    h.index_add_(0, flat[keep], amp[keep])
    h = h.reshape(n_src * n_snk, S, 3).permute(0, 2, 1)  # [series, 3, S]
    n = 1
    while n < S + exc.numel():
        n *= 2
    y = torch.fft.irfft(torch.fft.rfft(h, n=n) * torch.fft.rfft(exc, n=n), n=n)[..., :S]
    return y.permute(0, 2, 1).reshape(n_src, n_snk, S, 3).contiguous(), wake


def TimeDomainv3(source_num, sink_num, point_informationv2, full_index, scattering_coefficient, wavelength,
                 excitation_signal, sampling_freq, num_samples, alpha, beta):
    """(time_map float64 [source_num, sink_num, num_samples, 3], wake time float64) of
    lyceanem/electromagnetics/empropagation.py:2910-3170: wake times and source chunks as start_samples
    describes (the reference takes each wake with an atomic minimum that is only synchronised within a
    thread block, so its value there can depend on block scheduling; here it is taken first)."""
    del scattering_coefficient, wavelength  # unused by the reference's kernel
    pts = np.asarray(point_informationv2)
    pos = np.stack([pts["px"], pts["py"], pts["pz"]], 1).astype(np.float32)
    nrm = np.stack([pts["nx"], pts["ny"], pts["nz"]], 1).astype(np.float32)
    w = np.stack([pts["ex"], pts["ey"], pts["ez"]], 1).astype(np.complex64)
    magnetic = impedance = None
    if "Electric" in pts.dtype.names and not np.all(pts["Electric"]):
        magnetic = ~pts["Electric"].astype(bool)
        impedance = np.sqrt(np.real(pts["permeability"]).astype(np.float64)
                            / np.real(pts["permittivity"]).astype(np.float64)).astype(np.float32)
    amp, arrival, pair = path_times(full_index, pos, nrm, w, int(source_num), int(sink_num), alpha, beta, magnetic,
                                    impedance)
    tm, wake = time_map(amp, arrival, pair, int(source_num), int(sink_num), excitation_signal, sampling_freq,
                        num_samples)
    return tm.cpu().numpy(), np.float64(wake)
