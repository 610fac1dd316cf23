"""Drop-in for the reference's pybind11 module `lyceanem.em`.

Same four functions, same positional arguments, same return layout as
lyceanem/src/frequency_domain_models.cu:314-320, running on liblyem_gpu.so
through its host-buffer entry points (lyem_em_* in include/lyem.h).  Inputs
are converted like pybind11's array_t<float>/array_t<int> (dtype cast,
C-contiguous); shape errors raise RuntimeError with the reference's messages.
"""
import ctypes

import numpy as np

from ._native import check, lib


def _f(a):
    return np.ascontiguousarray(np.asarray(a), dtype=np.float32)


def _i(a):
    return np.ascontiguousarray(np.asarray(a), dtype=np.int32)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _need(cond, msg):
    if not cond:
        raise RuntimeError(msg)


def _check_points(name, a):
    _need(a.ndim == 2 and a.shape[1] == 3, f"{name} must be a 2D array with 3 columns")


def _check_e(arrs, n):
    names = ["ex_real", "ex_imag", "ey_real", "ey_imag", "ez_real", "ez_imag"]
    for nm, a in zip(names, arrs):
        _need(a.ndim == 1, f"{nm} must be a 1D array")
    for nm, a in zip(names, arrs):
        _need(a.shape[0] == n, f"Mismatch: {nm}.shape(0) != source_size")


def calculate_scattering_tiles(source, end, triangle_vertex, wave_length, ex_real, ex_imag, ey_real, ey_imag,
                               ez_real, ez_imag, normal, xmin, xmax, ymin, ymax, zmin, zmax, tile_size, bin_count,
                               bin_triangles, n_cellsx, n_cellsy, binned_tri_num, alpha, beta, not_self_to_self):
    """Per-pair scattering network, float32 [N*M*6] (lyceanem/src/frequency_domain_models.cu:44-187)."""
    src, snk, tv = _f(source), _f(end), _f(triangle_vertex)
    es = [_f(a) for a in (ex_real, ex_imag, ey_real, ey_imag, ez_real, ez_imag)]
    nrm, bc, bt = _f(normal), _i(bin_count), _i(bin_triangles)
    _check_points("source", src)
    _check_points("end", snk)
    _check_points("triangle_vertex", tv)
    _need(nrm.ndim == 2 and nrm.shape[1] == 3, "normal must be a 2D array with 3 columns")
    _need(bc.ndim == 1, "bin_count must be a 1D array")
    _need(bt.ndim == 1, "bin_triangles must be a 1D array")
    _need(bc.shape[0] == n_cellsx * n_cellsy, "bin_count must have n_cellsx * n_cellsy elements")
    _need(bt.shape[0] == binned_tri_num * 3, "bin_triangles 3* bintrinum elements")
    N, M = src.shape[0], snk.shape[0]
    _check_e(es, N)
    _need(nrm.shape[0] == N + M, "Mismatch: normal.shape(0) != points_size")
    out = np.zeros(N * M * 6, dtype=np.float32)
    st = lib.lyem_em_calculate_scattering_tiles(
        _p(src), N, _p(snk), M, _p(tv), tv.shape[0], float(wave_length), *[_p(a) for a in es], _p(nrm), float(xmin),
        float(xmax), float(ymin), float(ymax), float(zmin), float(zmax), float(tile_size), _p(bc), _p(bt),
        int(n_cellsx), int(n_cellsy), int(binned_tri_num), float(alpha), float(beta), int(bool(not_self_to_self)),
        _p(out))
    check(st, "calculate_scattering_tiles")
    return out


def calculate_scattering_brute_force(source, end, triangles, triangle_vertex, wave_length, ex_real, ex_imag, ey_real,
                                     ey_imag, ez_real, ez_imag, normal, alpha, beta, not_self_to_self):
    """Per-pair scattering network, float32 [N*M*6] (lyceanem/src/frequency_domain_models.cu:190-311)."""
    src, snk, tri, tv = _f(source), _f(end), _i(triangles), _f(triangle_vertex)
    es = [_f(a) for a in (ex_real, ex_imag, ey_real, ey_imag, ez_real, ez_imag)]
    nrm = _f(normal)
    _check_points("source", src)
    _check_points("end", snk)
    _need(tri.ndim == 2 and tri.shape[1] == 3, "triangles must be a 2D array with 3 columns")
    _check_points("triangle_vertex", tv)
    _need(nrm.ndim == 2 and nrm.shape[1] == 3, "normal must be a 2D array with 3 columns")
    N, M = src.shape[0], snk.shape[0]
    _check_e(es, N)
    _need(nrm.shape[0] == N + M, "Mismatch: normal.shape(0) != points_size")
    out = np.zeros(N * M * 6, dtype=np.float32)
    st = lib.lyem_em_calculate_scattering_brute_force(
        _p(src), N, _p(snk), M, _p(tri), tri.shape[0], _p(tv), tv.shape[0], float(wave_length),
        *[_p(a) for a in es], _p(nrm), float(alpha), float(beta), int(bool(not_self_to_self)), _p(out))
    check(st, "calculate_scattering_brute_force")
    return out


def bin_counts_to_numpy(tri_vertex, tri_index, ncells_x, ncells_y, ymin, cell_width, z_min):
    """Triangles per y-z cell, int32 [ncells_x*ncells_y] (lyceanem/src/terrain_acceleration_build.cuh:296-348)."""
    tv, ti = _f(tri_vertex), _i(tri_index)
    _need(tv.ndim == 2 and tv.shape[1] == 3, "tri_vertex must be a 2D array with 3 columns")
    _need(ti.ndim == 2 and ti.shape[1] == 3, "tri_index must be a 2D array with 3 columns")
    out = np.zeros(int(ncells_x) * int(ncells_y), dtype=np.int32)
    st = lib.lyem_em_bin_counts(_p(tv), tv.shape[0], _p(ti), ti.shape[0], int(ncells_x), int(ncells_y), float(ymin),
                                float(cell_width), float(z_min), _p(out))
    check(st, "bin_counts_to_numpy")
    return out


def bin_triangles_to_numpy(tri_vertex, tri_index, ncells_x, ncells_y, ymin, cell_width, z_min, bin_counts,
                           sum_bin_counts):
    """Vertex-index triples of the binned triangles in cell order, int32 [3*sum_bin_counts]
    (lyceanem/src/terrain_acceleration_build.cuh:370-431)."""
    tv, ti, bc = _f(tri_vertex), _i(tri_index), _i(bin_counts)
    _need(tv.ndim == 2 and tv.shape[1] == 3, "tri_vertex must be a 2D array with 3 columns")
    _need(ti.ndim == 2 and ti.shape[1] == 3, "tri_index must be a 2D array with 3 columns")
    _need(bc.ndim == 1 and bc.shape[0] == ncells_x * ncells_y,
          "bincounts is a 1d flattened 2d array thus must have 1d with ncountsy *ncountz")
    out = np.zeros(3 * int(sum_bin_counts), dtype=np.int32)
    st = lib.lyem_em_bin_triangles(_p(tv), tv.shape[0], _p(ti), ti.shape[0], int(ncells_x), int(ncells_y),
                                   float(ymin), float(cell_width), float(z_min), _p(bc), int(sum_bin_counts), _p(out))
    check(st, "bin_triangles_to_numpy")
    return out
