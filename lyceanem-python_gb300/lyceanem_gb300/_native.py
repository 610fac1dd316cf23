"""ctypes binding of liblyem_gpu.so (the C ABI declared in include/lyem.h).

The library is the only compute path of this package: if it is missing the
import of this module raises, there is no fallback.
"""
import ctypes
import os
import re

from . import build as _build

LIB_PATH = _build.LIB_PATH
HEADER = os.path.join(_build.INCLUDE, "lyem.h")

LYEM_OK = 0
LYEM_ERR_INVALID = 1
LYEM_ERR_CUDA = 2
LYEM_ERR_NOMEM = 3
LYEM_ERR_TIMEOUT = 4
LYEM_ERR_OVERFLOW = 5
LYEM_ERR_WORKSPACE = 6


class LyemError(RuntimeError):
    """A non-zero status returned by liblyem_gpu.so."""

    def __init__(self, status, where):
        self.status = status
        msg = _lib.lyem_status_string(status).decode() if _lib is not None else str(status)
        extra = ""
        if status == LYEM_ERR_CUDA and _lib is not None:
            extra = f" (cudaError {_lib.lyem_last_cuda_error()})"
        super().__init__(f"{where}: {msg}{extra}")


_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_f32 = ctypes.c_float
_f64 = ctypes.c_double
_sz = ctypes.c_size_t
_f32p = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u32p = ctypes.POINTER(ctypes.c_uint32)

class BatchScene(ctypes.Structure):
    """lyem_batch_scene of include/lyem.h (device pointers and sizes of one scene)."""
    _fields_ = [("src_pos", _vp), ("src_E", _vp), ("scat_pos", _vp), ("scat_nrm", _vp), ("scat_id", _vp),
                ("cell_start", _vp), ("cell_tris", _vp), ("cell_box", _vp), ("n_src", _i64), ("n_scat", _i64),
                ("grid_origin", _f32 * 3), ("grid_cell", _f32), ("grid_dims", _i32 * 3), ("reserved", _i32)]


class BatchConfig(ctypes.Structure):
    """lyem_batch_config of include/lyem.h."""
    _fields_ = [("freq_group", _i32), ("src_chunk", _i32), ("blocks_per_sm", _i32), ("cull", _i32), ("eps", _f32),
                ("self_to_self", _i32), ("alpha", _f64)]


_scp = ctypes.POINTER(BatchScene)
_cfgp = ctypes.POINTER(BatchConfig)
_f64p = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)

# argument types of every entry point of include/lyem.h
SIGNATURES = {
    "lyem_version": ([], ctypes.c_int),
    "lyem_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "lyem_last_cuda_error": ([], ctypes.c_int),
    "lyem_kernel_launches": ([], ctypes.c_uint64),
    "lyem_fp32_fma_probe": ([_i64, ctypes.POINTER(ctypes.c_double), _vp], ctypes.c_int),
    "lyem_device_errors": ([_vp, _u32p], ctypes.c_int),
    "lyem_pack_triangles": ([_vp, _i64, _vp, _i64, _vp, _vp], ctypes.c_int),
    "lyem_tris_bounds": ([_vp, _i64, _vp, _vp], ctypes.c_int),
    "lyem_grid_plan": ([_f32p, _i64, _f32, _f32p, _f32p, _i32p], ctypes.c_int),
    "lyem_grid_count_workspace": ([_i64], _sz),
    "lyem_grid_count": ([_vp, _i64, _f32p, _f32, _i32p, _vp, _vp, _vp, _sz, _vp], ctypes.c_int),
    "lyem_grid_fill_workspace": ([_i64, _i64], _sz),
    "lyem_grid_fill": ([_vp, _i64, _f32p, _f32, _i32p, _vp, _i64, _vp, _vp, _vp, _vp, _sz, _vp], ctypes.c_int),
    "lyem_spatial_order_workspace": ([_i64], _sz),
    "lyem_spatial_order": ([_vp, _i64, _vp, _vp, _sz, _vp], ctypes.c_int),
    "lyem_direction_order": ([_vp, _i64, _f32p, _vp, _vp, _sz, _vp], ctypes.c_int),
    "lyem_pair_stage_workspace": ([_i64, _i64, _i64, _i32, _i32], _sz),
    "lyem_pair_stage": ([_vp, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _vp, _vp, _f32p, _f32, _i32p, _f64, _f64,
                         _i32, _i32, _f32, _vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _vp, _sz,
                         _vp],
                        ctypes.c_int),
    "lyem_pair_stage_noalloc_scratch_bytes": ([], _sz),
    "lyem_pair_stage_noalloc": ([_vp, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _vp, _vp, _f32p, _f32, _i32p, _f64,
                                 _f64, _i32, _i32, _f32, _vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32,
                                 _vp], ctypes.c_int),
    "lyem_mask_to_bytes": ([_vp, _i64, _i64, _vp, _vp], ctypes.c_int),
    "lyem_adjoint_workspace": ([_i64, _i64, _i64], _sz),
    "lyem_adjoint": ([_vp, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _f64, _f64, _vp,
                      _vp, _vp, _vp, _vp, _sz, _vp], ctypes.c_int),
    "lyem_sweep_network_bytes": ([_i64, _i64, _i32], _sz),
    "lyem_sweep_weights_bytes": ([_i64, _i64, _i32], _sz),
    "lyem_sweep_prepare_network": ([_vp, _i64, _i64, _i32, _i64, _vp, _vp], ctypes.c_int),
    "lyem_sweep_prepare_weights": ([_vp, _i64, _i64, _i32, _vp, _vp], ctypes.c_int),
    "lyem_sweep_workspace_bytes": ([_i64, _i64, _i32], _sz),
    "lyem_sweep_run_ws": ([_vp, _i64, _i64, _i64, _vp, _vp, _i64, _i32, _vp, _i64, _vp, _sz, _vp], ctypes.c_int),
    "lyem_sweep_run": ([_vp, _i64, _i64, _i64, _vp, _vp, _i64, _i32, _vp, _i64, _vp], ctypes.c_int),
    "lyem_sweep_set_k_tile": ([_i32], ctypes.c_int),
    "lyem_sweep_set_multicast": ([_i32], ctypes.c_int),
    "lyem_batch_workspace": ([_scp, _i32, _i64, _i32, _cfgp], _sz),
    "lyem_batch_items": ([_scp, _i32, _i64, _i32, _cfgp, _i64p], ctypes.c_int64),
    "lyem_batch_prepare": ([_scp, _i32, _i64, _f64p, _i32, _cfgp, _vp, _sz, _vp], ctypes.c_int),
    "lyem_batch_launch": ([_scp, _i32, _vp, _vp, _vp, _i64, _f64p, _i32, _cfgp, _vp, _sz, _vp, _vp, _i32p, _vp],
                          ctypes.c_int),
    "lyem_tangential_project": ([_vp, _vp, _i64, _vp], ctypes.c_int),
    "lyem_path_field": ([_vp, _i64, _i32, _vp, _vp, _vp, _vp, _vp, _i64, _i64, _i64, _f64, _f64, _vp, _vp],
                        ctypes.c_int),
    "lyem_path_time": ([_vp, _i64, _i32, _vp, _vp, _vp, _vp, _vp, _i64, _i64, _i64, _f64, _f64, _vp, _vp, _vp, _vp],
                       ctypes.c_int),
    "lyem_em_bin_counts": ([_vp, _i64, _vp, _i64, _i32, _i32, _f32, _f32, _f32, _vp], ctypes.c_int),
    "lyem_em_bin_triangles": ([_vp, _i64, _vp, _i64, _i32, _i32, _f32, _f32, _f32, _vp, _i64, _vp], ctypes.c_int),
    "lyem_em_calculate_scattering_brute_force": (
        [_vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _f32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _f32, _f32, _i32, _vp],
        ctypes.c_int),
    "lyem_em_calculate_scattering_tiles": (
        [_vp, _i64, _vp, _i64, _vp, _i64, _f32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _f32, _f32, _f32, _f32, _f32, _f32,
         _f32, _vp, _vp, _i32, _i32, _i32, _f32, _f32, _i32, _vp], ctypes.c_int),
}

_lib = None


def header_symbols():
    """Names of the entry points declared in include/lyem.h."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"LYEM_API[^;(]*?\b(lyem_\w+)\s*\(", text, flags=re.S)))


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"liblyem_gpu.so is not built ({LIB_PATH}); run lyceanem_gb300.build.build_native()")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(status, where):
    if status != LYEM_OK:
        raise LyemError(status, where)


def f32arr(values):
    arr = (ctypes.c_float * len(values))(*[float(v) for v in values])
    return arr


def i32arr(values):
    return (ctypes.c_int32 * len(values))(*[int(v) for v in values])


lib = load()
