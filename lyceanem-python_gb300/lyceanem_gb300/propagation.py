"""Torch-level API of the GB300 raycasting + propagation path.

All tensors live on the current CUDA device and every call is ordered on the
current torch stream.  Points are float32 [n,3]; complex 3-vectors are
complex64 [n,3]; packed triangles are float32 [T,12] (v0, 0, e1, 0, e2, 0).

Reference behaviour (paths within LyceanEM-Python):
  - visibility: lyceanem/src/raycasting.cuh:19-95 (hit, points_to_rays),
    lyceanem/src/raycasting_brute_force.cuh:19-88, raycasting_accelerated.cuh:106-482
  - field per pair: lyceanem/src/em.cuh:18-120
  - source sum: lyceanem/models/frequency_domain.py:847-849
  - one bounce: lyceanem/models/frequency_domain.py:195-264
"""
import ctypes
import math

import torch

from . import _native
from ._native import check, f32arr, i32arr, lib

EPSILON = 0.000001  # lyceanem/src/math_utility.cuh:9
NUMBA_EPSILON = 1e-7  # lyceanem/raycasting/rayfunctions.py:19


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _dev(t, dtype):
    if not isinstance(t, torch.Tensor):
        t = torch.as_tensor(t)
    if not t.is_cuda:
        t = t.cuda()
    return t.to(dtype).contiguous()


def _points(t):
    t = _dev(t, torch.float32)
    return t.reshape(-1, 3).contiguous()


def _cvec(t, n):
    """complex [n,3] (or [3], broadcast) -> complex64 [n,3] contiguous."""
    t = _dev(t, torch.complex64)
    if t.dim() == 1:
        t = t.reshape(1, 3).expand(n, 3)
    return t.reshape(n, 3).contiguous()


def _ws(nbytes, device):
    return torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device=device)


def pack_triangles(vertices, faces):
    """Mesh vertices [V,3] + triangle indices [T,3] -> packed triangles [T,12]."""
    v = _points(vertices)
    f = _dev(faces, torch.int32).reshape(-1, 3).contiguous()
    out = torch.empty((f.shape[0], 12), dtype=torch.float32, device=v.device)
    check(lib.lyem_pack_triangles(_p(v), v.shape[0], _p(f), f.shape[0], _p(out), _stream()), "pack_triangles")
    return out


def triangle_bounds(tris):
    """Axis-aligned bounds of packed triangles as a host list (xmin, ymin, zmin, xmax, ymax, zmax)."""
    b = torch.empty(6, dtype=torch.float32, device=tris.device)
    check(lib.lyem_tris_bounds(_p(tris), tris.shape[0], _p(b), _stream()), "tris_bounds")
    return b.cpu().tolist()


class UniformGrid:
    """Uniform 3-D grid over packed triangles, built on the device.

    cell: edge length of the cubic cells in metres (None picks about one cell
    per triangle).  The triangles are stored again in cell order so the DDA
    reads each cell's triangles as consecutive float4 loads."""

    def __init__(self, tris, cell=None):
        tris = _dev(tris, torch.float32).reshape(-1, 12).contiguous()
        self.tris = tris
        dev = tris.device
        bounds = triangle_bounds(tris) if tris.shape[0] else [0, 0, 0, 1, 1, 1]
        org = (ctypes.c_float * 3)()
        cell_out = ctypes.c_float()
        dims = (ctypes.c_int32 * 3)()
        check(lib.lyem_grid_plan(f32arr(bounds), tris.shape[0], float(cell or 0.0), org, ctypes.byref(cell_out), dims),
              "grid_plan")
        self.origin = [org[0], org[1], org[2]]
        self.cell = cell_out.value
        self.dims = [dims[0], dims[1], dims[2]]
        self.bounds = bounds
        T = tris.shape[0]
        offsets = torch.empty(T + 1, dtype=torch.int32, device=dev)
        total = torch.zeros(1, dtype=torch.int64, device=dev)
        ws = _ws(lib.lyem_grid_count_workspace(T), dev)
        check(lib.lyem_grid_count(_p(tris), T, f32arr(self.origin), self.cell, i32arr(self.dims), _p(offsets),
                                  _p(total), _p(ws), ws.numel(), _stream()), "grid_count")
        self.n_refs = int(total.item())
        ncells = self.dims[0] * self.dims[1] * self.dims[2]
        self.cell_start = torch.empty(ncells + 1, dtype=torch.int32, device=dev)
        self.cell_tris = torch.empty((max(self.n_refs, 1), 12), dtype=torch.float32, device=dev)
        # per cell two children (the cell's triangles split at its centre): (loA, first ref) (hiA, first ref
        # of B) (loB, first ref of B) (hiB, end ref), each box that of the child's triangles within the cell
        self.cell_box = torch.empty((ncells, 16), dtype=torch.float32, device=dev)
        ws2 = _ws(lib.lyem_grid_fill_workspace(self.n_refs, ncells), dev)
        check(lib.lyem_grid_fill(_p(tris), T, f32arr(self.origin), self.cell, i32arr(self.dims), _p(offsets),
                                 self.n_refs, _p(self.cell_start), _p(self.cell_tris), _p(self.cell_box), _p(ws2),
                                 ws2.numel(), _stream()), "grid_fill")
        self._org_c = f32arr(self.origin)
        self._dims_c = i32arr(self.dims)

    @property
    def n_cells(self):
        return self.dims[0] * self.dims[1] * self.dims[2]

    @property
    def centre(self):
        """Centre of the grid box (the direction origin for far sinks, see direction_order)."""
        return [self.origin[k] + 0.5 * self.dims[k] * self.cell for k in range(3)]


class StageResult:
    __slots__ = ("sink", "pairs", "mask_bits", "counters", "n_src", "n_snk")

    def __init__(self, sink, pairs, mask_bits, counters, n_src, n_snk):
        self.sink, self.pairs, self.mask_bits, self.counters = sink, pairs, mask_bits, counters
        self.n_src, self.n_snk = n_src, n_snk

    def mask(self):
        """Visibility as a bool tensor [n_src, n_snk]."""
        out = torch.empty((self.n_src, self.n_snk), dtype=torch.uint8, device=self.mask_bits.device)
        check(lib.lyem_mask_to_bytes(_p(self.mask_bits), self.n_src, self.n_snk, _p(out), _stream()), "mask_to_bytes")
        return out.bool()


def _check_buffer(name, t, dtype, n, exact):
    """Caller-provided device buffer of the stage: a contiguous 1-D CUDA tensor of `dtype` with exactly
    (exact) or at least n entries; the kernels index it without bounds checks."""
    if t is None:
        return
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == dtype and t.dim() == 1 and t.is_contiguous()):
        raise ValueError(f"{name} must be a contiguous 1-D {dtype} CUDA tensor")
    if (t.numel() != n) if exact else (t.numel() < n):
        raise ValueError(f"{name} has {t.numel()} entries, {'' if exact else 'at least '}{n} needed")


def pair_stage(src_pos, src_E, snk_pos, snk_nrm, *, beta, alpha=0.0, tris=None, grid=None, src_W=None,
               self_to_self=False, cull=True, eps=EPSILON, sink_out=None, accumulate=False, want_pairs=False,
               want_mask=False, counters=None, src_visible=None, snk_visible=None, src_order=None, snk_order=None,
               src_chunk=0, traversal=0, workspace=None):
    """Visibility + fused field of every (source, sink) pair.

    Returns a StageResult whose .sink is complex64 [n_snk,3] with
        sink[m, c] (+)= sum_n W[n, c] * S[n, m, c]
    (W = src_W or 1), .pairs the per-pair network complex64 [n_src,n_snk,3]
    when want_pairs, and .mask_bits the visibility bit mask when want_mask.
    counters (int64 [2]) accumulates (visible pairs, ray/triangle tests);
    src_visible / snk_visible (int32 [n_src] / [n_snk]) accumulate visible pairs
    per source / per sink.
    src_order / snk_order (int32, e.g. from spatial_order) set the processing
    order only: which sources share a thread block and which sinks a warp.
    A src_order shorter than src_pos selects a subset: only the sources it
    lists (distinct rows) are traced, and the per-source outputs keep one row
    per row of src_pos (zero for the rows left out).
    src_chunk / traversal choose the launch shape and the ray schedule of the
    grid kernel (0 = automatic; see lyem_pair_stage in include/lyem.h).
    Visibility uses `grid` (a UniformGrid) if given, else brute force over
    `tris`.  self_to_self=False reproduces the reference's untested pair
    n == m (lyceanem/src/raycasting_brute_force.cuh:27)."""
    sp = _points(src_pos)
    dev = sp.device
    rows = sp.shape[0]
    N = rows if src_order is None else int(src_order.shape[0])
    if N > rows:
        raise ValueError(f"src_order lists {N} sources for {rows} rows")
    E = _cvec(src_E, rows)
    W = None if src_W is None else _cvec(src_W, rows)
    tp = _points(snk_pos)
    tn = _points(snk_nrm)
    M = tp.shape[0]
    _check_buffer("src_order", src_order, torch.int32, N, True)
    _check_buffer("snk_order", snk_order, torch.int32, M, True)
    _check_buffer("src_visible", src_visible, torch.int32, rows, False)
    _check_buffer("snk_visible", snk_visible, torch.int32, M, False)
    _check_buffer("counters", counters, torch.int64, 2, False)
    if grid is not None:
        tri_t, T = None, 0
        cs, ct, cb = grid.cell_start, grid.cell_tris, grid.cell_box
        org, cell, dims = grid._org_c, grid.cell, grid._dims_c
    else:
        tri_t = _dev(tris, torch.float32).reshape(-1, 12).contiguous() if tris is not None else \
            torch.zeros((0, 12), dtype=torch.float32, device=dev)
        T = tri_t.shape[0]
        cs = ct = cb = None
        org, cell, dims = f32arr([0, 0, 0]), 1.0, i32arr([1, 1, 1])
    if sink_out is None:
        sink_out = torch.empty((M, 3), dtype=torch.complex64, device=dev)
        accumulate = False
    alloc = torch.empty if N == rows else torch.zeros  # rows left out of a subset stay zero
    pairs = alloc((rows, M, 3), dtype=torch.complex64, device=dev) if want_pairs else None
    words = (M + 31) // 32
    mbits = alloc((rows, words), dtype=torch.int32, device=dev) if want_mask else None
    # the transposed schedule (traversal 38) takes 32 sources per block, whatever src_chunk says
    wchunk = 32 if (grid is not None and traversal == 38) else int(src_chunk)
    need = lib.lyem_pair_stage_workspace(N, M, T, int(grid is not None), wchunk)
    if workspace is None or workspace.numel() < need:
        workspace = _ws(need, dev)
    st = lib.lyem_pair_stage(_p(sp), _p(torch.view_as_real(E)), _p(None if W is None else torch.view_as_real(W)), N,
                             _p(tp), _p(tn), M, _p(tri_t), T, _p(cs), _p(ct), _p(cb), org, float(cell), dims,
                             float(alpha),
                             float(beta), int(bool(self_to_self)), int(bool(cull)), float(eps),
                             _p(torch.view_as_real(sink_out)), int(bool(accumulate)),
                             _p(None if pairs is None else torch.view_as_real(pairs)), _p(mbits), _p(counters),
                             _p(src_visible), _p(snk_visible), _p(src_order), _p(snk_order), int(src_chunk),
                             int(traversal), _p(workspace), workspace.numel(), _stream())
    check(st, "pair_stage")
    return StageResult(sink_out, pairs, mbits, counters, rows, M)


def spatial_order(points):
    """Morton order of a point set (int32 permutation, on the device)."""
    pts = _points(points)
    n = pts.shape[0]
    out = torch.empty(n, dtype=torch.int32, device=pts.device)
    if n:
        ws = _ws(lib.lyem_spatial_order_workspace(n), pts.device)
        check(lib.lyem_spatial_order(_p(pts), n, _p(out), _p(ws), ws.numel(), _stream()), "spatial_order")
    return out


def source_schedule(src, grid):
    """Grid schedule for a source set: the transposed one (traversal 38: the lanes of a warp are 32 sources,
    the warp walks one sink at a time) when every source lies within one grid cell of every other (the
    elements of an array), so that a warp's rays to a sink cross the same cells; otherwise the default (0).
    Meant for the source-summed field: with a per-pair network output the transposed schedule's pair writes
    are strided.  A device tensor is reduced on the device (one small synchronisation)."""
    if grid is None:
        return 0
    if isinstance(src, torch.Tensor):
        a = src.reshape(-1, 3)
        if a.shape[0] == 0:
            return 0
        lo, hi = torch.aminmax(a.float(), dim=0)
        ext = (hi - lo).double().cpu().numpy()
    else:
        import numpy as np
        a = np.asarray(src, np.float64).reshape(-1, 3)
        if a.shape[0] == 0:
            return 0
        ext = a.max(0) - a.min(0)
    return 38 if float((ext ** 2).sum()) ** 0.5 <= grid.cell else 0


def direction_order(points, centre):
    """Order of a point set by direction seen from `centre` (Z-order of elevation and azimuth; int32
    permutation on the device).  For far sinks it puts rays of nearly one direction in a warp."""
    pts = _points(points)
    n = pts.shape[0]
    out = torch.empty(n, dtype=torch.int32, device=pts.device)
    if n:
        ws = _ws(lib.lyem_spatial_order_workspace(n), pts.device)
        check(lib.lyem_direction_order(_p(pts), n, f32arr([float(c) for c in centre]), _p(out), _p(ws), ws.numel(),
                                       _stream()), "direction_order")
    return out


def device_errors():
    """Synchronise the current stream and read/clear the device error word."""
    flags = ctypes.c_uint32()
    st = lib.lyem_device_errors(_stream(), ctypes.byref(flags))
    return st, flags.value


def kernel_launches():
    """Cumulative number of kernels launched by liblyem_gpu.so in this process."""
    return int(lib.lyem_kernel_launches())


def fp32_fma_rate(iterations=1 << 16):
    """Measured FP32 FMA lane-operations per second of the current device."""
    out = ctypes.c_double()
    check(lib.lyem_fp32_fma_probe(int(iterations), ctypes.byref(out), _stream()), "fp32_fma_probe")
    return out.value


def wavenumber(wavelength):
    return 2.0 * math.pi / wavelength
