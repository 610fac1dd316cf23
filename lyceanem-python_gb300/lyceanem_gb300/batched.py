"""Many scenes x many frequencies, direct + one-bounce paths, in one persistent launch.

For every scene s and frequency f, BatchedScattering evaluates the sink field
of calculate_scattering_cuda (lyceanem/models/frequency_domain.py:195-264)
summed over the sources (:847-849):

    E[s, f, m] = sum_n S0_f(n, m) + sum_p e_p(f) (.) S2_f(p, m; e_p(f)),
    e_p(f)     = sum_n S1_f(n, p),

with the per-pair field of lyceanem/src/em.cuh:18-120 at beta_f = 2 pi f / c
and the visibility of lyceanem/src/raycasting.cuh:19-95 (resolved once for
all frequencies).  One launch (two memsets and one persistent kernel) covers
the whole batch; `capture()` records it in a CUDA graph that `run()` replays.
`autotune()` picks the frequencies per thread (which sets the sinks of a field
tile, 256 / ceil(F / group)), the sources per visibility item (the rays of a
block's tile) and the resident blocks per SM by timing the candidates on the
batch itself, and remembers the choice in a JSON cache keyed by the device and
the batch's sizes.  Given cell_scales it also picks the grid's cell edge per
scene, k * (box volume / triangles)^(1/3) with one k for the batch: visibility,
and so the field, is the same for every grid; only the traversal work changes.
"""
import ctypes
import hashlib
import json
import os

import numpy as np
import torch

from . import propagation as P
from ._native import BatchConfig, BatchScene, LyemError, check, lib

C0 = 299792458.0

# (frequencies per thread, sources per visibility item, blocks per SM).  Blocks per
# SM 3, 4, 6 or 8 select kernel variants whose registers are capped for that
# occupancy; 0 runs the uncapped variant with as many blocks as fit.  On the
# 64-scene batch with one 0.5 m cell (4.0e9 ray pairs, 9.9e11 ray-triangle tests) one launch took
# 5.41 s at (4, 64, 4) and 4.49 / 5.36 / 4.71 s at (2 / 1 / 4, 64, 8): the
# visibility phase dominates and gains from the extra resident warps more
# than the field phase loses to spilling.
CANDIDATES = [(2, 64, 8), (2, 64, 6), (1, 64, 8), (4, 64, 8), (2, 32, 8), (4, 64, 4), (4, 32, 3), (8, 32, 3),
              (4, 32, 0)]
DEFAULT = (2, 64, 8)


def stratified_subset(scenes, n_sinks, every=4):
    """Indices of every `every`-th scene in order of estimated work (N*M + N*P + P*M): a proxy
    batch that spans the batch's range of scene sizes, for the autotuner."""
    def cost(sc):
        N = np.asarray(sc.src).shape[0]
        Pn = 0 if getattr(sc, "scat", None) is None else np.asarray(sc.scat).shape[0]
        return N * n_sinks + N * Pn + Pn * n_sinks
    order = sorted(range(len(scenes)), key=lambda i: -cost(scenes[i]))
    return order[::every]


def _cache_path():
    return os.environ.get("LYEM_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "lyceanem_gb300", "batch_tune.json"))


def betas_of(frequencies):
    return 2.0 * np.pi * np.asarray(frequencies, np.float64) / C0


def is_uniform(betas):
    b = np.asarray(betas, np.float64)
    if b.size < 2:
        return True
    d = (b[-1] - b[0]) / (b.size - 1)
    dev = np.abs(b - (b[0] + d * np.arange(b.size))).max()
    return bool(dev <= 1e-12 * max(np.abs(b).max(), 1.0))


def density_cell(bounds, n_tris, scale):
    """Grid cell edge for a scene: scale * (volume of the triangles' box / triangle count)^(1/3),
    i.e. about scale^-3 triangles per cell, clipped to [0.05, 10] m."""
    lo, hi = np.asarray(bounds[:3], np.float64), np.asarray(bounds[3:], np.float64)
    vol = float(np.prod(np.maximum(hi - lo, 1e-3)))
    return float(np.clip(scale * (vol / max(int(n_tris), 1)) ** (1.0 / 3.0), 0.05, 10.0))


class _SceneData:
    """Device-resident data of one scene: sources, mesh grid, scatter points in Morton order."""

    def __init__(self, src, E, verts, faces, scat, scat_n, grid_cell):
        self.src = P._points(src)
        n = self.src.shape[0]
        self.E = P._cvec(E if E is not None else np.array([1.0, 0.0, 0.0]), n)
        self.Ef = torch.view_as_real(self.E).reshape(n, 6).contiguous()
        tris = P.pack_triangles(verts, faces)
        self.n_tris = tris.shape[0]
        if callable(grid_cell):
            grid_cell = grid_cell(P.triangle_bounds(tris) if self.n_tris else [0, 0, 0, 1, 1, 1], self.n_tris)
        self.grid = P.UniformGrid(tris, cell=grid_cell)
        if scat is not None and len(scat):
            s = P._points(scat)
            sn = P._points(scat_n)
            order = P.spatial_order(s)
            self.scat_id = order
            self.scat = s.index_select(0, order.long()).contiguous()
            self.scat_n = sn.index_select(0, order.long()).contiguous()
        else:
            self.scat_id = torch.zeros(1, dtype=torch.int32, device=self.src.device)
            self.scat = torch.zeros((0, 3), dtype=torch.float32, device=self.src.device)
            self.scat_n = torch.zeros((0, 3), dtype=torch.float32, device=self.src.device)

    def struct(self):
        g = self.grid
        b = BatchScene()
        b.src_pos = self.src.data_ptr()
        b.src_E = self.Ef.data_ptr()
        b.scat_pos = self.scat.data_ptr() if self.scat.shape[0] else None
        b.scat_nrm = self.scat_n.data_ptr() if self.scat.shape[0] else None
        b.scat_id = self.scat_id.data_ptr() if self.scat.shape[0] else None
        b.cell_start = g.cell_start.data_ptr()
        b.cell_tris = g.cell_tris.data_ptr()
        b.cell_box = g.cell_box.data_ptr()
        b.n_src = self.src.shape[0]
        b.n_scat = self.scat.shape[0]
        for k in range(3):
            b.grid_origin[k] = g.origin[k]
            b.grid_dims[k] = g.dims[k]
        b.grid_cell = g.cell
        return b


class BatchedScattering:
    """Direct + one-bounce sink fields of many scenes at many frequencies.

    grid_cell: the grid's cell edge in metres, one value or one per scene (None: about one cell per
      triangle).  cell_scale k (instead): per-scene cells from the scene's triangle density,
      k * (box volume / triangles)^(1/3) (density_cell); autotune() can choose k.
    scenes: sequence of objects with attributes (or dict keys) src [N,3],
      verts [V,3], faces [T,3], optionally E [N,3] complex (default +x),
      scat [P,3] and scat_n [P,3] (scatter points and normals; P may be 0).
    sinks, sink_normals: [M,3], shared by all scenes; processed in direction order seen from their
      centroid (sink_order="direction", for far-field spheres) or in Morton order ("spatial").
    frequencies (Hz) or betas (rad/m): the frequency list, shared by all scenes.
    Output of run(): complex64 [n_scenes, n_freq, M, 3] on the device."""

    def __init__(self, scenes, sinks, sink_normals, frequencies=None, *, betas=None, alpha=0.0, grid_cell=0.5,
                 self_to_self=False, cull=True, eps=P.EPSILON, config=None, cell_scale=None, sink_order="direction"):
        if betas is None:
            betas = betas_of(frequencies)
        self.betas = np.ascontiguousarray(np.asarray(betas, np.float64).ravel())
        self.uniform = is_uniform(self.betas)
        self.alpha, self.self_to_self, self.cull, self.eps = float(alpha), bool(self_to_self), bool(cull), float(eps)

        def get(s, k):
            if isinstance(s, dict):
                return s.get(k)
            return getattr(s, k, None)

        scenes = list(scenes)
        if cell_scale is not None:
            grid_cell = lambda bounds, n_tris: density_cell(bounds, n_tris, cell_scale)  # noqa: E731
        cells = list(grid_cell) if isinstance(grid_cell, (list, tuple, np.ndarray)) else [grid_cell] * len(scenes)
        if len(cells) != len(scenes):
            raise ValueError("grid_cell: one value, or one per scene")
        self.data = [_SceneData(get(s, "src"), get(s, "E"), get(s, "verts"), get(s, "faces"), get(s, "scat"),
                                get(s, "scat_n"), c) for s, c in zip(scenes, cells)]
        snk = P._points(sinks)
        snk_n = P._points(sink_normals)
        if sink_order == "direction":  # warps of sinks in one direction from the sinks' centroid
            self.snk_id = P.direction_order(snk, snk.double().mean(0).tolist())
        else:
            self.snk_id = P.spatial_order(snk)
        self.snk = snk.index_select(0, self.snk_id.long()).contiguous()
        self.snk_n = snk_n.index_select(0, self.snk_id.long()).contiguous()
        self.n_scenes, self.n_freq, self.n_snk = len(self.data), self.betas.size, snk.shape[0]
        self.device = snk.device
        self._structs = (BatchScene * self.n_scenes)(*[d.struct() for d in self.data])
        self._beta_c = self.betas.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self.field = torch.empty((self.n_scenes, self.n_freq, self.n_snk, 3), dtype=torch.complex64,
                                 device=self.device)
        self.counters = torch.zeros((self.n_scenes, 4), dtype=torch.int64, device=self.device)
        self.graph = None
        self.ws = None
        self.blocks = 0
        self.cell_scale = None if cell_scale is None else float(cell_scale)
        self.configure(config if config is not None else self._default())

    def set_cell_scale(self, scale):
        """Rebuild every scene's grid with the density rule at `scale` (density_cell) and rewrite the
        work list; results do not depend on the grid, only the traversal work does."""
        for d in self.data:
            g = d.grid
            d.grid = P.UniformGrid(g.tris, cell=density_cell(g.bounds, d.n_tris, scale))
        self.cell_scale = float(scale)
        self._structs = (BatchScene * self.n_scenes)(*[d.struct() for d in self.data])
        self.configure(self.config)

    def grid_cells(self):
        return [d.grid.cell for d in self.data]

    # ------------------------------------------------------------ configuration

    def _default(self):
        return DEFAULT if self.uniform else (1, DEFAULT[1], DEFAULT[2])

    def _cfg(self, c):
        cfg = BatchConfig()
        cfg.freq_group, cfg.src_chunk, cfg.blocks_per_sm = int(c[0]), int(c[1]), int(c[2])
        cfg.cull = 1 if self.cull else 0
        cfg.eps = self.eps
        cfg.self_to_self = 1 if self.self_to_self else 0
        cfg.alpha = self.alpha
        return cfg

    def configure(self, c):
        """Select (frequencies per thread, sources per visibility item, blocks per SM) and write the work list."""
        c = tuple(int(v) for v in c)
        if c[0] > 1 and not self.uniform:
            raise ValueError("frequency groups above 1 need a uniformly spaced frequency list")
        self.config = c
        self._cfg_c = self._cfg(c)
        nbytes = lib.lyem_batch_workspace(self._structs, self.n_scenes, self.n_snk, self.n_freq,
                                          ctypes.byref(self._cfg_c))
        if nbytes == 0:
            raise LyemError(1, "batch_workspace")
        if self.ws is None or self.ws.numel() < nbytes:
            self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        check(lib.lyem_batch_prepare(self._structs, self.n_scenes, self.n_snk, self._beta_c, self.n_freq,
                                     ctypes.byref(self._cfg_c), ctypes.c_void_p(self.ws.data_ptr()), self.ws.numel(),
                                     P._stream()), "batch_prepare")
        self.graph = None

    def items(self):
        """Work items of the launch per kind: visibility (sources->scatter, sources->sinks,
        scatter->sinks), scatter fields, sink fields."""
        per = (ctypes.c_int64 * 5)()
        n = lib.lyem_batch_items(self._structs, self.n_scenes, self.n_snk, self.n_freq, ctypes.byref(self._cfg_c),
                                 per)
        if n < 0:
            raise LyemError(int(-n), "batch_items")
        return list(per)

    # ------------------------------------------------------------ execution

    def launch(self):
        """One launch on the current stream (no allocation, no synchronisation)."""
        blocks = ctypes.c_int32()
        check(lib.lyem_batch_launch(self._structs, self.n_scenes, ctypes.c_void_p(self.snk.data_ptr()),
                                    ctypes.c_void_p(self.snk_n.data_ptr()), ctypes.c_void_p(self.snk_id.data_ptr()),
                                    self.n_snk, self._beta_c, self.n_freq, ctypes.byref(self._cfg_c),
                                    ctypes.c_void_p(self.ws.data_ptr()), self.ws.numel(),
                                    ctypes.c_void_p(self.field.data_ptr()), ctypes.c_void_p(self.counters.data_ptr()),
                                    ctypes.byref(blocks), P._stream()), "batch_launch")
        self.blocks = blocks.value
        return self.field

    def capture(self):
        """Record the launch in a CUDA graph (after one eager launch, which sets the kernel attributes)."""
        self.launch()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch()
        self.graph = g
        return g

    def run(self):
        """The batch's fields, complex64 [n_scenes, n_freq, M, 3] (graph replay when captured)."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launch()
        return self.field

    # ------------------------------------------------------------ accounting

    def paths(self):
        """Paths per launch: sum over scenes and frequencies of N*M + N*P*M."""
        M = self.n_snk
        tot = 0
        for d in self.data:
            N, Pn = d.src.shape[0], d.scat.shape[0]
            tot += N * M + N * Pn * M
        return tot * self.n_freq

    def pairs(self):
        """Ray pairs whose visibility is resolved per launch: N*P + N*M + P*M summed over scenes."""
        M = self.n_snk
        return sum(d.src.shape[0] * d.scat.shape[0] + d.src.shape[0] * M + d.scat.shape[0] * M for d in self.data)

    # ------------------------------------------------------------ autotuner

    def signature(self, cell_scales=None):
        sizes = [(d.src.shape[0], d.scat.shape[0], d.n_tris) for d in self.data]
        mode = list(cell_scales) if cell_scales else [round(c, 6) for c in self.grid_cells()]
        h = hashlib.sha1(json.dumps([sizes, self.n_snk, self.n_freq, self.uniform, self.cull, mode]).encode())
        return f"{torch.cuda.get_device_name(self.device)}|{h.hexdigest()}"

    def autotune(self, candidates=None, reps=1, use_cache=True, log=None, proxy=None, cell_scales=None):
        """Times each candidate configuration (one warm launch, then `reps` timed ones) on
        this batch, or on `proxy` (a smaller BatchedScattering with the same frequencies,
        e.g. a cost-stratified subset of the scenes), keeps the fastest for this batch and
        returns {config: ms}.  With cell_scales, each scale of the density rule for the grid
        cells (set_cell_scale) is tried with every candidate, and the keys are config + (scale,)."""
        key = self.signature(cell_scales)
        path = _cache_path()
        cache = {}
        if use_cache and os.path.exists(path):
            try:
                with open(path) as f:
                    cache = json.load(f)
            except (OSError, ValueError):
                cache = {}
        if use_cache and key in cache:
            best = tuple(cache[key]["config"])
            if cell_scales and len(best) == 4:
                self.config = best[:3]
                self.set_cell_scale(best[3])
            else:
                self.configure(best[:3])
            return {best: cache[key]["ms"]}
        cands = candidates or CANDIDATES
        if not self.uniform:
            cands = sorted({(1, c[1], c[2]) for c in cands})
        target = proxy if proxy is not None else self
        results = {}
        for scale in (cell_scales or [None]):
            if scale is not None:
                target.set_cell_scale(scale)
            for c in cands:
                try:
                    target.configure(c)
                except (ValueError, LyemError):
                    continue
                target.launch()
                torch.cuda.synchronize()
                t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                t0.record()
                for _ in range(reps):
                    target.launch()
                t1.record()
                torch.cuda.synchronize()
                k = tuple(c) + ((scale,) if scale is not None else ())
                results[k] = t0.elapsed_time(t1) / reps
                if log:
                    log(f"autotune {k}: {results[k]:.2f} ms")
        st, flags = P.device_errors()
        if st != 0 or flags != 0:
            raise LyemError(st or 2, f"batch autotune: device error word {flags:#x}")
        best = min(results, key=results.get)
        self.config = best[:3]
        if len(best) == 4:
            self.set_cell_scale(best[3])
        else:
            self.configure(best[:3])
        if use_cache:
            cache[key] = {"config": list(best), "ms": results[best]}
            try:
                os.makedirs(os.path.dirname(path), exist_ok=True)
                with open(path, "w") as f:
                    json.dump(cache, f, indent=1)
            except OSError:
                pass
        return results
