"""Host side of the batched launch (no GPU): work-list sizes, workspace layout and
argument checks of lyem_batch_workspace / lyem_batch_items."""
import ctypes

import pytest

from lyceanem_gb300._native import BatchConfig, BatchScene, lib

FAKE = 0x10000  # 256-byte aligned stand-in device address; these calls never dereference it


def _scene(n_src, n_scat, dims=(4, 4, 4)):
    s = BatchScene()
    s.src_pos = s.src_E = FAKE
    s.scat_pos = s.scat_nrm = FAKE if n_scat else None
    s.scat_id = None
    s.cell_start = s.cell_tris = s.cell_box = FAKE
    s.n_src, s.n_scat = n_src, n_scat
    for k in range(3):
        s.grid_origin[k] = -1.0
        s.grid_dims[k] = dims[k]
    s.grid_cell = 0.5
    return s


def _cfg(fg=4, chunk=32, bps=0):
    c = BatchConfig()
    c.freq_group, c.src_chunk, c.blocks_per_sm, c.cull, c.eps, c.self_to_self, c.alpha = fg, chunk, bps, 1, 1e-6, 0, 0.0
    return c


def _ceil(a, b):
    return -(-a // b)


@pytest.mark.parametrize("fg,chunk", [(1, 32), (2, 64), (4, 32), (8, 64)])
def test_item_counts(fg, chunk):
    sizes = [(100, 37), (16, 0), (1000, 513)]
    scenes = (BatchScene * 3)(*[_scene(n, p) for n, p in sizes])
    M, F = 1000, 64
    cfg = _cfg(fg, chunk)
    per = (ctypes.c_int64 * 5)()
    n = lib.lyem_batch_items(scenes, 3, M, F, ctypes.byref(cfg), per)
    groups = _ceil(F, fg)

    def field_items(nk, pairs_per_sink):
        # a field item is a run of k 32-slot chunks (slot = point * groups + group),
        # k = ceil(2^14 / candidate pairs of a chunk), 1..64
        chunks = _ceil(nk * groups, 32)
        k = min(64, max(1, _ceil(1 << 14, max(1, pairs_per_sink * 32 // groups))))
        return _ceil(chunks, k)

    # visibility items: one source chunk x 32 sinks (one warp)
    vis = [sum(_ceil(N, chunk) * _ceil(Pn, 32) for N, Pn in sizes),
           sum(_ceil(N, chunk) * _ceil(M, 32) for N, _ in sizes),
           sum(_ceil(Pn, chunk) * _ceil(M, 32) for _, Pn in sizes)]
    expect = vis + [sum(field_items(Pn, N) for N, Pn in sizes), sum(field_items(M, N + Pn) for N, Pn in sizes)]
    assert list(per) == expect
    assert n == sum(expect)
    ws = lib.lyem_batch_workspace(scenes, 3, M, F, ctypes.byref(cfg))
    assert ws > 0 and ws % 256 == 0
    # masks (one bit per pair, rows padded to 32 sources) and the scatter excitations dominate
    bits = sum(Pn * _ceil(N, 32) + M * _ceil(N, 32) + M * _ceil(Pn, 32) for N, Pn in sizes) * 4
    assert ws >= bits + sum(Pn * F * 24 for _, Pn in sizes)


def test_rejects_bad_arguments():
    scenes = (BatchScene * 1)(_scene(64, 10))
    for cfg in (_cfg(fg=3), _cfg(chunk=48), _cfg(bps=9)):
        assert lib.lyem_batch_workspace(scenes, 1, 100, 16, ctypes.byref(cfg)) == 0
    # any number of frequency groups (slots of 32 (point, group) pairs per warp); at most 4,096 frequencies
    assert lib.lyem_batch_workspace(scenes, 1, 100, 300, ctypes.byref(_cfg(fg=1))) > 0
    assert lib.lyem_batch_workspace(scenes, 1, 100, 5000, ctypes.byref(_cfg(fg=2))) == 0
    bad = (BatchScene * 1)(_scene(64, 10))
    bad[0].cell_start = None
    assert lib.lyem_batch_workspace(bad, 1, 100, 16, ctypes.byref(_cfg())) == 0
    bad = (BatchScene * 1)(_scene(64, 10, dims=(0, 4, 4)))
    assert lib.lyem_batch_workspace(bad, 1, 100, 16, ctypes.byref(_cfg())) == 0
    assert lib.lyem_batch_workspace(scenes, 0, 100, 16, ctypes.byref(_cfg())) == 0
    assert lib.lyem_batch_items(scenes, 1, 0, 16, ctypes.byref(_cfg()), None) < 0


def test_density_cell():
    from lyceanem_gb300.batched import density_cell
    # 10 x 10 x 1 m box, 1000 triangles: 0.1 m^3 per triangle
    c = density_cell([0, 0, 0, 10, 10, 1], 1000, 1.0)
    assert abs(c - 0.1 ** (1 / 3)) < 1e-12
    assert abs(density_cell([0, 0, 0, 10, 10, 1], 1000, 2.0) - 2 * c) < 1e-12
    # flat box: the thin axis counts as 1 mm, and the result is clipped to [0.05, 10] m
    assert density_cell([0, 0, 0, 1, 1, 0], 10 ** 6, 1.0) == 0.05
    assert density_cell([0, 0, 0, 1e3, 1e3, 1e3], 1, 1.0) == 10.0
    assert density_cell([0, 0, 0, 1, 1, 1], 0, 1.0) == 1.0
