"""lyem_pair_stage_noalloc, the pair stage for callers that may not allocate device memory.

Such callers (a host whose own allocator owns all device memory, or code that
forbids allocation calls once running) cannot pass lyem_pair_stage a scratch
buffer; this entry point keeps its scratch in a fixed array inside the library.
The test calls it through the C ABI twice in a row (the second call sees the
first call's leftovers in the shared scratch) and checks each result against
lyem_pair_stage with a caller-provided workspace.  The file is collected last so
that a run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

from helpers import random_scene, rel_err

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-5


@pytest.fixture(scope="module")
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from lyceanem_gb300 import build
    build.build_native()
    from lyceanem_gb300 import _native
    return _native.load()


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _args(src, E, snk, snk_n, tris, grid):
    """Common leading arguments of both entry points (device tensors, brute force or grid)."""
    from lyceanem_gb300._native import f32arr, i32arr
    if grid is None:
        g = (None, None, None, f32arr([0, 0, 0]), 1.0, i32arr([1, 1, 1]))
        t, T = tris, tris.shape[0]
    else:
        g = (_p(grid.cell_start), _p(grid.cell_tris), _p(grid.cell_box), f32arr(grid.origin), grid.cell,
             i32arr(grid.dims))
        t, T = None, 0
    return [_p(src), _p(torch.view_as_real(E)), None, src.shape[0], _p(snk), _p(snk_n), snk.shape[0], _p(t), T, *g]


def _run_both(lib, src, E, snk, snk_n, tris, grid, beta):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    M = snk.shape[0]
    words = (M + 31) // 32
    out_ref = torch.empty((M, 3), dtype=torch.complex64, device="cuda")
    out_na = torch.full((M, 3), float("nan"), dtype=torch.complex64, device="cuda")
    bits_ref = torch.zeros((src.shape[0], words), dtype=torch.int32, device="cuda")
    bits_na = torch.zeros_like(bits_ref)
    common = _args(src, E, snk, snk_n, tris, grid) + [0.0, beta, 0, 1, 1e-6]
    use_grid = int(grid is not None)
    ws_bytes = lib.lyem_pair_stage_workspace(src.shape[0], M, tris.shape[0], use_grid, 0)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    st = lib.lyem_pair_stage(*common, _p(torch.view_as_real(out_ref)), 0, None, _p(bits_ref), None, None, None, None,
                             None, 0, 0, _p(ws), ws_bytes, stream)
    assert st == 0
    st = lib.lyem_pair_stage_noalloc(*common, _p(torch.view_as_real(out_na)), 0, None, _p(bits_na), None, None, None,
                                     None, None, 0, 0, stream)
    assert st == 0
    torch.cuda.synchronize()
    return out_ref.cpu().numpy(), out_na.cpu().numpy(), bits_ref.cpu().numpy(), bits_na.cpu().numpy()


def test_noalloc_matches_workspace_entry_point_twice(lib):
    from lyceanem_gb300 import propagation as P
    assert lib.lyem_pair_stage_noalloc_scratch_bytes() == 32 << 20
    # first call: brute force on a larger scene; second call: grid on a smaller
    # scene, so it runs over the first call's leftovers in the shared scratch
    cases = [(random_scene(41, n_src=70, n_snk=900, n_tris=400), None),
             (random_scene(42, n_src=23, n_snk=333, n_tris=250), 0.3)]
    for (src, snk, snk_n, v, f, E), cell in cases:
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
        src_d, snk_d, nrm_d, E_d = t(src), t(snk), t(snk_n), t(E)
        tris = P.pack_triangles(t(v), t(f))
        grid = P.UniformGrid(tris, cell=cell) if cell else None
        ref, got, bref, bgot = _run_both(lib, src_d, E_d, snk_d, nrm_d, tris, grid, 2 * np.pi / 0.05)
        assert np.isfinite(got).all()
        assert rel_err(got, ref) < FIELD_TOL
        assert np.array_equal(bref, bgot)
    st, flags = P.device_errors()
    assert st == 0 and flags == 0


def test_noalloc_rejects_problems_beyond_the_scratch(lib):
    from lyceanem_gb300._native import LYEM_ERR_WORKSPACE
    # 4096 sources x 200,000 sinks needs at least 128 chunks x 200,000 x 24 B = 614 MB of partial sums
    n_src, n_snk = 4096, 200000
    assert lib.lyem_pair_stage_workspace(n_src, n_snk, 10, 0, 32) > lib.lyem_pair_stage_noalloc_scratch_bytes()
    src = torch.zeros((n_src, 3), device="cuda")
    E = torch.zeros((n_src, 3), dtype=torch.complex64, device="cuda")
    snk = torch.ones((n_snk, 3), device="cuda")
    out = torch.zeros((n_snk, 3), dtype=torch.complex64, device="cuda")
    tris = torch.zeros((10, 12), device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    common = _args(src, E, snk, snk, tris, None) + [0.0, 1.0, 0, 1, 1e-6]
    st = lib.lyem_pair_stage_noalloc(*common, _p(torch.view_as_real(out)), 0, None, None, None, None, None, None,
                                     None, 0, 0, stream)
    assert st == LYEM_ERR_WORKSPACE
    torch.cuda.synchronize()
    assert torch.all(out == 0)
