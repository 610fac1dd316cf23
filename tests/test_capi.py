"""The C-ABI library builds, loads without a GPU, and exports every entry point of include/lyem.h."""
import ctypes

import numpy as np


def test_library_exports_header_symbols():
    from lyceanem_gb300 import build
    build.build_native()
    from lyceanem_gb300 import _native
    names = _native.header_symbols()
    assert len(names) >= 15
    lib = _native.load()
    for n in names:
        assert hasattr(lib, n), n
    # every declared entry point has a ctypes signature, and nothing extra is bound
    assert sorted(_native.SIGNATURES) == names


def test_status_strings_and_version():
    from lyceanem_gb300._native import lib
    assert lib.lyem_version() >= 100
    assert lib.lyem_status_string(0) == b"ok"
    assert lib.lyem_status_string(4) == b"bounded device wait expired"
    assert lib.lyem_status_string(99) == b"unknown status"


def test_grid_plan_host_logic():
    from lyceanem_gb300._native import lib, f32arr
    org = (ctypes.c_float * 3)()
    cell = ctypes.c_float()
    dims = (ctypes.c_int32 * 3)()
    b = f32arr([-10, -10, -1, 10, 10, 5])
    assert lib.lyem_grid_plan(b, 120000, 0.5, org, ctypes.byref(cell), dims) == 0
    assert cell.value == 0.5
    assert list(dims) == [41, 41, 13]
    for k, lo in enumerate([-10, -10, -1]):
        assert org[k] < lo and org[k] > lo - 0.01
        assert org[k] + dims[k] * cell.value > [10, 10, 5][k]
    # automatic cell: about one cell per triangle
    assert lib.lyem_grid_plan(b, 1000, 0.0, org, ctypes.byref(cell), dims) == 0
    n = dims[0] * dims[1] * dims[2]
    assert 500 <= n <= 2000
    # invalid arguments are reported, not crashed on
    assert lib.lyem_grid_plan(b, -1, 0.5, org, ctypes.byref(cell), dims) == 1
    assert lib.lyem_grid_plan(None, 10, 0.5, org, ctypes.byref(cell), dims) == 1


def test_workspace_queries():
    from lyceanem_gb300._native import lib
    ws = lib.lyem_pair_stage_workspace(1024, 65341, 0, 1, 0)
    assert ws >= 24 * 65341
    assert lib.lyem_pair_stage_workspace(64, 2664, 1024, 0, 1) == 64 * 2664 * 24 + 256
    assert lib.lyem_grid_count_workspace(1000) > 4 * 1000
    assert lib.lyem_grid_fill_workspace(10000, 100) > 16 * 10000


def test_device_entry_points_reject_bad_arguments_without_gpu_work():
    from lyceanem_gb300._native import lib
    # negative sizes and null pointers are rejected before any CUDA call
    assert lib.lyem_pack_triangles(None, 3, None, -1, None, None) == 1
    assert lib.lyem_pack_triangles(None, 3, None, 0, None, None) == 0
    assert lib.lyem_mask_to_bytes(None, -1, 3, None, None) == 1
    assert lib.lyem_em_bin_counts(None, 0, None, 0, 0, 1, 0.0, 1.0, 0.0, None) == 1
    out = np.zeros(1, np.int32)
    assert lib.lyem_em_bin_counts(None, 0, None, 0, 1, 1, 0.0, -1.0, 0.0, out.ctypes.data) == 1
    # the culling test relies on a determinant threshold that is finite and not negative
    d = ctypes.c_void_p(256)
    for eps in (-1e-6, float("nan"), float("inf")):
        assert lib.lyem_pair_stage(d, d, None, 4, d, d, 4, d, 1, None, None, None, None, 0.0, None, 0.0, 1.0, 0, 1,
                                   eps, None, 0, None, None, None, None, None, None, None, 0, 0, None, 0, None) == 1


def test_direction_order_argument_checks():
    """Argument checks of lyem_direction_order run on the host (no device call for these)."""
    from lyceanem_gb300._native import lib, f32arr
    c = f32arr([0, 0, 0])
    assert lib.lyem_direction_order(None, 0, c, None, None, 0, None) == 0  # nothing to order
    assert lib.lyem_direction_order(None, -1, c, None, None, 0, None) == 1  # LYEM_ERR_INVALID
    assert lib.lyem_direction_order(None, 5, c, None, None, 0, None) == 1
    assert lib.lyem_direction_order(ctypes.c_void_p(16), 5, f32arr([0, float("nan"), 0]), ctypes.c_void_p(16),
                                    None, 0, None) == 1
    assert lib.lyem_direction_order(ctypes.c_void_p(16), 5, c, ctypes.c_void_p(16), None, 0, None) == 6  # workspace


def test_header_compiles_as_c_and_links(tmp_path):
    """include/lyem.h is plain C: a C program that includes it links against liblyem_gpu.so and calls the
    host-only entry points (no GPU needed)."""
    import os
    import shutil
    import subprocess
    from lyceanem_gb300 import _native
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "caller.c"
    src.write_text(
        '#include "lyem.h"\n#include <stdio.h>\n'
        "int main(void) {\n"
        "  float org[3], cell; int32_t dims[3];\n"
        "  const float b[6] = {-10.f, -10.f, -1.f, 10.f, 10.f, 5.f};\n"
        "  if (lyem_grid_plan(b, 120000, 0.5f, org, &cell, dims) != LYEM_OK) return 1;\n"
        '  printf("%d %s %d %d %d\\n", lyem_version(), lyem_status_string(LYEM_ERR_WORKSPACE), dims[0], dims[1],\n'
        "         dims[2]);\n"
        "  return 0;\n}\n")
    exe = tmp_path / "caller"
    libdir = os.path.dirname(_native.LIB_PATH)
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(root, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-llyem_gpu", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert int(out[0]) >= 100 and out[-3:] == ["41", "41", "13"]


def test_sweep_modes_host_checks():
    """Beam-sweep sizes and argument checks (host only, no device call): operand sizes of the tensor-core
    modes (3, 4: a 256-byte header and K-major planes with the source count rounded up to 8), no
    workspace for any mode, the removed four-product modes (1, 2) and unknown modes refused, operands
    that are not 256-byte aligned refused."""
    from lyceanem_gb300._native import lib
    assert lib.lyem_sweep_workspace_bytes(1024, 16, 3) == 0
    assert lib.lyem_sweep_network_bytes(10, 16, 3) == 256 + 18 * 16 * 16 * 2
    assert lib.lyem_sweep_network_bytes(16, 16, 4) == 256 + 18 * 16 * 16 * 2
    assert lib.lyem_sweep_network_bytes(10, 16, 0) == 3 * 10 * 16 * 8
    assert lib.lyem_sweep_weights_bytes(10, 4, 4) == 256 + 6 * 4 * 16 * 2
    assert lib.lyem_sweep_weights_bytes(10, 4, 0) == 0
    for mode in (1, 2, 5):
        assert lib.lyem_sweep_network_bytes(10, 16, mode) == 0
    fake = ctypes.c_void_p(256)
    odd = ctypes.c_void_p(256 + 64)
    assert lib.lyem_sweep_run_ws(fake, 10, 16, 16, None, fake, 4, 1, fake, 16, None, 0, None) == 1  # mode 1 gone
    assert lib.lyem_sweep_run(fake, 10, 16, 16, None, fake, 4, 5, fake, 16, None) == 1  # no mode 5
    assert lib.lyem_sweep_run(odd, 10, 16, 16, None, fake, 4, 3, fake, 16, None) == 1  # unaligned network
    assert lib.lyem_sweep_prepare_weights(fake, 10, 4, 3, odd, None) == 1  # unaligned weight operand
    assert lib.lyem_sweep_set_k_tile(48) == 1
    assert lib.lyem_sweep_set_k_tile(64) == 0
