"""CPU check that the culling test's reciprocal-free decisions (guard bands on u
and v, then cull_tail in lyem_device.cuh) equal the reference's rounded
sequence (F = rn(1/A), U, V, t; lyceanem/src/raycasting.cuh:44-66) on inputs
concentrated at every decision boundary.  The device header is compiled for the
host by nvcc (tests/cull_decisions.cu), so the checked code is the kernels' own."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("cull") / "cull_decisions")
    cmd = [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "lyceanem-python_gb300", "csrc"),
           "-o", exe, os.path.join(ROOT, "tests", "cull_decisions.cu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_reciprocal_free_decisions_match_reference(checker, seed):
    r = subprocess.run([checker, "4000000", str(seed)], capture_output=True, text=True)
    lines = r.stdout.strip().splitlines()
    cases, mismatches, fast = lines[-1].split()
    assert int(cases) == 4000000
    assert int(mismatches) == 0, r.stdout
    assert r.returncode == 0
    assert float(fast) > 0.2  # the fast decisions are exercised, not only the fallback
