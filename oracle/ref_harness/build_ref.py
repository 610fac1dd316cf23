"""Compiles harness.cu against the reference's headers into oracle/_ref/ (test infrastructure only).

Run where the reference tree is mounted: its root is the argument, else the
environment variable LYEM_REFERENCE_ROOT, else /root/reference.  Builds two
cubins for sm_103a with the reference's release flags (-O3 -DNDEBUG): the
default (nvcc free to contract a*b+c into FMA, as the reference's own build)
and --fmad=false, which bracket the reference binary's arithmetic.
"""
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")


DEFAULT_ROOT = "/root/reference"


def reference_root():
    """Root of the mounted reference tree (LYEM_REFERENCE_ROOT overrides the default)."""
    return os.environ.get("LYEM_REFERENCE_ROOT", DEFAULT_ROOT)


def build(ref_root=None, verbose=False):
    """Builds the harness cubins; None when the reference's sources are not mounted."""
    src = os.path.join(ref_root or reference_root(), "lyceanem", "src")
    if not os.path.isdir(src):
        return None
    import pybind11
    os.makedirs(OUT, exist_ok=True)
    outs = []
    for name, extra in (("ref_harness.cubin", []), ("ref_harness_nofma.cubin", ["--fmad=false"])):
        out = os.path.join(OUT, name)
        if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(os.path.join(HERE, "harness.cu")):
            outs.append(out)
            continue
        cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-DNDEBUG", "-std=c++17",
               *extra, "-I", src, "-I", pybind11.get_include(), "-I", sysconfig.get_paths()["include"],
               "-o", out, os.path.join(HERE, "harness.cu")]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        outs.append(out)
    return outs


if __name__ == "__main__":
    print(build(*(sys.argv[1:2] or []), verbose=True))
