"""In-tree build of liblyem_gpu.so (the CUDA kernels and the C ABI of include/lyem.h).

Each .cu file of csrc/ is compiled by nvcc for sm_103a only, in parallel, and
linked into lyceanem_gb300/_lib/liblyem_gpu.so.  Objects are rebuilt when a
source or header is newer than the library.
"""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
PROJECT_DIR = os.path.dirname(PKG_DIR)
REPO_DIR = os.path.dirname(PROJECT_DIR)
CSRC = os.path.join(PROJECT_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
OBJ_DIR = os.path.join(PROJECT_DIR, "_build")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "liblyem_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]
_CUDA_LIB = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(shutil.which("nvcc") or
                                                                         "/usr/local/cuda/bin/nvcc"))), "lib64")
LINK_LIBS = ["-lcublas", "-Xlinker", "-rpath", "-Xlinker", _CUDA_LIB]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblyem_gpu.so")
    return cand


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_native(force=False, verbose=False, jobs=None):
    """Compile csrc/*.cu for sm_103a and link liblyem_gpu.so; returns its path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    srcs = sources()
    objs = []
    todo = []
    for src in srcs:
        obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            todo.append((src, obj))

    def compile_one(item):
        src, obj = item
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj + ".tmp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        os.replace(obj + ".tmp", obj)

    if todo:
        with ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(compile_one, todo))
    if force or todo or _stale(LIB_PATH, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB_PATH + ".tmp", *objs, *LINK_LIBS]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of liblyem_gpu.so failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build_native(force="--force" in sys.argv, verbose=True))
