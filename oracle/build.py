"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/lyem_oracle.c into oracle/_build/liblyem_oracle.so with gcc.
-ffp-contract=off is required: the visibility restatement is bit-faithful FP32
and every fused multiply-add in it is an explicit fmaf() call.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liblyem_oracle.so")
SRC = os.path.join(HERE, "lyem_oracle.c")

CFLAGS = ["-O3", "-fPIC", "-shared", "-std=c11", "-fopenmp", "-ffp-contract=off",
          "-fno-fast-math", "-Wall", "-Wno-unknown-pragmas"]


def build_oracle(force=False, verbose=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    cmd = ["gcc", *CFLAGS, "-o", LIB + ".tmp", SRC, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv, verbose=True))
