"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/bem_oracle.c into oracle/_build/libbem_oracle.so with gcc.
-ffp-contract=off keeps the arithmetic free of fused multiply-adds on both
x86_64 and aarch64; -fcx-limited-range makes complex * and / use the textbook
formulas of num-complex.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libbem_oracle.so")
SRC = os.path.join(HERE, "bem_oracle.c")
HDR = os.path.join(HERE, "bem_oracle.h")


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR))):
        return LIB
    cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fcx-limited-range", "-Wall", "-Wno-unused-function",
           SRC, "-o", LIB + ".tmp", "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
