"""Build recipe for the oracle shared library (test infrastructure only).

Compiles oracle/ocean_oracle.c with the host C compiler into
oracle/_build/libocean_oracle.so (OpenMP enabled, no fast-math, no FMA
contraction: the FP32 parts round the same on x86_64 and aarch64).  Portable C.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ocean_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libocean_oracle.so")


def build(force: bool = False, quiet: bool = True) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-fno-fast-math", "-ffp-contract=off",
           "-o", LIB + ".tmp", SRC, "-lm"]
    if not quiet:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, quiet=False)
