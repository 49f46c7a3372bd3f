"""Build recipe for the CPU oracle (test infrastructure, not product).

Compiles ``lbm_oracle.cpp`` into ``oracle/_build/liblbm_oracle.so`` with
``-ffp-contract=off`` (no fused multiply-add, so the float build evaluates the
reference's expressions as separately rounded IEEE operations; GCC contracts
by default on aarch64) and OpenMP.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liblbm_oracle.so")
SRC = os.path.join(HERE, "lbm_oracle.cpp")


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-o", LIB + ".tmp", SRC]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
