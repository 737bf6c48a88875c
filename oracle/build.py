"""Build the C oracle (test infrastructure only) into oracle/_build/.

gcc, -O2, -ffp-contract=off (no FMA contraction on any host architecture so
the order of roundings is the one written), OpenMP for the timed CPU
baseline.  No -march=native: the same flags build here and on an aarch64
host.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libd3d_oracle.so")
SRC = os.path.join(HERE, "d3d_oracle.c")


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
           SRC, "-o", LIB + ".tmp", "-lm"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
