"""Build the CPU oracle (test infrastructure only) into oracle/_build/liboracle.so.

    python oracle/build.py

g++ with OpenMP at the reference's release optimisation level (-O3 -funroll-loops; no
-march=native, so the library builds the same way on x86_64 and aarch64 hosts); no FMA
contraction, so both hosts evaluate every term with the same roundings.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")
SRC = os.path.join(HERE, "inca_oracle.cpp")


def build(force=False):
    os.makedirs(OUT, exist_ok=True)
    deps = [SRC,
            os.path.join(HERE, "..", "inca_parallel_gb300", "csrc", "lebedev_table.h"),
            os.path.join(HERE, "..", "inca_parallel_gb300", "csrc", "hermite_table.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-O3", "-funroll-loops", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
