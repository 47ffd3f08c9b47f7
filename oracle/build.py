"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/ht3d_oracle.cpp`` into ``oracle/_build/libht3d_oracle.so``
with ``-ffp-contract=off`` so every FP64 rounding follows the source, and
OpenMP over the outermost loop like ParallelStencil's Threads backend.

The reference (tduretz/HydroThermal3D) is Julia only; there is no C/C++ source
of it to compile, so no ``oracle/_ref`` is produced.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ht3d_oracle.cpp")
# the library's exponentials (shared so both sides evaluate the laws to the same bits)
EXPO = os.path.join(os.path.dirname(HERE), "hydrothermal3d_gb300", "csrc", "expo.h")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libht3d_oracle.so")

CXXFLAGS = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall"]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(EXPO)):
        return LIB
    cmd = ["g++", *CXXFLAGS, "-o", LIB + ".tmp", SRC]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
