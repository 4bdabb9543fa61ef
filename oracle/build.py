"""Build recipe for the oracle library (test infrastructure).

Compiles hg_oracle.cpp (the restated passes), hg_adjoint_ref.cpp (the FP64
reference adjoint) and hg_terrain_ref.cpp (the reference's terrain generator
and rain) and hg_render_ref.cpp (the terrain ray-marcher) with g++ into
oracle/libhg_oracle.so.  The flags keep
IEEE single/double semantics: no fused multiply-add contraction and no
fast-math, so the float instantiation rounds once per GLSL operation.
OpenMP parallelises every pass over rows (the timed CPU baseline).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, "hg_oracle.cpp"), os.path.join(HERE, "hg_adjoint_ref.cpp"),
        os.path.join(HERE, "hg_terrain_ref.cpp"), os.path.join(HERE, "hg_render_ref.cpp")]
LIB = os.path.join(HERE, "libhg_oracle.so")
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
         "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function"]


def build(force=False, verbose=False):
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in SRCS):
        return LIB
    cmd = ["g++", *FLAGS, *SRCS, "-o", LIB + ".tmp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
