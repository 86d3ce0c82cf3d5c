"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle.cpp into oracle/_build/liblh_oracle.so with FMA contraction
off, so that every float operation rounds on its own exactly as the CUDA
kernels (built with --fmad=false) do.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liblh_oracle.so")

FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math",
         "-fno-finite-math-only", "-Wall", "-Wno-unused-function"]


def build(force=False):
    src = os.path.join(HERE, "oracle.cpp")
    deps = [src, os.path.join(HERE, "oracle.h"),
            os.path.join(HERE, "..", "include", "lh", "lh.h"),
            os.path.join(HERE, "..", "include", "lh", "shared.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++"] + FLAGS + [src, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
