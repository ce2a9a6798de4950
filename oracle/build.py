"""Build recipe for the CPU FP64 oracle (test infrastructure).

Compiles ``ba_oracle.cpp`` with g++ and OpenMP into ``oracle/_build/libbaoracle.so``.
FMA contraction is disabled so that x86_64 and aarch64 builds round identically.
The reference itself is not built: it needs the absent PlaMatrix and PlaCamera
libraries (see the oracle header).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libbaoracle.so")
SOURCES = [os.path.join(HERE, "ba_oracle.cpp")]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SOURCES + [os.path.join(HERE, "ba_oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-o", LIB + ".tmp"] + SOURCES
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
