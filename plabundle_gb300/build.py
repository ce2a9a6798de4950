"""Builds the GB300 backend library ``plabundle_gb300/_lib/libpbgpu.so`` for sm_103a.

Each translation unit is compiled by nvcc in parallel (one ``-gencode`` for sm_103a) and the
objects are linked into one shared library that exports the C ABI of ``include/pb_gpu.h``.
FMA contraction is left on for device code (it is part of the kernels' arithmetic); host code
is compiled with ``-ffp-contract=off`` so that x86_64 and aarch64 hosts round identically.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpbgpu.so")
SOURCES = ["pb_host.cpp", "pb_assemble.cu", "pb_kernels.cu", "pb_pcg.cu", "pb_dense.cu", "pb_solver.cu", "pb_noalloc.cu", "pb_batch.cu", "pb_adjoint.cu", "pb_bne.cpp", "pb_schur.cu", "pb_survey.cu", "pb_rig.cu"]
HEADERS = ["pb_internal.h", "pb_device.cuh", "pb_kernels.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _flags(verbose_ptxas: bool) -> list:
    f = ["-O3", "-std=c++20", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-pthread",
         "-I", os.path.join(ROOT, "include")] + ARCH
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(OBJ_DIR, src + ".o")
    cmd = [_nvcc()] + _flags(verbose_ptxas) + ["-c", os.path.join(CSRC, src), "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas:
        sys.stderr.write(res.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in SOURCES + HEADERS] + [os.path.join(ROOT, "include", "pb_gpu.h"),
                                                                  os.path.abspath(__file__)]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart", "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
