import ctypes as C
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


@pytest.fixture(scope="session")
def host_probe(tmp_path_factory):
    """tests/host_probe.cpp compiled with the host planner (pb_host.cpp): CPU-only entry points
    into the product's host logic."""
    from plabundle_gb300 import native
    here = os.path.dirname(os.path.abspath(__file__))
    out = str(tmp_path_factory.mktemp("probe") / "libhostprobe.so")
    cmd = ["g++", "-std=c++20", "-O1", "-fPIC", "-shared", "-pthread", "-I", os.path.join(ROOT, "include"),
           os.path.join(here, "host_probe.cpp"), os.path.join(ROOT, "plabundle_gb300", "csrc", "pb_host.cpp"),
           "-o", out]
    subprocess.run(cmd, check=True, capture_output=True)
    L = C.CDLL(out)
    L.probe_chunks.argtypes = [C.POINTER(native.ProblemDesc), C.POINTER(native.SolveOptionsC), C.c_int,
                               C.c_size_t, C.POINTER(C.c_longlong)]
    L.probe_chunks.restype = C.c_int
    L.probe_model.argtypes = [C.POINTER(native.ProblemDesc), C.POINTER(native.SolveOptionsC), C.c_void_p,
                              C.c_void_p, C.c_void_p]
    L.probe_model.restype = C.c_int
    L.probe_cp_whitening.argtypes = [C.c_void_p, C.c_void_p]
    L.probe_cp_whitening.restype = C.c_int
    L.probe_rig.argtypes = [C.POINTER(native.ProblemDesc), C.POINTER(native.SolveOptionsC)] + [C.c_void_p] * 4 + \
        [C.c_int] + [C.c_void_p] * 3
    L.probe_rig.restype = C.c_int
    L.probe_rig_terms.argtypes = [C.POINTER(native.ProblemDesc), C.POINTER(native.SolveOptionsC)]
    L.probe_rig_terms.restype = C.c_int
    L.probe_message.restype = C.c_char_p
    return L
