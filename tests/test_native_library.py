"""CPU checks of the native boundary: the library builds, loads without a GPU and exports every
entry point declared in include/pb_gpu.h.  No compute call is made here."""
import ctypes
import os
import re

import pytest

from plabundle_gb300 import build, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "pb_gpu.h")).read()
    return sorted(set(re.findall(r"^(?:pb_status|const char\*)\s+(pb_\w+)\(", text, re.M)))


@pytest.fixture(scope="module")
def lib_path():
    return build.build()


def test_header_declares_the_abi():
    names = declared_functions()
    assert "pb_gpu_solve" in names and "pb_gpu_upload" in names and len(names) >= 20


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared_functions()) <= set(native.EXPORTED) | {"pb_gpu_last_error", "pb_status_name"}


def test_python_binding_loads(lib_path):
    L = native.load()
    assert L.pb_status_name(0).decode() == "ok"
    assert L.pb_status_name(8).decode() == "unsupported"


def test_struct_layouts_match_header():
    # pb_solve_options: 4 ints + ... ; the ctypes mirror must keep the field order of the header
    text = open(os.path.join(ROOT, "include", "pb_gpu.h")).read()
    block = text.split("typedef struct pb_solve_options {")[1].split("} pb_solve_options;")[0]
    fields = re.findall(r"^\s+\w+\s+(\w+)(?:\[\d+\])?;", block, re.M)
    assert fields == [f for f, _ in native.SolveOptionsC._fields_]
    block = text.split("typedef struct pb_solve_report {")[1].split("} pb_solve_report;")[0]
    fields = re.findall(r"^\s+\w+\s+(\w+);", block, re.M)
    assert fields == [f for f, _ in native.SolveReportC._fields_]
    block = text.split("typedef struct pb_problem_desc {")[1].split("} pb_problem_desc;")[0]
    fields = re.findall(r"^\s+(?:const\s+)?\w+\*?\s+(\w+);", block, re.M)
    assert fields == [f for f, _ in native.ProblemDesc._fields_]
