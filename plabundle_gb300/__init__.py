"""GB300-native reduced-Schur bundle-adjustment backend for plabundle.

The compute path is ``libpbgpu.so`` (hand-written sm_103a CUDA kernels plus the C++ host
driver) behind the C ABI of ``include/pb_gpu.h``; this package is its Python host mirror of
``plabundle::Solver::solve(Problem, SolveOptions, SolverWorkspace)``.
"""
from .problem import (Backend, CalibrationOptions, Gauge, GaugePolicy, ImageRobustLoss, IntrinsicParameter,
                      Precision, Problem, Result, SolveOptions, SolveStatus, backend_name, intrinsic_mask,
                      shared_intrinsic_parameter_enabled, summarize_problem)
from .solver import Solver, SolverWorkspace

__all__ = ["Backend", "CalibrationOptions", "Gauge", "GaugePolicy", "ImageRobustLoss", "IntrinsicParameter",
           "Precision", "Problem", "Result", "SolveOptions", "SolveStatus", "Solver", "SolverWorkspace",
           "backend_name", "intrinsic_mask", "shared_intrinsic_parameter_enabled", "summarize_problem"]
