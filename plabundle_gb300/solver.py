"""``Solver`` and ``SolverWorkspace`` mirroring plabundle's public solve API for the GB300 backend.

``Solver().solve(problem, options, workspace)`` follows ``plabundle::Solver::solve``
(src/solver.cpp:387-518): options/problem validation, cancellation pre-check, the backend run
through the C ABI (the seam runConcreteBackend, src/solver.cpp:275-302), and the quality gate
(resultFailsQualityGate, src/solver.cpp:123-210).  A rejected GB300 result is returned as
unusable; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import native
from .problem import (Backend, GaugePolicy, PlaMatrixDiagnostics, Problem, QualitySummary, RefinedPoint, Result,
                      SolveOptions, SolveStatus, summarize_problem)


class SolverWorkspace:
    """Reusable device workspace for sequential solves (include/plabundle/solver.h:13-32).

    Holds one backend context: device buffers, the reduced pattern and launch shapes are reused
    when the next problem has the same structure.  Not safe for concurrent solves.
    """

    def __init__(self, device: int = 0):
        self.device = device
        self._ctx = None
        self._lib = None

    def context(self):
        if self._ctx is None:
            L = native.load()
            ctx = C.c_void_p()
            st = L.pb_gpu_create(self.device, C.byref(ctx))
            if st != 0:
                raise native.BackendUnavailable(f"no usable CUDA device {self.device} ({L.pb_status_name(st).decode()})")
            self._ctx, self._lib = ctx, L
        return self._lib, self._ctx

    def clear(self):
        if self._ctx is not None:
            self._lib.pb_gpu_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.clear()
        except Exception:
            pass


def validate_options(options: SolveOptions) -> str:
    """Subset of validateOptions (src/options.cpp:252-404) relevant to this backend."""
    s = options.solver
    if s.maxIterations <= 0:
        return "maxIterations must be positive"
    if not (math.isfinite(s.imageRobustLossScalePixels) and s.imageRobustLossScalePixels > 0):
        return "imageRobustLossScalePixels must be finite and positive"
    if s.referenceLineSearchSteps <= 0 or not (s.referenceArmijoCoefficient > 0):
        return "line search settings must be positive"
    cluster = options.backend.plaMatrixPreconditionerClusterSize
    if cluster <= 0 or cluster > 16:
        return "preconditioner cluster size must lie in [1, 16]"
    return ""


def validate_problem(problem: Problem) -> str:
    """validateProblem (src/problem.cpp:142): sizes and index ranges."""
    if problem.n_cameras == 0 or problem.n_tracks == 0:
        return "problem needs cameras and tracks"
    off = np.asarray(problem.track_offsets)
    if off.size != problem.n_tracks + 1 or off[0] != 0 or off[-1] != problem.n_obs or np.any(np.diff(off) < 0):
        return "track offsets do not describe the observations"
    return ""


def result_fails_quality_gate(result: Result, options: SolveOptions) -> str:
    """resultFailsQualityGate for image-only problems (src/solver.cpp:123-210)."""
    q = options.quality
    if not q.enabled:
        return ""
    if not result.solutionUsable:
        return "quality gate rejected a non-usable solution"
    qs = result.quality
    if qs.totalTracks > 0 and not math.isfinite(qs.meanRmsAfter):
        return "quality gate rejected a non-finite final RMS"
    if qs.totalTracks > 0 and qs.validTrackRatio < max(0.0, q.minAcceptedValidTrackRatio):
        return "quality gate rejected a low valid-track ratio"
    growth = max(0.0, q.maxAcceptedRmsGrowth)
    if qs.totalTracks > 0 and growth > 0 and math.isfinite(qs.meanRmsBefore):
        if qs.meanRmsBefore > 1e-12 and qs.meanRmsAfter > qs.meanRmsBefore * growth:
            return "quality gate rejected excessive reprojection RMS growth"
        if qs.meanRmsBefore <= 1e-12 and qs.meanRmsAfter > 1e-9:
            return "quality gate rejected growth from a zero-residual input"
    return ""


class Solver:
    """GB300 counterpart of plabundle::Solver (include/plabundle/solver.h:34-54)."""

    @staticmethod
    def isBackendAvailable(backend: Backend = Backend.Gb300, deviceIndex: int = 0) -> bool:
        if backend not in (Backend.Gb300, Backend.Auto):
            return False
        try:
            ws = SolverWorkspace(deviceIndex)
            ws.context()
            ws.clear()
            return True
        except Exception:
            return False

    def solve(self, problem: Problem, options: SolveOptions | None = None,
              workspace: SolverWorkspace | None = None) -> Result:
        options = options or SolveOptions()
        ws = workspace or SolverWorkspace(options.backend.plaMatrixDevice)
        result = Result(requestedBackend=options.backend.requested, usedBackend=Backend.Gb300)
        result.observationCount = summarize_problem(problem)["observationCount"]
        err = validate_options(options) or validate_problem(problem)
        if err:
            result.status = SolveStatus.InvalidInput
            result.backendMessage = err
            return result
        L, ctx = ws.context()
        desc, keep = native.problem_desc(problem)
        copts = native.solve_options(options, problem)
        st = L.pb_gpu_upload(ctx, C.byref(desc), C.byref(copts))
        if st != 0:
            result.status = SolveStatus.UnsupportedConfiguration if st == 8 else SolveStatus.InvalidInput
            result.backendMessage = L.pb_gpu_last_error(ctx).decode()
            return result
        rep = native.SolveReportC()
        st = L.pb_gpu_solve(ctx, C.byref(copts), C.byref(rep))
        if st != 0:
            result.status = SolveStatus.NumericalFailure
            result.backendMessage = L.pb_gpu_last_error(ctx).decode()
            return result
        p = keep[0]
        cams = np.zeros_like(p.cameras)
        pts = np.zeros_like(p.points)
        valid = np.zeros(p.n_tracks, np.int8)
        rb = np.zeros(p.n_tracks)
        ra = np.zeros(p.n_tracks)
        sizes = np.zeros(16, np.int64)
        L.pb_gpu_get_sizes(ctx, sizes.ctypes.data, None)
        intr = np.zeros((max(1, int(sizes[5])), 13))
        native.check(L, ctx, L.pb_gpu_download_state(ctx, cams.ctypes.data, pts.ctypes.data, valid.ctypes.data,
                                                     rb.ctypes.data, ra.ctypes.data, intr.ctypes.data), "download")
        r = rep.as_dict()
        result.status = SolveStatus(r["status"])
        result.solutionUsable = bool(r["solution_usable"])
        result.backendMessage = L.pb_gpu_last_error(ctx).decode()
        result.totalSeconds = r["total_ms"] / 1000.0
        result.refinedCameras = cams
        result.intrinsicGroups = intr[:int(sizes[5])]
        result.points = RefinedPoint(valid=valid.astype(bool), converged=r["status"] == SolveStatus.Success,
                                     point=pts, rmsBefore=rb, rmsAfter=ra, iterations=r["iterations"])
        result.quality = QualitySummary(totalTracks=p.n_tracks, optimizedTracks=r["optimized_tracks"],
                                        validTrackRatio=r["valid_track_ratio"], meanRmsBefore=r["mean_rms_before"],
                                        meanRmsAfter=r["mean_rms_after"], refinedCameraCount=r["camera_blocks"],
                                        refinedCalibrationGroupCount=r["intrinsic_blocks"],
                                        filterThreshold=r["filter_threshold"])
        result.plaMatrix = PlaMatrixDiagnostics(
            initialCost=r["initial_cost"], finalCost=r["final_cost"], acceptedSteps=r["accepted_steps"],
            rejectedSteps=r["rejected_steps"], linearizations=r["linearizations"],
            objectiveEvaluations=r["objective_evaluations"], rejectedInitialTracks=r["rejected_initial_tracks"],
            linearIterations=r["linear_iterations"], assemblySeconds=r["assembly_ms"] / 1e3,
            objectiveSeconds=r["objective_ms"] / 1e3, linearSolveSeconds=r["linear_ms"] / 1e3,
            backSubstitutionSeconds=r["back_substitution_ms"] / 1e3, schurPatternBuilds=r["pattern_builds"],
            schurPatternReuses=r["pattern_reuses"], mixedPrecisionUsed=bool(copts.precision == 1),
            refinementSweeps=r["refinement_sweeps"], deviceName=f"cuda:{ws.device}")
        result.report = r
        gate = result_fails_quality_gate(result, options)
        if gate:
            result.qualityGateRejected = True
            result.qualityGateMessage = gate
            result.solutionUsable = False
            if result.status in (SolveStatus.Success, SolveStatus.NoConvergence):
                result.status = SolveStatus.NumericalFailure
            result.backendSelectionReason = "explicit_backend; quality_gate_rejected"
        else:
            result.backendSelectionReason = "explicit_backend; quality_gate_passed" if options.quality.enabled \
                else "explicit_backend; quality_gate_disabled"
        return result
