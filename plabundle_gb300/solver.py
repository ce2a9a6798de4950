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
from typing import Optional

import numpy as np

from . import native
from .problem import (Backend, GaugePolicy, PlaMatrixDiagnostics, Problem, QualitySummary, RefinedPoint, Result,
                      SolveOptions, SolveStatus, backend_name, summarize_problem)


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


def control_point_rms_uncertainty(problem: Problem, options: SolveOptions) -> float:
    """The control-point entry of constraintRmsUncertainty (src/solver.cpp:50-95):
    sqrt(mean over valid constraints of |W^-1|_F^2 / (controlPointWeight * weight))
    (controlPointRmsUncertaintyMeters, src/control_point.cpp:167-200)."""
    var, n = 0.0, 0
    for _, c in problem.controlPoints:
        W = control_point_whitening(c)
        if W is None:
            continue
        d = np.linalg.det(W)
        if not np.isfinite(d) or abs(d) <= 1e-18:
            continue
        u2 = float((np.linalg.inv(W) ** 2).sum())
        var += u2 / (options.constraints.controlPointWeight * c.weight)
        n += 1
    return math.sqrt(var / n) if n else 0.0


def control_point_whitening(c) -> Optional[np.ndarray]:
    """makeControlPointWhitening (src/control_point.cpp:91-165) for the statistics: None when the
    constraint does not validate."""
    from .problem import ControlPointUncertainty
    if not np.all(np.isfinite(c.point)) or not (np.isfinite(c.weight) and c.weight > 0):
        return None
    M = np.asarray(c.uncertaintyMatrix, np.float64).reshape(3, 3)
    if c.uncertainty == ControlPointUncertainty.IsotropicSigma:
        return np.eye(3) / c.sigmaMeters if np.isfinite(c.sigmaMeters) and c.sigmaMeters > 0 else None
    A = M if c.uncertainty == ControlPointUncertainty.Covariance else M.T @ M
    if not np.all(np.isfinite(A)) or not np.allclose(A, A.T, rtol=0, atol=1e-10 * max(1.0, np.abs(A).max())):
        return None
    try:
        L = np.linalg.cholesky(A)
    except np.linalg.LinAlgError:
        return None
    if np.any(np.diag(L) ** 2 <= 1e-12 * max(1.0, np.abs(A).max())):
        return None
    return np.linalg.inv(L) if c.uncertainty == ControlPointUncertainty.Covariance else M


def control_point_stats(problem: Problem, points: Optional[np.ndarray], valid: np.ndarray):
    """computeControlPointStats (src/internal/BundleAdjustQuality.cpp:179-211): count and RMS of
    |X - P| over the constraints of the tracks valid in the result, X the initial point (before)
    or the refined one (after)."""
    X = problem.points if points is None else points
    s, n = 0.0, 0
    for t, c in problem.controlPoints:
        if not valid[t]:
            continue
        d2 = float(((np.asarray(X[t]) - np.asarray(c.point)) ** 2).sum())
        if not np.isfinite(d2):
            continue
        s += d2
        n += 1
    return n, (math.sqrt(s / n) if n else 0.0)


def scale_bar_rms_uncertainty(problem: Problem, options: SolveOptions) -> float:
    """sqrt(mean over the bars of sigma^2 / (scaleBarWeight * weight)) (constraintRmsUncertainty,
    src/solver.cpp:84-88)."""
    bars = problem.scaleBarConstraints
    var = sum(b.sigmaMeters ** 2 / (options.constraints.scaleBarWeight * b.weight) for b in bars)
    return math.sqrt(var / len(bars)) if bars else 0.0


def scale_bar_stats(problem: Problem, points: Optional[np.ndarray], valid: np.ndarray):
    """computeScaleBarStats (src/internal/BundleAdjustQuality.cpp:213-259): count and RMS of
    |X_a - X_b| - measured distance over the usable bars whose two tracks are valid in the result,
    the initial points (before) or the refined ones (after)."""
    X = problem.points if points is None else points
    s, n = 0.0, 0
    for b in problem.scaleBarConstraints:
        a, c = b.trackIndexA, b.trackIndexB
        if a < 0 or c < 0 or a == c or a >= problem.n_tracks or c >= problem.n_tracks:
            continue
        if not (math.isfinite(b.measuredDistanceMeters) and b.measuredDistanceMeters > 0):
            continue
        if not (valid[a] and valid[c]):
            continue
        r = float(np.linalg.norm(np.asarray(X[a]) - np.asarray(X[c]))) - b.measuredDistanceMeters
        if not math.isfinite(r):
            continue
        s += r * r
        n += 1
    return n, (math.sqrt(s / n) if n else 0.0)


def constraint_gate(count: int, before: float, after: float, growth: float, unc: float, what: str) -> str:
    """constraintRmsPassesQualityGate (src/internal/BundleAdjustQuality.cpp:504-540)."""
    if count <= 0:
        return ""
    if not (math.isfinite(before) and math.isfinite(after) and math.isfinite(unc)) or unc < 0:
        return f"quality gate rejected invalid {what} RMS or uncertainty"
    if after > max(1.0, growth) * max(before, unc):
        return f"quality gate rejected {what} RMS growth beyond the uncertainty threshold"
    return ""


def result_fails_quality_gate(result: Result, options: SolveOptions, problem: Optional[Problem] = None) -> str:
    """resultFailsQualityGate (src/solver.cpp:123-210) for image and control-point terms."""
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
    # constraintRmsPassesQualityGate (src/internal/BundleAdjustQuality.cpp:504-540)
    if problem is not None and qs.controlPointConstraintCount > 0:
        unc = control_point_rms_uncertainty(problem, options)
        before, after = qs.controlPointRmsBeforeMeters, qs.controlPointRmsAfterMeters
        if not (math.isfinite(before) and math.isfinite(after) and math.isfinite(unc)) or unc < 0:
            return "quality gate rejected invalid control-point constraint RMS or uncertainty"
        if after > max(1.0, q.maxAcceptedConstraintRmsGrowth) * max(before, unc):
            return "quality gate rejected control-point constraint RMS growth beyond the uncertainty threshold"
    if problem is not None and qs.scaleBarConstraintCount > 0:
        msg = constraint_gate(qs.scaleBarConstraintCount, qs.scaleBarRmsBeforeMeters, qs.scaleBarRmsAfterMeters,
                              q.maxAcceptedConstraintRmsGrowth, scale_bar_rms_uncertainty(problem, options),
                              "scale-bar constraint")
        if msg:
            return msg
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
        requested = options.backend.requested
        if requested not in (Backend.Auto, Backend.Gb300):
            # explicit backend that this build does not provide (src/solver.cpp:450-467); there is
            # no CPU fallback to run instead
            result = Result(requestedBackend=requested, usedBackend=requested, usedGpu=False,
                            status=SolveStatus.BackendUnavailable, solutionUsable=False,
                            backendMessage=f"backend {backend_name(requested)} is not provided by the GB300 build",
                            backendSelectionReason="explicit_backend")
            result.observationCount = summarize_problem(problem)["observationCount"]
            return result
        ws = workspace or SolverWorkspace(options.backend.plaMatrixDevice)
        result = Result(requestedBackend=requested, usedBackend=Backend.Gb300)
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
        result.refinedRig = native.refined_rig(L, ctx, problem)
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
        if problem.controlPoints:
            v = result.points.valid
            result.quality.controlPointConstraintCount, result.quality.controlPointRmsBeforeMeters = \
                control_point_stats(problem, None, v)
            _, result.quality.controlPointRmsAfterMeters = control_point_stats(problem, pts, v)
        if problem.scaleBarConstraints:
            v = result.points.valid
            result.quality.scaleBarConstraintCount, result.quality.scaleBarRmsBeforeMeters = \
                scale_bar_stats(problem, None, v)
            _, result.quality.scaleBarRmsAfterMeters = scale_bar_stats(problem, pts, v)
        result.report = r
        gate = result_fails_quality_gate(result, options, problem)
        if gate:
            result.qualityGateRejected = True
            result.qualityGateMessage = gate
            result.solutionUsable = False
            if result.status in (SolveStatus.Success, SolveStatus.NoConvergence):
                result.status = SolveStatus.NumericalFailure
            how = "explicit_backend" if requested == Backend.Gb300 else "auto_selected_gb300"
            result.backendSelectionReason = how + "; quality_gate_rejected"
        else:
            how = "explicit_backend" if requested == Backend.Gb300 else "auto_selected_gb300"
            result.backendSelectionReason = how + ("; quality_gate_passed" if options.quality.enabled
                                                   else "; quality_gate_disabled")
        return result
