"""ctypes binding of the C ABI in include/pb_gpu.h (libpbgpu.so, built in-tree for sm_103a).

There is no CPU fallback: if the library is missing or no CUDA device is usable, the calls
raise ``BackendUnavailable``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libpbgpu.so")

EXPORTED = [
    "pb_gpu_create", "pb_gpu_destroy", "pb_gpu_last_error", "pb_status_name", "pb_gpu_upload",
    "pb_gpu_reset_state", "pb_gpu_get_sizes", "pb_gpu_get_active", "pb_gpu_get_pairs",
    "pb_gpu_linearize_observations", "pb_gpu_linearize_schur", "pb_gpu_get_reduced", "pb_gpu_solve_reduced",
    "pb_gpu_back_substitute", "pb_gpu_eval_cost", "pb_gpu_eval_cost_batch", "pb_gpu_apply_step", "pb_gpu_solve",
    "pb_gpu_download_state", "pb_gpu_solve_problem", "pb_gpu_request_cancel", "pb_gpu_get_stream",
    "pb_gpu_set_timing",
    "pb_gpu_kernel_times", "pb_gpu_objective_noalloc", "pb_gpu_solve_batch",
    "pb_gpu_save_state", "pb_gpu_restore_state", "pb_gpu_set_observations", "pb_gpu_backward",
    "pb_gpu_newton_step", "pb_gpu_get_rig", "pb_gpu_get_history",
    "pb_bne_create", "pb_bne_destroy", "pb_bne_clear_values", "pb_bne_sizes", "pb_bne_add_residual_blocks",
    "pb_bne_add_primary_residual_blocks", "pb_bne_add_primary_residual_block",
    "pb_bne_add_eliminated_residual_block", "pb_bne_add_residual_block", "pb_bne_add_primary_gradient_block",
    "pb_bne_add_primary_hessian_block", "pb_bne_finalize_primary_diagonal", "pb_bne_merge_from",
    "pb_bne_merge_eliminated_shard_from", "pb_bne_export", "pb_gpu_solve_damped_schur",
]


class BackendUnavailable(RuntimeError):
    pass


class ProblemDesc(C.Structure):
    _fields_ = [("n_cameras", C.c_int32), ("cameras", C.c_void_p), ("n_tracks", C.c_int32),
                ("track_offsets", C.c_void_p), ("points", C.c_void_p), ("n_obs", C.c_int64),
                ("obs_camera", C.c_void_p), ("obs_u", C.c_void_p), ("obs_v", C.c_void_p),
                ("obs_weight", C.c_void_p), ("obs_scale", C.c_void_p), ("n_fixed_cameras", C.c_int32),
                ("fixed_cameras", C.c_void_p), ("n_fixed_tracks", C.c_int32), ("fixed_tracks", C.c_void_p),
                ("calibration_group_ids", C.c_void_p), ("intrinsic_reference_cameras", C.c_void_p),
                ("n_control_points", C.c_int32), ("control_point_track", C.c_void_p),
                ("control_point_data", C.c_void_p), ("n_scale_bars", C.c_int32), ("scale_bar_tracks", C.c_void_p),
                ("scale_bar_data", C.c_void_p), ("n_rig_captures", C.c_int32), ("rig_captures", C.c_void_p),
                ("rig_capture_info", C.c_void_p), ("n_rig_sensors", C.c_int32), ("rig_sensors", C.c_void_p),
                ("rig_sensor_info", C.c_void_p), ("rig_camera_capture", C.c_void_p),
                ("rig_camera_sensor", C.c_void_p)]


class SolveOptionsC(C.Structure):
    _fields_ = [("max_iterations", C.c_int32), ("robust_loss", C.c_int32), ("robust_loss_scale", C.c_double),
                ("armijo_coefficient", C.c_double), ("line_search_steps", C.c_int32),
                ("enable_point_filter", C.c_int32), ("filter_max_reproj_error", C.c_double),
                ("filter_sigma_factor", C.c_double), ("max_initial_track_rms", C.c_double),
                ("refine_camera_pose", C.c_int32), ("gauge_policy", C.c_int32),
                ("gauge_anchor_camera", C.c_int32), ("gauge_scale_camera", C.c_int32),
                ("gauge_baseline", C.c_double), ("intrinsic_mask", C.c_uint32), ("precision", C.c_int32),
                ("max_linear_iterations", C.c_int32), ("linear_relative_tolerance", C.c_double),
                ("linear_absolute_tolerance", C.c_double), ("refinement_sweeps", C.c_int32),
                ("preconditioner_cluster_size", C.c_int32), ("linear_solver", C.c_int32),
                ("calibration", C.c_double * 32), ("control_point_weight", C.c_double),
                ("control_point_huber_delta", C.c_double), ("factor_reuse", C.c_int32),
                ("general_path", C.c_int32), ("scale_bar_weight", C.c_double),
                ("scale_bar_huber_delta", C.c_double)]


class SolveReportC(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "status", "solution_usable", "iterations", "accepted_steps", "rejected_steps", "linearizations",
        "objective_evaluations", "linear_iterations", "refinement_sweeps", "active_tracks", "observation_count",
        "rejected_initial_tracks", "optimized_tracks", "camera_blocks", "intrinsic_blocks", "pattern_builds",
        "pattern_reuses", "gpu_kernel_launches")] + [(n, C.c_double) for n in (
            "initial_cost", "final_cost", "mean_rms_before", "mean_rms_after", "valid_track_ratio",
            "filter_threshold", "assembly_ms", "linear_ms", "back_substitution_ms", "objective_ms", "total_ms")] + [
        (n, C.c_int32) for n in ("promoted_point_blocks", "general_path_used", "rig_capture_blocks",
                                 "rig_sensor_blocks")]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None


class AdjointReportC(C.Structure):
    _fields_ = [("status", C.c_int32), ("linear_iterations", C.c_int32), ("gpu_kernel_launches", C.c_int32),
                ("point_blocks_singular", C.c_int32), ("relative_residual", C.c_double),
                ("hessian_ms", C.c_double), ("solve_ms", C.c_double), ("gradient_ms", C.c_double),
                ("total_ms", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class SchurOptionsC(C.Structure):
    _fields_ = [("max_iterations", C.c_int32), ("relative_tolerance", C.c_double),
                ("absolute_tolerance", C.c_double), ("preconditioner_cluster_size", C.c_int32),
                ("use_initial_guess", C.c_int32), ("use_mixed_precision", C.c_int32)]


class SchurReportC(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "converged", "iterations", "schur_pattern_reused", "schur_assembly_on_device", "mixed_precision_used",
        "symbolic_analysis_reused", "eliminated_singular")] + [(n, C.c_double) for n in (
            "relative_residual", "small_block_inverse_ms", "schur_accumulation_ms", "schur_assembly_ms",
            "cholesky_factorization_ms", "triangular_solve_ms", "linear_solve_ms", "back_substitution_ms",
            "total_ms")] + [("preconditioner_name", C.c_char * 64), ("device_name", C.c_char * 64)]

    def as_dict(self):
        d = {name: getattr(self, name) for name, _ in self._fields_}
        for k in ("preconditioner_name", "device_name"):
            d[k] = d[k].decode()
        return d


def library_path() -> str:
    return LIB_PATH


def load(build_if_missing: bool = False):
    """Loads libpbgpu.so (exports checked); raises BackendUnavailable when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build as _build
            _build.build()
        else:
            raise BackendUnavailable(f"GB300 backend library not built: {LIB_PATH}")
    L = C.CDLL(LIB_PATH)
    for name in EXPORTED:
        if not hasattr(L, name):
            raise BackendUnavailable(f"{LIB_PATH} does not export {name}")
    vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    L.pb_gpu_create.argtypes = [i32, C.POINTER(vp)]
    L.pb_gpu_destroy.argtypes = [vp]
    L.pb_gpu_last_error.restype = C.c_char_p
    L.pb_gpu_last_error.argtypes = [vp]
    L.pb_status_name.restype = C.c_char_p
    L.pb_status_name.argtypes = [i32]
    L.pb_gpu_upload.argtypes = [vp, C.POINTER(ProblemDesc), C.POINTER(SolveOptionsC)]
    L.pb_gpu_reset_state.argtypes = [vp]
    L.pb_gpu_get_sizes.argtypes = [vp, vp, C.POINTER(dbl)]
    L.pb_gpu_get_active.argtypes = [vp, vp, vp, vp, vp]
    L.pb_gpu_get_pairs.argtypes = [vp, vp]
    L.pb_gpu_linearize_observations.argtypes = [vp, i32] + [vp] * 7
    L.pb_gpu_linearize_schur.argtypes = [vp, dbl, i32, C.POINTER(dbl), C.POINTER(i32)]
    L.pb_gpu_get_reduced.argtypes = [vp, vp, vp, vp]
    L.pb_gpu_solve_reduced.argtypes = [vp, vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(dbl)]
    L.pb_gpu_back_substitute.argtypes = [vp, vp, C.POINTER(dbl), C.POINTER(i32)]
    L.pb_gpu_eval_cost.argtypes = [vp, C.POINTER(dbl)]
    L.pb_gpu_eval_cost_batch.argtypes = [vp, vp, i32, vp]
    L.pb_gpu_apply_step.argtypes = [vp, dbl]
    L.pb_gpu_solve.argtypes = [vp, C.POINTER(SolveOptionsC), C.POINTER(SolveReportC)]
    L.pb_gpu_download_state.argtypes = [vp] + [vp] * 6
    L.pb_gpu_solve_problem.argtypes = [vp, C.POINTER(ProblemDesc), C.POINTER(SolveOptionsC),
                                       C.POINTER(SolveReportC)] + [vp] * 5
    L.pb_gpu_request_cancel.argtypes = [vp, i32]
    L.pb_gpu_set_timing.argtypes = [vp, i32]
    L.pb_gpu_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.pb_gpu_kernel_times.argtypes = [vp, vp]
    L.pb_gpu_solve_batch.argtypes = [i32, i32, vp, C.POINTER(SolveOptionsC), i32, vp, vp, vp, vp, vp]
    L.pb_gpu_objective_noalloc.argtypes = [vp, i32, vp, i32, vp, vp, vp, vp, vp, i64, i32, dbl, vp,
                                           C.POINTER(dbl), C.POINTER(i64)]
    L.pb_gpu_save_state.argtypes = [vp]
    L.pb_gpu_restore_state.argtypes = [vp]
    L.pb_gpu_set_observations.argtypes = [vp, i64, vp, vp, vp]
    L.pb_gpu_backward.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.POINTER(AdjointReportC)]
    L.pb_gpu_newton_step.argtypes = [vp, C.POINTER(dbl), C.POINTER(dbl)]
    L.pb_gpu_get_rig.argtypes = [vp, vp, vp, vp, vp]
    L.pb_gpu_get_history.argtypes = [vp, i32, vp, vp, vp, C.POINTER(i32)]
    L.pb_bne_create.argtypes = [i32, i32, i32, i32, C.POINTER(vp)]
    L.pb_bne_destroy.argtypes = [vp]
    L.pb_bne_clear_values.argtypes = [vp]
    L.pb_bne_sizes.argtypes = [vp, vp]
    L.pb_bne_add_residual_blocks.argtypes = [vp, vp, vp, i32, i32, vp, vp, i32, dbl]
    L.pb_bne_add_primary_residual_blocks.argtypes = [vp, vp, vp, i32, vp, i32, dbl]
    L.pb_bne_add_primary_residual_block.argtypes = [vp, i32, vp, vp, i32, dbl]
    L.pb_bne_add_eliminated_residual_block.argtypes = [vp, i32, vp, vp, i32, dbl]
    L.pb_bne_add_residual_block.argtypes = [vp, i32, vp, i32, vp, vp, i32, dbl]
    L.pb_bne_add_primary_gradient_block.argtypes = [vp, i32, vp]
    L.pb_bne_add_primary_hessian_block.argtypes = [vp, i32, i32, vp]
    L.pb_bne_finalize_primary_diagonal.argtypes = [vp, dbl, dbl]
    L.pb_bne_merge_from.argtypes = [vp, vp]
    L.pb_bne_merge_eliminated_shard_from.argtypes = [vp, vp, i32]
    L.pb_bne_export.argtypes = [vp] + [vp] * 6
    L.pb_gpu_solve_damped_schur.argtypes = [vp, vp, dbl, C.POINTER(SchurOptionsC), vp, vp, C.POINTER(SchurReportC)]
    for name in EXPORTED:
        if name not in ("pb_gpu_last_error", "pb_status_name"):
            getattr(L, name).restype = i32
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data


def problem_desc(problem):
    """Builds the C descriptor; returns (desc, keepalive) where keepalive owns the arrays."""
    p = problem.normalized()
    fixed_c = np.ascontiguousarray(p.fixedCameraIndices, np.int32)
    fixed_t = np.ascontiguousarray(p.fixedTrackIndices, np.int32)
    cp_track, cp_data = control_point_arrays(p)
    sb_tracks, sb_data = scale_bar_arrays(p)
    keep = [p, fixed_c, fixed_t, cp_track, cp_data, sb_tracks, sb_data]
    desc = ProblemDesc(p.n_cameras, _ptr(p.cameras), p.n_tracks, _ptr(p.track_offsets), _ptr(p.points), p.n_obs,
                       _ptr(p.obs_camera), _ptr(p.obs_u), _ptr(p.obs_v), _ptr(p.obs_weight), _ptr(p.obs_scale),
                       fixed_c.size, _ptr(fixed_c), fixed_t.size, _ptr(fixed_t), _ptr(p.cameraCalibrationGroupIds),
                       _ptr(p.sharedIntrinsicReferenceCameras), cp_track.size, _ptr(cp_track), _ptr(cp_data),
                       sb_data.shape[0], _ptr(sb_tracks), _ptr(sb_data))
    rig = getattr(p, "rig", None)
    if rig is not None and not rig.empty() and rig.captures:
        arrs = rig.arrays(p.n_cameras)
        keep.extend(arrs)
        cap, cap_info, sen, sen_info, cam_cap, cam_sen = arrs
        desc.n_rig_captures = cap.shape[0]
        desc.rig_captures = _ptr(cap)
        desc.rig_capture_info = _ptr(cap_info)
        desc.n_rig_sensors = sen.shape[0]
        desc.rig_sensors = _ptr(sen)
        desc.rig_sensor_info = _ptr(sen_info)
        desc.rig_camera_capture = _ptr(cam_cap)
        desc.rig_camera_sensor = _ptr(cam_sen)
    return desc, keep


def rig_state(L, ctx, problem):
    """(captures [n, 12], sensors [n, 12], capture blocks, sensor blocks) of the context's current
    state, or None when the problem has no rig."""
    rig = getattr(problem, "rig", None)
    if rig is None or not rig.captures:
        return None
    cap = np.zeros((len(rig.captures), 12))
    sen = np.zeros((len(rig.sensors), 12))
    kb = np.zeros(len(rig.captures), np.int32)
    sb = np.zeros(len(rig.sensors), np.int32)
    check(L, ctx, L.pb_gpu_get_rig(ctx, cap.ctypes.data, sen.ctypes.data, kb.ctypes.data, sb.ctypes.data), "get_rig")
    return cap, sen, kb, sb


def refined_rig(L, ctx, problem):
    """Result::refinedRig: the problem's rig topology with the accepted capture and sensor
    parameters, or None without a rig."""
    import dataclasses
    st = rig_state(L, ctx, problem)
    if st is None:
        return None
    cap, sen, _, _ = st
    rig = problem.rig
    caps = [dataclasses.replace(c, rigToWorldRotation=tuple(cap[i, :9]), rigCenterInWorld=tuple(cap[i, 9:12]))
            for i, c in enumerate(rig.captures)]
    sens = [dataclasses.replace(s, cameraToRigRotation=tuple(sen[i, :9]), cameraCenterInRig=tuple(sen[i, 9:12]))
            for i, s in enumerate(rig.sensors)]
    return dataclasses.replace(rig, captures=caps, sensors=sens, cameraBindings=list(rig.cameraBindings))


def scale_bar_arrays(problem):
    """(track pairs int32 [n, 2], records float64 [n, 3]: distance, sigma, weight) of the problem's
    scale bars."""
    bars = getattr(problem, "scaleBarConstraints", None) or []
    tracks = np.ascontiguousarray(np.array([(b.trackIndexA, b.trackIndexB) for b in bars], np.int32).reshape(-1, 2))
    data = np.ascontiguousarray(np.array([(b.measuredDistanceMeters, b.sigmaMeters, b.weight) for b in bars],
                                         np.float64).reshape(-1, 3))
    return tracks, data


def control_point_arrays(problem):
    """(track indices int32 [n], records float64 [n, 15]) of the problem's control points."""
    cps = getattr(problem, "controlPoints", None) or []
    track = np.ascontiguousarray([t for t, _ in cps], np.int32)
    data = np.ascontiguousarray(np.array([c.record() for _, c in cps], np.float64).reshape(-1, 15))
    return track, data


def solve_options(options, problem=None) -> SolveOptionsC:
    from .problem import Precision, intrinsic_mask
    s, cal, b = options.solver, options.calibration, options.backend
    o = SolveOptionsC()
    o.max_iterations = s.maxIterations
    o.robust_loss = int(s.imageRobustLoss)
    o.robust_loss_scale = s.imageRobustLossScalePixels
    o.armijo_coefficient = s.referenceArmijoCoefficient
    o.line_search_steps = s.referenceLineSearchSteps
    o.enable_point_filter = int(s.enablePointFilter)
    o.filter_max_reproj_error = s.filterMaxReprojError
    o.filter_sigma_factor = s.filterSigmaFactor
    o.max_initial_track_rms = s.maxInitialTrackRms
    o.refine_camera_pose = int(cal.refineCameraPose)
    g = problem.gauge if problem is not None else None
    o.gauge_policy = int(g.policy) if g else 0
    o.gauge_anchor_camera = g.referenceAnchorCameraIndex if g else -1
    o.gauge_scale_camera = g.referenceScaleCameraIndex if g else -1
    o.gauge_baseline = g.referenceBaseline if g else 0.0
    o.intrinsic_mask = intrinsic_mask(cal)
    o.precision = int(Precision.Mixed if b.enablePlaMatrixMixedPrecision else Precision.Fp64)
    o.max_linear_iterations = b.maxLinearIterations
    # 0: the reference's tolerance of the path (2e-10 online, 1e-12 general)
    o.linear_relative_tolerance = float(getattr(b, "linearRelativeTolerance", 0.0))
    o.linear_absolute_tolerance = 1.0e-12
    o.refinement_sweeps = b.refinementSweeps
    o.preconditioner_cluster_size = b.plaMatrixPreconditionerClusterSize
    o.linear_solver = int(b.linearSolver)
    for i, v in enumerate(cal.numeric_block()):
        o.calibration[i] = v
    con = getattr(options, "constraints", None)
    o.control_point_weight = con.controlPointWeight if con is not None else 1.0
    o.control_point_huber_delta = con.controlPointHuberDeltaMeters if con is not None else 0.2
    o.factor_reuse = int(getattr(b, "factorReuse", 0))
    o.general_path = 0 if s.useReferenceOnlineSchur else 1
    o.scale_bar_weight = con.scaleBarWeight if con is not None else 1.0
    o.scale_bar_huber_delta = con.scaleBarHuberDeltaMeters if con is not None else 0.2
    return o


def check(L, ctx, status: int, what: str):
    if status != 0:
        msg = L.pb_gpu_last_error(ctx).decode() if ctx else ""
        raise RuntimeError(f"{what} failed: {L.pb_status_name(status).decode()} {msg}")
