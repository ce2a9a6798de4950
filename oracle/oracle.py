"""ctypes wrapper of the CPU FP64 oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this module; the
product path never imports it.  Parity is unpinned (see ba_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import build as _oracle_build  # noqa: E402

_P = 13


class OrcProblem(C.Structure):
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


class OrcOptions(C.Structure):
    _fields_ = [("max_iterations", C.c_int32), ("robust_loss", C.c_int32), ("robust_loss_scale", C.c_double),
                ("armijo_coefficient", C.c_double), ("line_search_steps", C.c_int32),
                ("enable_point_filter", C.c_int32), ("filter_max_reproj_error", C.c_double),
                ("filter_sigma_factor", C.c_double), ("max_initial_track_rms", C.c_double),
                ("refine_camera_pose", C.c_int32), ("gauge_policy", C.c_int32),
                ("gauge_anchor_camera", C.c_int32), ("gauge_scale_camera", C.c_int32),
                ("gauge_baseline", C.c_double), ("intrinsic_mask", C.c_uint32), ("num_threads", C.c_int32),
                ("linear_solver", C.c_int32), ("max_linear_iterations", C.c_int32),
                ("linear_relative_tolerance", C.c_double), ("linear_absolute_tolerance", C.c_double),
                ("calibration", C.c_double * 32), ("control_point_weight", C.c_double),
                ("control_point_huber_delta", C.c_double), ("general_path", C.c_int32),
                ("residual_gate", C.c_int32), ("scale_bar_weight", C.c_double),
                ("scale_bar_huber_delta", C.c_double)]


class OrcReport(C.Structure):
    _fields_ = [("status", C.c_int32), ("solution_usable", C.c_int32), ("iterations", C.c_int32),
                ("accepted_steps", C.c_int32), ("rejected_steps", C.c_int32), ("linearizations", C.c_int32),
                ("objective_evaluations", C.c_int32), ("linear_iterations", C.c_int32),
                ("initial_cost", C.c_double), ("final_cost", C.c_double), ("active_tracks", C.c_int32),
                ("observation_count", C.c_int32), ("rejected_initial_tracks", C.c_int32),
                ("optimized_tracks", C.c_int32), ("mean_rms_before", C.c_double),
                ("mean_rms_after", C.c_double), ("valid_track_ratio", C.c_double),
                ("filter_threshold", C.c_double), ("solve_seconds", C.c_double),
                ("assembly_seconds", C.c_double), ("linear_seconds", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _oracle_build.build()
        L = C.CDLL(path)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(OrcProblem), C.POINTER(OrcOptions), C.POINTER(C.c_int32)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_info.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
        L.orc_active.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.orc_linearize_observations.argtypes = [C.c_void_p] + [C.c_void_p] * 7
        L.orc_build.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_int32)]
        L.orc_pairs.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_reduced.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.orc_solve_linear.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.orc_back_substitute.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                                          C.POINTER(C.c_int32)]
        L.orc_cost.restype = C.c_double
        L.orc_cost.argtypes = [C.c_void_p]
        L.orc_solve.argtypes = [C.c_void_p, C.POINTER(OrcReport)] + [C.c_void_p] * 6
        L.orc_general_build.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_void_p]
        L.orc_general_export.argtypes = [C.c_void_p] + [C.c_void_p] * 6
        L.orc_general_solve.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_void_p,
                                        C.POINTER(C.c_int32)]
        L.orc_rig.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.orc_control_point_whitening.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_control_point_whitening.restype = C.c_int32
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def make_options(options, num_threads: int = 0, linear_solver: int = 0, residual_gate: bool = True) -> OrcOptions:
    from plabundle_gb300.problem import intrinsic_mask
    s, cal = options.solver, options.calibration
    o = OrcOptions()
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
    o.intrinsic_mask = intrinsic_mask(cal)
    o.num_threads = num_threads or s.numThreads
    o.linear_solver = linear_solver
    o.max_linear_iterations = options.backend.maxLinearIterations
    # the reference's tolerances: 2e-10 online, 1e-12 on the general path (BundleAdjustPlaMatrix.cpp:321-330)
    o.general_path = 0 if s.useReferenceOnlineSchur else 1
    o.residual_gate = 1 if residual_gate else 0
    o.linear_relative_tolerance = 2.0e-10 if s.useReferenceOnlineSchur else 1.0e-12
    o.linear_absolute_tolerance = 1.0e-12
    for i, v in enumerate(cal.numeric_block()):
        o.calibration[i] = v
    o.control_point_weight = options.constraints.controlPointWeight
    o.control_point_huber_delta = options.constraints.controlPointHuberDeltaMeters
    o.scale_bar_weight = getattr(options.constraints, "scaleBarWeight", 1.0)
    o.scale_bar_huber_delta = getattr(options.constraints, "scaleBarHuberDeltaMeters", 0.2)
    return o


def control_point_whitening(record):
    """(valid, W 3x3) of one ControlPointConstraint record (15 doubles)."""
    rec = np.ascontiguousarray(record, np.float64)
    W = np.zeros(9)
    ok = lib().orc_control_point_whitening(rec.ctypes.data, W.ctypes.data)
    return bool(ok), W.reshape(3, 3)


def scale_bars(problem):
    """(tracks int32 [n, 2], records float64 [n, 3]: distance, sigma, weight) of the problem's
    scale bars."""
    bars = getattr(problem, "scaleBarConstraints", None) or []
    tracks = np.ascontiguousarray(np.array([(b.trackIndexA, b.trackIndexB) for b in bars], np.int32).reshape(-1, 2))
    data = np.ascontiguousarray(np.array([(b.measuredDistanceMeters, b.sigmaMeters, b.weight) for b in bars],
                                         np.float64).reshape(-1, 3))
    return tracks, data


def control_points(problem):
    """(track int32 [n], records float64 [n, 15]) of Problem.controlPoints."""
    cps = getattr(problem, "controlPoints", None) or []
    track = np.ascontiguousarray([t for t, _ in cps], np.int32)
    data = np.ascontiguousarray(np.array([c.record() for _, c in cps], np.float64).reshape(-1, 15))
    return track, data


class Oracle:
    """One oracle instance over a problem (holds the active problem and the reduced system)."""

    def __init__(self, problem, options, num_threads: int = 0, linear_solver: int = 0, residual_gate: bool = True):
        self.problem = p = problem.normalized()
        self._keep = [p.cameras, p.points, p.track_offsets, p.obs_camera, p.obs_u, p.obs_v, p.obs_weight,
                      p.obs_scale]
        fixed_c = np.ascontiguousarray(p.fixedCameraIndices, np.int32)
        fixed_t = np.ascontiguousarray(p.fixedTrackIndices, np.int32)
        cp_t, cp_d = control_points(p)
        sb_t, sb_d = scale_bars(p)
        self._keep += [fixed_c, fixed_t, p.cameraCalibrationGroupIds, p.sharedIntrinsicReferenceCameras, cp_t, cp_d,
                       sb_t, sb_d]
        self.desc = OrcProblem(p.n_cameras, _ptr(p.cameras), p.n_tracks, _ptr(p.track_offsets), _ptr(p.points),
                               p.n_obs, _ptr(p.obs_camera), _ptr(p.obs_u), _ptr(p.obs_v), _ptr(p.obs_weight),
                               _ptr(p.obs_scale), fixed_c.size, _ptr(fixed_c), fixed_t.size, _ptr(fixed_t),
                               _ptr(p.cameraCalibrationGroupIds), _ptr(p.sharedIntrinsicReferenceCameras),
                               cp_t.size, _ptr(cp_t) if cp_t.size else None, _ptr(cp_d) if cp_t.size else None,
                               sb_d.shape[0], _ptr(sb_t) if sb_d.shape[0] else None,
                               _ptr(sb_d) if sb_d.shape[0] else None)
        rig = getattr(p, "rig", None)
        if rig is not None and rig.captures:
            arrs = rig.arrays(p.n_cameras)
            self._keep += list(arrs)
            cap, cap_info, sen, sen_info, cam_cap, cam_sen = arrs
            self.desc.n_rig_captures = cap.shape[0]
            self.desc.rig_captures = _ptr(cap)
            self.desc.rig_capture_info = _ptr(cap_info)
            self.desc.n_rig_sensors = sen.shape[0]
            self.desc.rig_sensors = _ptr(sen)
            self.desc.rig_sensor_info = _ptr(sen_info)
            self.desc.rig_camera_capture = _ptr(cam_cap)
            self.desc.rig_camera_sensor = _ptr(cam_sen)
        self.opts = make_options(options, num_threads, linear_solver, residual_gate)
        g = p.gauge
        self.opts.gauge_policy = int(g.policy)
        self.opts.gauge_anchor_camera = g.referenceAnchorCameraIndex
        self.opts.gauge_scale_camera = g.referenceScaleCameraIndex
        self.opts.gauge_baseline = g.referenceBaseline
        st = C.c_int32(0)
        self.h = lib().orc_create(C.byref(self.desc), C.byref(self.opts), C.byref(st))
        self.status = st.value

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        counts = np.zeros(16, np.int32)
        base = C.c_double(0)
        lib().orc_info(self.h, _ptr(counts), C.byref(base))
        keys = ["primary", "camera_blocks", "intrinsic_blocks", "track_blocks", "active_tracks",
                "observation_count", "rejected_initial_tracks", "n_pairs", "gauge_anchor", "gauge_scale",
                "fixed_cameras", "first_fixed_camera", "ref_param"]
        d = {k: int(v) for k, v in zip(keys, counts)}
        d["gauge_baseline"] = base.value
        return d

    def active(self):
        p = self.problem
        at = np.zeros(p.n_tracks, np.int8)
        tb = np.zeros(p.n_tracks, np.int32)
        cb = np.zeros(p.n_cameras, np.int32)
        ib = np.zeros(p.n_cameras, np.int32)
        lib().orc_active(self.h, _ptr(at), _ptr(cb), _ptr(ib), _ptr(tb))
        return {"active_track": at, "camera_block": cb, "intrinsic_block": ib, "track_block": tb}

    def linearize_observations(self):
        n = self.problem.n_obs
        out = {"residual": np.zeros((n, 2)), "point_jacobian": np.zeros((n, 2, 3)),
               "pose_jacobian": np.zeros((n, 2, _P)), "intrinsic_jacobian": np.zeros((n, 2, _P)),
               "normal_weight": np.zeros(n), "cost": np.zeros(n), "valid": np.zeros(n, np.int8)}
        lib().orc_linearize_observations(self.h, *(_ptr(out[k]) for k in
                                                  ["residual", "point_jacobian", "pose_jacobian",
                                                   "intrinsic_jacobian", "normal_weight", "cost", "valid"]))
        return out

    def build(self, damping: float = 0.0):
        cost = C.c_double(0)
        sing = C.c_int32(0)
        rc = lib().orc_build(self.h, damping, C.byref(cost), C.byref(sing))
        if rc != 0:
            raise RuntimeError(f"oracle build failed ({rc})")
        return cost.value, bool(sing.value)

    def reduced(self):
        info = self.info()
        P, npairs = info["primary"], info["n_pairs"]
        pairs = np.zeros((npairs, 2), np.int32)
        diag = np.zeros((P, _P, _P))
        off = np.zeros((npairs, _P, _P))
        grad = np.zeros(P * _P)
        direct = np.zeros(P * _P)
        lib().orc_pairs(self.h, _ptr(pairs))
        lib().orc_reduced(self.h, _ptr(diag), _ptr(off), _ptr(grad), _ptr(direct))
        return {"pairs": pairs, "diag": diag, "off": off, "gradient": grad, "direct_rhs": direct}

    def dense_reduced(self):
        r = self.reduced()
        P = r["diag"].shape[0]
        S = np.zeros((P * _P, P * _P))
        for b in range(P):
            S[b * _P:(b + 1) * _P, b * _P:(b + 1) * _P] = r["diag"][b]
        for s, (i, j) in enumerate(r["pairs"]):
            S[i * _P:(i + 1) * _P, j * _P:(j + 1) * _P] = r["off"][s]
            S[j * _P:(j + 1) * _P, i * _P:(i + 1) * _P] = r["off"][s].T
        return S, r

    def solve_linear(self):
        P = self.info()["primary"]
        step = np.zeros(P * _P)
        cv = C.c_int32(0)
        it = C.c_int32(0)
        rc = lib().orc_solve_linear(self.h, _ptr(step), C.byref(cv), C.byref(it))
        if rc != 0:
            raise RuntimeError("oracle linear solve failed")
        return step, bool(cv.value), it.value

    def back_substitute(self, step):
        info = self.info()
        elim = np.zeros(info["track_blocks"] * 3)
        dd = C.c_double(0)
        ok = C.c_int32(0)
        step = np.ascontiguousarray(step, np.float64)
        lib().orc_back_substitute(self.h, _ptr(step), _ptr(elim), C.byref(dd), C.byref(ok))
        return elim, dd.value, bool(ok.value)

    def cost(self):
        return lib().orc_cost(self.h)

    def general_equations(self):
        """Block normal equations of the general path at the current state (buildNormalEquations):
        dense primary matrix, primary gradient, eliminated blocks and gradient, couplings."""
        cost = C.c_double(0)
        counts = np.zeros(3, np.int32)
        if lib().orc_general_build(self.h, C.byref(cost), _ptr(counts)) != 0:
            raise RuntimeError("oracle general build failed")
        P, E, nc = (int(v) for v in counts)
        n = P * _P
        out = {"cost": cost.value, "H": np.zeros((n, n)), "g": np.zeros(n), "Hee": np.zeros((E, 3, 3)),
               "ge": np.zeros((E, 3)), "coupling_index": np.zeros((nc, 2), np.int32), "W": np.zeros((nc, _P, 3))}
        lib().orc_general_export(self.h, *(_ptr(out[k]) for k in ("H", "g", "Hee", "ge", "coupling_index", "W")))
        return out

    def general_solve(self, damping, tolerance=1e-12):
        """solveDampedSchurComplement restated on the equations of the last general_equations()."""
        info = self.info()
        x = np.zeros(info["primary"] * _P)
        y = np.zeros(info["track_blocks"] * 3)
        cv = C.c_int32(0)
        if lib().orc_general_solve(self.h, damping, tolerance, _ptr(x), _ptr(y), C.byref(cv)) != 0:
            raise RuntimeError("oracle general solve failed (not numerically SPD)")
        return x, y, bool(cv.value)

    def solve(self):
        p = self.problem
        rep = OrcReport()
        cams = np.zeros_like(p.cameras)
        pts = np.zeros_like(p.points)
        valid = np.zeros(p.n_tracks, np.int8)
        rb = np.zeros(p.n_tracks)
        ra = np.zeros(p.n_tracks)
        intr = np.zeros((max(1, p.n_cameras), _P))
        lib().orc_solve(self.h, C.byref(rep), _ptr(cams), _ptr(pts), _ptr(valid), _ptr(rb), _ptr(ra), _ptr(intr))
        n_groups = self.info()["intrinsic_blocks"]
        out = {"report": rep.as_dict(), "cameras": cams, "points": pts, "valid": valid.astype(bool),
               "rms_before": rb, "rms_after": ra, "intrinsics": intr[:n_groups]}
        rig = self.rig()
        if rig is not None:
            out.update(rig)
        return out

    def rig(self):
        """Rig problems: current captures and sensors (12 doubles each) and their rig blocks."""
        rig = getattr(self.problem, "rig", None)
        if rig is None or not rig.captures:
            return None
        cap = np.zeros((len(rig.captures), 12))
        sen = np.zeros((len(rig.sensors), 12))
        kb = np.zeros(len(rig.captures), np.int32)
        sb = np.zeros(len(rig.sensors), np.int32)
        if lib().orc_rig(self.h, _ptr(cap), _ptr(sen), _ptr(kb), _ptr(sb)) != 0:
            return None
        return {"captures": cap, "sensors": sen, "capture_block": kb, "sensor_block": sb}
