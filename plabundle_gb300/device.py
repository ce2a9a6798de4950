"""Thin object wrapper over the per-kernel C ABI entry points (upload, linearise, Schur,
reduced solve, back-substitution, objective, solve, download)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native
from .problem import Precision, Problem, SolveOptions

P = 13


class Gb300Context:
    def __init__(self, device: int = 0):
        self.L = native.load()
        self.ctx = C.c_void_p()
        st = self.L.pb_gpu_create(device, C.byref(self.ctx))
        if st != 0:
            raise native.BackendUnavailable(f"pb_gpu_create failed: {self.L.pb_status_name(st).decode()}")
        self._keep = None
        self.problem = None

    def close(self):
        if self.ctx:
            self.L.pb_gpu_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        native.check(self.L, self.ctx, st, what)

    def upload(self, problem: Problem, options: SolveOptions):
        desc, keep = native.problem_desc(problem)
        self.copts = native.solve_options(options, problem)
        self._keep = (desc, keep)
        self.problem = keep[0]
        return self.L.pb_gpu_upload(self.ctx, C.byref(desc), C.byref(self.copts))

    def sizes(self):
        s = np.zeros(16, np.int64)
        base = C.c_double(0)
        self._check(self.L.pb_gpu_get_sizes(self.ctx, s.ctypes.data, C.byref(base)), "sizes")
        keys = ["n_cameras", "n_tracks", "n_obs", "primary", "camera_blocks", "intrinsic_blocks", "track_blocks",
                "active_tracks", "observation_count", "rejected_initial_tracks", "n_pairs", "dim", "ni",
                "gauge_anchor", "gauge_scale", "chunks"]
        d = {k: int(v) for k, v in zip(keys, s)}
        d["gauge_baseline"] = base.value
        return d

    def active(self):
        p = self.problem
        at = np.zeros(p.n_tracks, np.int8)
        tb = np.zeros(p.n_tracks, np.int32)
        cb = np.zeros(p.n_cameras, np.int32)
        ib = np.zeros(p.n_cameras, np.int32)
        self._check(self.L.pb_gpu_get_active(self.ctx, at.ctypes.data, cb.ctypes.data, ib.ctypes.data, tb.ctypes.data),
                    "active")
        return {"active_track": at, "camera_block": cb, "intrinsic_block": ib, "track_block": tb}

    def pairs(self):
        n = self.sizes()["n_pairs"]
        out = np.zeros((n, 2), np.int32)
        self._check(self.L.pb_gpu_get_pairs(self.ctx, out.ctypes.data), "pairs")
        return out

    def linearize_observations(self, precision=Precision.Fp64):
        n = self.problem.n_obs
        out = {"residual": np.zeros((n, 2)), "point_jacobian": np.zeros((n, 2, 3)),
               "pose_jacobian": np.zeros((n, 2, P)), "intrinsic_jacobian": np.zeros((n, 2, P)),
               "normal_weight": np.zeros(n), "cost": np.zeros(n), "valid": np.zeros(n, np.int8)}
        self._check(self.L.pb_gpu_linearize_observations(
            self.ctx, int(precision), *(out[k].ctypes.data for k in
                                        ["residual", "point_jacobian", "pose_jacobian", "intrinsic_jacobian",
                                         "normal_weight", "cost", "valid"])), "linearize")
        return out

    def linearize_schur(self, damping=0.0, precision=Precision.Fp64):
        cost = C.c_double(0)
        sing = C.c_int32(0)
        st = self.L.pb_gpu_linearize_schur(self.ctx, damping, int(precision), C.byref(cost), C.byref(sing))
        self._check(st, "linearize_schur")
        return cost.value, bool(sing.value)

    def reduced(self):
        n = self.sizes()["dim"]
        S = np.zeros((n, n))
        rhs = np.zeros(n)
        direct = np.zeros(n)
        self._check(self.L.pb_gpu_get_reduced(self.ctx, S.ctypes.data, rhs.ctypes.data, direct.ctypes.data), "reduced")
        return S, rhs, direct

    def solve_reduced(self):
        n = self.sizes()["dim"]
        step = np.zeros(n)
        cv = C.c_int32(0)
        it = C.c_int32(0)
        rr = C.c_double(0)
        st = self.L.pb_gpu_solve_reduced(self.ctx, step.ctypes.data, C.byref(cv), C.byref(it), C.byref(rr))
        self._check(st, "solve_reduced")
        return step, bool(cv.value), it.value, rr.value

    def back_substitute(self):
        n = self.sizes()["track_blocks"]
        elim = np.zeros(n * 3)
        dd = C.c_double(0)
        ok = C.c_int32(0)
        self._check(self.L.pb_gpu_back_substitute(self.ctx, elim.ctypes.data, C.byref(dd), C.byref(ok)), "backsub")
        return elim, dd.value, bool(ok.value)

    def cost(self):
        c = C.c_double(0)
        self._check(self.L.pb_gpu_eval_cost(self.ctx, C.byref(c)), "cost")
        return c.value

    def cost_batch(self, alphas):
        a = np.ascontiguousarray(alphas, np.float64)
        out = np.zeros(a.size)
        self._check(self.L.pb_gpu_eval_cost_batch(self.ctx, a.ctypes.data, a.size, out.ctypes.data), "cost_batch")
        return out

    def solve(self):
        rep = native.SolveReportC()
        self._check(self.L.pb_gpu_solve(self.ctx, C.byref(self.copts), C.byref(rep)), "solve")
        return rep.as_dict()

    def stream_handle(self) -> int:
        s = C.c_void_p()
        self._check(self.L.pb_gpu_get_stream(self.ctx, C.byref(s)), "stream")
        return s.value or 0

    def set_timing(self, on: bool):
        self.L.pb_gpu_set_timing(self.ctx, 1 if on else 0)

    def kernel_times(self):
        out = np.zeros(8)
        self.L.pb_gpu_kernel_times(self.ctx, out.ctypes.data)
        return {"assemble_ms": out[0], "assemble_launches": int(out[1]), "pcg_ms": out[2],
                "pcg_launches": int(out[3]), "cost_ms": out[4], "cost_launches": int(out[5]),
                "reduce_ms": out[6], "reduce_launches": int(out[7])}

    def download(self):
        p = self.problem
        cams = np.zeros_like(p.cameras)
        pts = np.zeros_like(p.points)
        valid = np.zeros(p.n_tracks, np.int8)
        rb = np.zeros(p.n_tracks)
        ra = np.zeros(p.n_tracks)
        ng = self.sizes()["intrinsic_blocks"]
        intr = np.zeros((max(1, ng), P))
        self._check(self.L.pb_gpu_download_state(self.ctx, cams.ctypes.data, pts.ctypes.data, valid.ctypes.data,
                                                 rb.ctypes.data, ra.ctypes.data, intr.ctypes.data), "download")
        return {"cameras": cams, "points": pts, "valid": valid.astype(bool), "rms_before": rb, "rms_after": ra,
                "intrinsics": intr[:ng]}

    def history(self):
        """Cost history of the last solve: LM iterations, costs and host ms since the solve
        started (the initial cost, then every accepted step)."""
        n = C.c_int32(0)
        self._check(self.L.pb_gpu_get_history(self.ctx, 0, None, None, None, C.byref(n)), "history")
        it = np.zeros(n.value, np.int32)
        cost = np.zeros(n.value)
        ms = np.zeros(n.value)
        self._check(self.L.pb_gpu_get_history(self.ctx, n.value, it.ctypes.data, cost.ctypes.data, ms.ctypes.data,
                                               C.byref(n)), "history")
        return {"iterations": it, "cost": cost, "ms": ms}

    def rig(self):
        """Rig problems: current captures and sensors (12 doubles each) and their pose blocks."""
        st = native.rig_state(self.L, self.ctx, self.problem)
        if st is None:
            return None
        cap, sen, kb, sb = st
        return {"captures": cap, "sensors": sen, "capture_block": kb, "sensor_block": sb}

    # ---- snapshot / measurement updates / backward pass -------------------------------------
    def save_state(self):
        self._check(self.L.pb_gpu_save_state(self.ctx), "save_state")

    def restore_state(self):
        self._check(self.L.pb_gpu_restore_state(self.ctx), "restore_state")

    def set_observations(self, index, u, v):
        idx = np.ascontiguousarray(index, np.int64)
        uu = np.ascontiguousarray(u, np.float64)
        vv = np.ascontiguousarray(v, np.float64)
        self._check(self.L.pb_gpu_set_observations(self.ctx, idx.size, idx.ctypes.data, uu.ctypes.data, vv.ctypes.data),
                    "set_observations")

    def backward(self, grad_cameras=None, grad_points=None, grad_intrinsics=None):
        """dL/d(observations), dL/d(initial poses), dL/d(initial points) of a scalar loss of the
        converged state (pb_gpu_backward); the inputs are dL/d(final state) in the solver's chart."""
        p = self.problem
        def arr(a, shape):
            return None if a is None else np.ascontiguousarray(np.broadcast_to(a, shape), np.float64)
        gc = arr(grad_cameras, (p.n_cameras, 6))
        gp = arr(grad_points, (p.n_tracks, 3))
        ng = self.sizes()["intrinsic_blocks"]
        gi = arr(grad_intrinsics, (max(1, ng), P)) if grad_intrinsics is not None else None
        go = np.zeros((p.n_obs, 2))
        gic = np.zeros((p.n_cameras, 6))
        gip = np.zeros((p.n_tracks, 3))
        rep = native.AdjointReportC()
        ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
        self._check(self.L.pb_gpu_backward(self.ctx, ptr(gc), ptr(gp), ptr(gi), go.ctypes.data, gic.ctypes.data,
                                           gip.ctypes.data, C.byref(rep)), "backward")
        return {"observations": go, "initial_cameras": gic, "initial_points": gip, "report": rep.as_dict()}

    def newton_step(self):
        """One exact-Hessian Newton step from the current state (pb_gpu_newton_step); returns
        (largest primary step component, reduced gradient norm before the step)."""
        sm = C.c_double(0)
        gn = C.c_double(0)
        self._check(self.L.pb_gpu_newton_step(self.ctx, C.byref(sm), C.byref(gn)), "newton_step")
        return sm.value, gn.value

