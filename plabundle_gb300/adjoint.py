"""Backward pass of a converged bundle adjustment (pb_gpu_backward) and its helpers.

No counterpart in the reference, which has no adjoint.  `Gb300Context.backward` returns the
gradients of a scalar loss of the refined state with respect to every 2D observation and every
initial pose, by implicit differentiation of the LM fixed point with the exact Hessian.

    ctx = Gb300Context(0); ctx.upload(problem, options); ctx.solve()
    polish(ctx)                                  # optional: Gauss-Newton to the fixed point
    cams = ctx.download()["cameras"]
    L, g = camera_centre_loss(cams, targets)     # L = sum |C_i - T_i|^2, g = dL/d(final pose)
    out = ctx.backward(grad_cameras=g)           # out["observations"]: dL/d(u, v)
"""
from __future__ import annotations

import numpy as np

from .problem import Precision


def camera_centre_loss(cameras: np.ndarray, targets: np.ndarray):
    """L = sum_i |C_i - T_i|^2 over the camera centres and its gradient w.r.t. the final poses in
    the backward pass's layout (n_cameras x 6: rotation increment, world centre)."""
    d = cameras[:, 9:12] - targets
    g = np.zeros((cameras.shape[0], 6))
    g[:, 3:6] = 2.0 * d
    return float((d * d).sum()), g


def newton_polish(ctx, iterations: int = 6, tol: float = 0.0):
    """Exact-Hessian Newton steps from a converged state (pb_gpu_newton_step): quadratic
    convergence to the fixed point, where the Gauss-Newton steps of `polish` converge linearly
    (slowly, when the robust loss's curvature makes the exact Hessian much smaller than
    J^T W J).  The fixed point is the zero of the gradient either way.  Returns the list of
    (largest step component, reduced gradient norm) per step."""
    trace = []
    for _ in range(iterations):
        sm, gn = ctx.newton_step()
        trace.append((sm, gn))
        if tol > 0.0 and sm <= tol:
            break
    return trace


def polish(ctx, iterations: int = 8, precision=Precision.Fp64, tol: float = 0.0):
    """Full Gauss-Newton steps (no damping, no line search) from the current state: converges
    to the same fixed point as the LM solve, past its stopping rule (step RMS 1e-6).  Returns the
    objective after the last step.  Use it only from a converged state."""
    cost = None
    for _ in range(iterations):
        cost, singular = ctx.linearize_schur(0.0, precision)
        if singular:
            raise RuntimeError("singular point block while polishing")
        step, converged, _, _ = ctx.solve_reduced()
        ctx.back_substitute()
        ctx._check(ctx.L.pb_gpu_apply_step(ctx.ctx, 1.0), "apply_step")
        if tol > 0.0 and np.max(np.abs(step)) <= tol:
            break
    return ctx.cost() if cost is not None else None
