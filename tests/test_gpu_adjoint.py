"""GPU backward pass (pb_gpu_backward) against the CPU implicit-differentiation reference and
against central finite differences of re-converged solves.

Workload: an aerial grid of 30 cameras (6 x 5) and 3 000 points, two calibration groups refining
f, cx, cy, k1-k3, p1, p2, Cauchy loss at 1.5 px; loss L = sum_i |C_i - (C_i_true + N(0, 0.1 m))|^2
over the refined camera centres.  Tolerances: the GPU and the CPU reference evaluate the same
mathematics at the same state in FP64 but solve the exact Hessian, whose Jacobi-scaled
condition number is about 3e10 here, by different methods (reduced dense-Cholesky-preconditioned
CG against sparse LU of the full Hessian with refinement), so they agree to about eps * kappa:
relative 1e-6 on the gradient vectors (observed about 1e-7).  The finite differences (h = 1e-3
px, 16 observations) carry their own truncation and re-convergence error: relative 1e-4, the
stated bar for the adjoint.
"""
import numpy as np
import pytest

from plabundle_gb300 import synth
from plabundle_gb300.adjoint import camera_centre_loss, newton_polish, polish
from plabundle_gb300.problem import ImageRobustLoss, Precision, SolveOptions

pytestmark = pytest.mark.gpu


def _options(mixed=False):
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Cauchy
    o.solver.imageRobustLossScalePixels = 1.5
    o.calibration.refineSharedFocalLength = True
    o.calibration.refineSharedPrincipalPoint = True
    o.calibration.refineSharedRadialDistortion = True
    o.backend.enablePlaMatrixMixedPrecision = mixed
    o.solver.maxIterations = 100
    return o


@pytest.fixture(scope="module")
def solved():
    from plabundle_gb300.device import Gb300Context
    import orc_adjoint as A
    p = synth.aerial_grid_problem(seed=21, n_along=6, n_lines=5, n_points=3000)
    ctx = Gb300Context(0)
    assert ctx.upload(p, _options()) == 0
    rep = ctx.solve()
    assert rep["status"] == 1
    trace = newton_polish(ctx, iterations=4)
    d = ctx.download()
    T = A.centre_targets(p.truth_cameras, 0.1, seed=4)
    L, g = camera_centre_loss(d["cameras"], T)
    out = ctx.backward(grad_cameras=g)
    yield {"p": p, "ctx": ctx, "d": d, "T": T, "L": L, "g": g, "out": out, "trace": trace}
    ctx.close()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_backward_matches_cpu_implicit_differentiation(solved):
    import oracle as O
    import orc_adjoint as A
    p, d, T, out = solved["p"], solved["d"], solved["T"], solved["out"]
    assert out["report"]["relative_residual"] < 1e-10
    orc = O.Oracle(p, _options())
    adj = A.AdjointOracle(orc, d["cameras"], d["points"], d["intrinsics"])
    z = np.zeros(adj.n_vars)
    L, dL = adj.centre_loss(z, T)
    assert abs(L - solved["L"]) <= 1e-12 * L
    tot, _ = adj.implicit(dL, z)
    go = adj.observation_gradient(tot, p.n_obs)
    gi = adj.initial_pose_gradient(tot, p.cameras)
    assert _rel(out["observations"], go) < 1e-6
    assert _rel(out["initial_cameras"], gi) < 1e-6
    # only fixed cameras and the gauge pair carry initial-pose gradients
    nz = np.nonzero(np.abs(out["initial_cameras"]).sum(1))[0]
    assert set(nz.tolist()) <= {adj.anchor, adj.scale}
    assert np.all(out["initial_points"] == 0.0)


def test_backward_matches_finite_differences(solved):
    p, ctx, T, out = solved["p"], solved["ctx"], solved["T"], solved["out"]
    go = out["observations"]
    ctx.save_state()
    rng = np.random.default_rng(7)
    cand = np.nonzero(np.abs(go).sum(1) > 0)[0]
    pick = rng.choice(cand, 16, replace=False)
    h = 1e-3
    fd = np.zeros((pick.size, 2))
    try:
        for i, k in enumerate(pick):
            for a in range(2):
                vals = []
                for sgn in (1.0, -1.0):
                    u, v = p.obs_u[k], p.obs_v[k]
                    ctx.set_observations([k], [u + sgn * h * (a == 0)], [v + sgn * h * (a == 1)])
                    ctx.restore_state()
                    newton_polish(ctx, iterations=3)
                    vals.append(camera_centre_loss(ctx.download()["cameras"], T)[0])
                    ctx.set_observations([k], [u], [v])
                fd[i, a] = (vals[0] - vals[1]) / (2.0 * h)
    finally:
        ctx.restore_state()
    assert _rel(go[pick], fd) < 1e-4, np.c_[go[pick], fd]


def test_backward_mixed_precision_context_agrees(solved):
    """The mixed path factors H in FP32 and runs the CG in FP64: same gradients to CG tolerance."""
    from plabundle_gb300.device import Gb300Context
    p, d, out = solved["p"], solved["d"], solved["out"]
    ctx = Gb300Context(0)
    try:
        assert ctx.upload(p, _options(mixed=True)) == 0
        rep = ctx.solve()
        assert rep["status"] == 1
        newton_polish(ctx, iterations=4)
        d2 = ctx.download()
        # same fixed point, so nearly the same state and gradient
        _, g2 = camera_centre_loss(d2["cameras"], solved["T"])
        out2 = ctx.backward(grad_cameras=g2)
        assert out2["report"]["relative_residual"] < 1e-10
        assert _rel(out2["observations"], out["observations"]) < 1e-5
    finally:
        ctx.close()


def test_newton_polish_converges_quadratically_to_the_gauss_newton_fixed_point(solved):
    """Exact-Hessian Newton steps from the LM solution: within two steps the reduced gradient
    falls by more than four orders of magnitude, to the rounding floor of its FP64 evaluation
    (pixel residuals of ~1e3 px carry ~1e-13 px of rounding, times Jacobians of ~1e3 and summed
    over thousands of observations per camera), and the steps shrink to ~1e-9.  Full
    Gauss-Newton steps from there do not move the state."""
    trace = solved["trace"]
    g = [gn for _, gn in trace]
    steps = [sm for sm, _ in trace]
    assert g[2] < 1e-4 * g[0], g
    assert steps[-1] < 1e-3 * steps[0], steps
    ctx = solved["ctx"]
    ctx.save_state()
    try:
        before = ctx.download()["cameras"][:, 9:12].copy()
        polish(ctx, iterations=3)
        after = ctx.download()["cameras"][:, 9:12]
        assert np.abs(after - before).max() < 1e-9
    finally:
        ctx.restore_state()
