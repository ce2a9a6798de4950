"""Scale bars on the general path (ScaleBarConstraint, include/plabundle/constraints.h:93-101).

The tracks of a bar become primary point blocks (prepareActiveProblem,
BundleAdjustPlaMatrixProblem.cpp:235-266), the bar adds a Huber-weighted 1-D residual
s (|X_a - X_b| - L) on them (linearizeScaleBar, BundleAdjustPlaMatrixConstraints.cpp:118-153;
assembleScaleBars, BundleAdjustPlaMatrixAssemblySurvey.cpp:131-186), the problem gets an absolute
scale (no baseline camera in the automatic gauge) and is solved on the general path
(canUseReferenceOnlineSchur, BundleAdjustPlaMatrixReferenceSchur.cpp:667-673).

CPU: the oracle's restatement (gradient of the bar terms against central differences of its own
objective, validation, gauge, convergence).  GPU: the device path (the reduced system extended by
the promoted points, pb_survey.cu) against the oracle's general path on the 20-camera ring and a
20-camera aerial block with shared intrinsics and control points, and the statistics of the
public solve.
"""
import copy

import numpy as np
import pytest

import oracle as O
from plabundle_gb300 import synth
from plabundle_gb300.problem import ImageRobustLoss, ScaleBarConstraint, SolveOptions, SolveStatus

KP = 13


def ring_with_bars(n=4):
    p = synth.ring_problem()
    return synth.with_scale_bars(p, n=n, sigma=0.005, seed=1, max_length=2.0)


def aerial_with_bars():
    p = synth.aerial_grid_problem(seed=3, n_along=5, n_lines=4, n_points=3000)
    synth.with_control_points(p, n=8, sigma=0.02, seed=2)
    return synth.with_scale_bars(p, n=6, sigma=0.005, seed=4, max_length=25.0)


def ring_options(mixed=False):
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Huber
    o.solver.imageRobustLossScalePixels = 1.5
    o.backend.enablePlaMatrixMixedPrecision = mixed
    return o


def aerial_options(mixed=False):
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Cauchy
    o.solver.imageRobustLossScalePixels = 1.5
    o.calibration.refineSharedFocalLength = True
    o.calibration.refineSharedPrincipalPoint = True
    o.calibration.refineSharedRadialDistortion = True
    o.solver.maxIterations = 60
    o.backend.enablePlaMatrixMixedPrecision = mixed
    return o


def bar_residuals(problem, points):
    return np.array([np.linalg.norm(points[b.trackIndexA] - points[b.trackIndexB]) - b.measuredDistanceMeters
                     for b in problem.scaleBarConstraints])


def test_oracle_promotes_the_bar_tracks_and_takes_the_scale_from_the_bars():
    p = ring_with_bars()
    orc = O.Oracle(p, ring_options())
    assert orc.status == 0
    info = orc.info()
    bar_tracks = {t for b in p.scaleBarConstraints for t in (b.trackIndexA, b.trackIndexB)}
    act = orc.active()
    promoted = [t for t in bar_tracks if act["active_track"][t]]
    # promoted tracks are primary blocks, not eliminated ones; the cameras come first
    assert info["primary"] == info["camera_blocks"] + len(promoted)
    assert all(act["track_block"][t] < 0 for t in promoted)
    # absolute scale from the bars: camera 0 fixed, no fixed-baseline camera
    assert info["fixed_cameras"] == 1 and info["first_fixed_camera"] == 0 and info["gauge_scale"] == -1
    assert info["ref_param"] == 0


def test_oracle_bar_gradient_matches_central_differences():
    """g = sum w J^T r of the general equations in a promoted block equals the derivative of the
    oracle's objective with respect to that point (IRLS weight = the robust loss's derivative)."""
    p = ring_with_bars(2)
    opts = ring_options()
    orc = O.Oracle(p, opts)
    eq = orc.general_equations()
    info = orc.info()
    b = p.scaleBarConstraints[0]
    t = b.trackIndexA
    # primary block of the track: cameras, then the promoted tracks in track order
    bar_tracks = sorted({tt for bb in p.scaleBarConstraints for tt in (bb.trackIndexA, bb.trackIndexB)})
    pb = info["camera_blocks"] + bar_tracks.index(t)
    h = 1e-6
    for a in range(3):
        costs = []
        for s in (1.0, -1.0):
            q = copy.deepcopy(p)
            q.points = np.array(p.points, copy=True)
            q.points[t, a] += s * h
            costs.append(O.Oracle(q, opts).cost())
        fd = (costs[0] - costs[1]) / (2 * h)
        assert abs(eq["g"][pb * KP + a] - fd) <= 1e-5 * max(1.0, abs(fd)), (a, eq["g"][pb * KP + a], fd)


@pytest.mark.parametrize("bad", [
    dict(trackIndexA=3, trackIndexB=3),
    dict(trackIndexA=-1),
    dict(measuredDistanceMeters=0.0),
    dict(sigmaMeters=float("nan")),
    dict(weight=-1.0),
])
def test_oracle_rejects_an_invalid_bar(bad):
    p = ring_with_bars(1)
    b = p.scaleBarConstraints[0]
    for k, v in bad.items():
        setattr(b, k, v)
    assert O.Oracle(p, ring_options()).status != 0


def test_oracle_general_path_with_bars_converges_and_fits_the_bars():
    p = ring_with_bars()
    ref = O.Oracle(p, ring_options(), residual_gate=False).solve()
    assert ref["report"]["status"] == SolveStatus.Success
    before = np.abs(bar_residuals(p, p.points)).mean()
    after = np.abs(bar_residuals(p, ref["points"])).mean()
    assert after < 0.2 * before, (before, after)


def solve_gpu(problem, options):
    from plabundle_gb300.device import Gb300Context
    ctx = Gb300Context(0)
    st = ctx.upload(problem, options)
    assert st == 0, ctx.L.pb_gpu_last_error(ctx.ctx)
    rep = ctx.solve()
    out = ctx.download()
    ctx.close()
    return rep, out


def centre_error(out, ref):
    C_ref = ref["cameras"][:, 9:12]
    scale = np.linalg.norm(C_ref - C_ref.mean(0), axis=1).max()
    return np.abs(out["cameras"][:, 9:12] - C_ref).max() / scale


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,opts", [("ring", ring_with_bars, ring_options),
                                            ("aerial", aerial_with_bars, aerial_options)])
def test_device_path_with_bars_follows_the_oracle(name, make, opts):
    """FP64: the oracle's general-path solve (iterations within a few, cost to 1e-9, camera centres
    and the bar points to 1e-7 of the scene extent, identical inliers); mixed: the same fixed point
    (1e-6 cost, 1e-5 centres).  The online path is never used with bars, even when requested."""
    p = make()
    ref = O.Oracle(p, opts(), residual_gate=False).solve()
    rr = ref["report"]
    assert rr["status"] == SolveStatus.Success
    bar_tracks = sorted({t for b in p.scaleBarConstraints for t in (b.trackIndexA, b.trackIndexB)})
    C_ref = ref["cameras"][:, 9:12]
    extent = np.linalg.norm(C_ref - C_ref.mean(0), axis=1).max()
    for mixed in (False, True):
        o = opts(mixed)
        assert o.solver.useReferenceOnlineSchur
        rep, out = solve_gpu(p, o)
        assert rep["general_path_used"] == 1 and rep["promoted_point_blocks"] == len(bar_tracks)
        assert rep["status"] == SolveStatus.Success
        np.testing.assert_allclose(rep["initial_cost"], rr["initial_cost"], rtol=1e-12)
        rel = abs(rep["final_cost"] - rr["final_cost"]) / rr["final_cost"]
        cerr = centre_error(out, ref)
        perr = np.abs(out["points"][bar_tracks] - ref["points"][bar_tracks]).max() / extent
        assert np.array_equal(out["valid"], ref["valid"])
        if not mixed:
            assert abs(rep["iterations"] - rr["iterations"]) <= 3, (rep["iterations"], rr["iterations"])
            assert rel < 1e-9 and cerr < 1e-7 and perr < 1e-7, (rel, cerr, perr)
        else:
            assert rel < 1e-6 and cerr < 1e-5 and perr < 1e-5, (rel, cerr, perr)


@pytest.mark.gpu
def test_public_solve_reports_scale_bar_statistics():
    from plabundle_gb300.solver import Solver, scale_bar_stats
    p = ring_with_bars()
    res = Solver().solve(p, ring_options(True))
    assert res.status == SolveStatus.Success and res.solutionUsable
    q = res.quality
    n, before = scale_bar_stats(p, None, res.points.valid)
    assert q.scaleBarConstraintCount == n == len(p.scaleBarConstraints)
    assert q.scaleBarRmsBeforeMeters == pytest.approx(before)
    assert q.scaleBarRmsAfterMeters < 0.2 * q.scaleBarRmsBeforeMeters


@pytest.mark.gpu
def test_device_rejects_an_invalid_bar():
    from plabundle_gb300.device import Gb300Context
    p = ring_with_bars(1)
    p.scaleBarConstraints.append(ScaleBarConstraint(trackIndexA=5, trackIndexB=5, measuredDistanceMeters=1.0))
    ctx = Gb300Context(0)
    assert ctx.upload(p, ring_options()) != 0
    assert "scale-bar" in ctx.L.pb_gpu_last_error(ctx.ctx).decode()
    ctx.close()
