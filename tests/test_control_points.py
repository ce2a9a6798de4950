"""CPU tests of the control-point (survey target) terms: the whitening of the three uncertainty
forms against the reference's known answers (test/test_covariance_whitening.cpp:39-96), the
product's host validation and gauge decisions against the oracle's, the oracle's objective
against an independent numpy restatement, the plain parameterisation's Jacobian columns against
central differences of its retraction, and the survey frame recovered by the oracle's solve.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from plabundle_gb300 import native, synth
from plabundle_gb300.problem import (ControlPointConstraint, ControlPointUncertainty, GaugePolicy, ImageRobustLoss,
                                     SolveOptions, SolveStatus)

COV = ControlPointUncertainty.Covariance
SQI = ControlPointUncertainty.SqrtInformation


def record(kind, matrix=(0.0,) * 9, sigma=1.0, weight=1.0, point=(0.0, 0.0, 0.0)):
    return ControlPointConstraint(point=point, sigmaMeters=sigma, weight=weight, uncertainty=kind,
                                  uncertaintyMatrix=tuple(matrix)).record()


def host_whitening(probe, rec):
    W = np.zeros(9)
    ok = probe.probe_cp_whitening(np.ascontiguousarray(rec).ctypes.data, W.ctypes.data)
    return bool(ok), W.reshape(3, 3)


def both_whitenings(probe, rec):
    a, Wa = O.control_point_whitening(rec)
    b, Wb = host_whitening(probe, rec)
    assert a == b
    if a:
        np.testing.assert_allclose(Wb, Wa, rtol=1e-14, atol=1e-15)
    return a, Wa


def test_covariance_whitening_gives_identity_information(host_probe):
    """test_covariance_whitening.cpp:39-69: W C W^T = I to 1e-12, RMS uncertainty |W^-1|_F = sqrt(18)."""
    C3 = np.array([[4.0, 2.0, 0.0], [2.0, 5.0, 0.0], [0.0, 0.0, 9.0]])
    ok, W = both_whitenings(host_probe, record(COV, C3.reshape(9)))
    assert ok
    np.testing.assert_allclose(W @ C3 @ W.T, np.eye(3), atol=1e-12)
    assert abs(np.linalg.norm(np.linalg.inv(W)) - np.sqrt(18.0)) < 1e-12


def test_near_singular_covariance_and_information_are_rejected(host_probe):
    """test_covariance_whitening.cpp:71-84."""
    assert not both_whitenings(host_probe, record(COV, np.diag([1.0, 1.0, 1e-14]).reshape(9)))[0]
    assert not both_whitenings(host_probe, record(SQI, np.diag([1.0, 1.0, 0.0]).reshape(9)))[0]


def test_correlated_sqrt_information_is_taken_as_is(host_probe):
    """test_covariance_whitening.cpp:86-96: the whitening is the matrix itself, bit for bit."""
    M = (2.0, 0.5, 0.0, 0.0, 3.0, -0.25, 0.0, 0.0, 4.0)
    ok, W = both_whitenings(host_probe, record(SQI, M))
    assert ok and np.array_equal(W.reshape(9), np.array(M))


@pytest.mark.parametrize("rec,valid", [
    (record(ControlPointUncertainty.IsotropicSigma, sigma=0.02), True),
    (record(ControlPointUncertainty.IsotropicSigma, sigma=0.0), False),
    (record(ControlPointUncertainty.IsotropicSigma, sigma=0.02, weight=0.0), False),
    (record(ControlPointUncertainty.IsotropicSigma, sigma=0.02, weight=float("nan")), False),
    (record(ControlPointUncertainty.IsotropicSigma, sigma=0.02, point=(0.0, float("inf"), 0.0)), False),
    (record(COV, (1.0, 0.5, 0.0, 0.4, 1.0, 0.0, 0.0, 0.0, 1.0)), False),   # not symmetric
    (record(COV, (1.0, 2.0, 0.0, 2.0, 1.0, 0.0, 0.0, 0.0, 1.0)), False),   # indefinite
    (record(SQI, (1.0, 0.0, 0.0, 0.0, float("nan"), 0.0, 0.0, 0.0, 1.0)), False),
])
def test_control_point_validation_matches_the_reference_rules(host_probe, rec, valid):
    """validateControlPointConstraint (control_point.cpp:205-220): finite target, positive
    weight, positive sigma, symmetric positive definite covariance / information."""
    ok, W = both_whitenings(host_probe, rec)
    assert ok == valid
    if ok:
        np.testing.assert_allclose(W, np.eye(3) / 0.02, rtol=1e-15)


def ring_options():
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Huber
    o.solver.imageRobustLossScalePixels = 1.5
    return o


def host_model(probe, problem, options):
    desc, keep = native.problem_desc(problem)
    o = native.solve_options(options, problem)
    out_i = np.zeros(12, np.int32)
    fixed = np.zeros(problem.n_cameras + 2, np.int32)
    out_d = np.zeros(2)
    probe.probe_model(C.byref(desc), C.byref(o), out_i.ctypes.data, fixed.ctypes.data, out_d.ctypes.data)
    del keep
    return {"status": int(out_i[0]), "ref_param": int(out_i[1]), "fixed_cameras": int(out_i[2]),
            "gauge_anchor": int(out_i[3]), "gauge_scale": int(out_i[4]), "kept": int(out_i[5]),
            "camera_blocks": int(out_i[6]), "active_tracks": int(out_i[7]), "observation_count": int(out_i[8]),
            "rejected_initial_tracks": int(out_i[9]), "track_blocks": int(out_i[10]), "first_fixed": int(fixed[0]) if out_i[2] else -1,
            "gauge_baseline": float(out_d[0])}


def base_ring():
    return synth.ring_problem(seed=5, n_cameras=8, n_points=300)


def two_camera_track(p):
    off = np.asarray(p.track_offsets)
    return [t for t in range(p.n_tracks) if np.unique(p.obs_camera[off[t]:off[t + 1]]).size >= 2]


def gcps(p, tracks, points=None):
    pts = p.truth_points if points is None else points
    return [(int(t), ControlPointConstraint(point=tuple(pts[i] if points is not None else pts[t]), sigmaMeters=0.02))
            for i, t in enumerate(tracks)]


def gauge_cases():
    """(name, problem, gauge policy, fixed cameras, expected oracle status)."""
    out = []
    p = synth.with_control_points(base_ring(), n=10)
    out.append(("complete", p, GaugePolicy.AutoAnchor, [], 0))
    p = base_ring()
    t = two_camera_track(p)
    p.controlPoints = gcps(p, t[:1])
    out.append(("one_target_gives_scale", p, GaugePolicy.AutoAnchor, [], 0))
    p = base_ring()
    line = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [2.0, 2.0, 2.0]])
    p.controlPoints = gcps(p, two_camera_track(p)[:3], line)
    out.append(("collinear_targets", p, GaugePolicy.AutoAnchor, [], 0))
    p = base_ring()
    p.controlPoints = gcps(p, two_camera_track(p)[:1], p.cameras[0:1, 9:12])
    out.append(("target_on_the_anchor_centre", p, GaugePolicy.AutoAnchor, [], 0))
    p = base_ring()
    p.controlPoints = gcps(p, two_camera_track(p)[:1])
    out.append(("explicit_one_fixed_and_scale", p, GaugePolicy.RequireExplicitGauge, [2], 0))
    p = synth.with_control_points(base_ring(), n=6)
    out.append(("explicit_complete_targets", p, GaugePolicy.RequireExplicitGauge, [], 0))
    p = base_ring()
    p.controlPoints = gcps(p, two_camera_track(p)[:1])
    out.append(("explicit_without_fixed_camera", p, GaugePolicy.RequireExplicitGauge, [], 5))
    p = synth.with_control_points(base_ring(), n=5)
    p.controlPoints.append((0, ControlPointConstraint(point=(0.0, 0.0, 0.0), sigmaMeters=-1.0)))
    out.append(("invalid_constraint", p, GaugePolicy.AutoAnchor, [], 4))
    return out


@pytest.mark.parametrize("case", gauge_cases(), ids=lambda c: c[0])
def test_host_gauge_and_parameterisation_match_the_oracle(host_probe, case):
    """validateAndNormalizeBundleAdjustOptions (BundleAdjustValidation.cpp:772-893) with control
    points, decided by the product's host planner and by the oracle: status, fixed cameras, the
    anchor / scale cameras of the gauge tangent and its baseline, and the switch to the plain
    parameterisation."""
    name, p, policy, fixed, expected = case
    p.gauge.policy = policy
    p.fixedCameraIndices = list(fixed)
    o = ring_options()
    h = host_model(host_probe, p, o)
    orc = O.Oracle(p, o)
    assert h["status"] == orc.status == expected, (h, orc.status)
    if expected:
        return
    i = orc.info()
    assert h["ref_param"] == i["ref_param"] == 0
    assert h["fixed_cameras"] == i["fixed_cameras"]
    assert h["first_fixed"] == i["first_fixed_camera"]
    assert (h["gauge_anchor"], h["gauge_scale"]) == (i["gauge_anchor"], i["gauge_scale"])
    assert h["gauge_baseline"] == i["gauge_baseline"]
    assert h["camera_blocks"] == i["camera_blocks"]
    if name in ("complete", "explicit_complete_targets"):
        assert i["fixed_cameras"] == 0 and i["gauge_scale"] == -1
    if name in ("one_target_gives_scale", "collinear_targets"):
        assert i["fixed_cameras"] == 1 and i["gauge_scale"] == -1
    if name == "target_on_the_anchor_centre":
        assert i["fixed_cameras"] == 1 and i["gauge_scale"] > 0


def numpy_whitening(c):
    if c.uncertainty == ControlPointUncertainty.IsotropicSigma:
        return np.eye(3) / c.sigmaMeters
    M = np.array(c.uncertaintyMatrix, float).reshape(3, 3)
    if c.uncertainty == COV:
        return np.linalg.inv(np.linalg.cholesky(M))
    return M


def huber(s, delta):
    return 0.5 * s if s <= delta * delta else delta * np.sqrt(s) - 0.5 * delta * delta


@pytest.mark.parametrize("cp_weight", [1.0, 3.0, 0.0])
def test_oracle_objective_adds_the_huber_control_point_costs(cp_weight):
    """evaluateObjective with control points (BundleAdjustPlaMatrixAssembly.cpp:674-690):
    image cost + sum over the active tracks' constraints of Huber_delta(|sqrt(cw w) W (X - P)|^2),
    restated here with numpy whitenings; weight 0 drops the terms but keeps the plain chart."""
    p = synth.with_control_points(base_ring(), n=10)
    o = ring_options()
    o.constraints.controlPointWeight = cp_weight
    orc = O.Oracle(p, o)
    assert orc.status == 0 and orc.info()["ref_param"] == 0
    plain = base_ring()
    ref_img = O.Oracle(plain, o)
    act = orc.active()["active_track"]
    expect = 0.0
    for t, c in p.controlPoints:
        if not act[t]:
            continue
        r = np.sqrt(cp_weight * c.weight) * numpy_whitening(c) @ (p.points[t] - np.array(c.point))
        expect += huber(float(r @ r), o.constraints.controlPointHuberDeltaMeters) if cp_weight > 0 else 0.0
    got = orc.cost() - ref_img.cost()
    assert abs(got - expect) <= 1e-9 * max(1.0, expect), (got, expect)
    if cp_weight > 0:
        assert expect > 0


def exp_left(cam, w):
    out = cam.copy()
    out[0:9] = (synth.rotation_from_axis_angle(np.asarray(w)) @ cam[0:9].reshape(3, 3)).reshape(9)
    return out


def residual(cam, X, u, v):
    px, ok = synth.project(cam[None], np.zeros(1, int), X[None])
    assert ok[0]
    return px[0] - np.array([u, v])


def test_plain_parameterisation_columns_match_its_retraction():
    """With control points the observation Jacobian takes the plain columns (rotation Jw x (X - C),
    BundleAdjustPlaMatrixProjection.cpp:208-214; unscaled point columns), which must be the
    derivatives of the pose delta C2W' = Exp(w) C2W, C' = C + dC and of X' = X + dX."""
    p = synth.with_control_points(synth.ring_problem(seed=3, n_cameras=6, n_points=60, outlier_frac=0.0), n=6)
    orc = O.Oracle(p, SolveOptions())
    lin = orc.linearize_observations()
    act = orc.active()
    rng = np.random.default_rng(1)
    checked = 0
    for k in rng.choice(p.n_obs, size=40, replace=False):
        if not lin["valid"][k]:
            continue
        t = int(np.searchsorted(p.track_offsets, k, side="right") - 1)
        c = int(p.obs_camera[k])
        cam, X, u, v = p.cameras[c], p.points[t], p.obs_u[k], p.obs_v[k]
        for col in range(3):
            e = np.zeros(3)
            e[col] = 1e-6
            num = (residual(cam, X + e, u, v) - residual(cam, X - e, u, v)) / 2e-6
            np.testing.assert_allclose(lin["point_jacobian"][k][:, col], num, atol=2e-5 * max(1, np.abs(num).max()))
        if act["camera_block"][c] < 0:
            continue
        for col in range(6):
            h = 1e-7 if col >= 3 else 1e-6
            d = np.zeros(6)
            d[col] = h
            plus, minus = exp_left(cam, d[:3]), exp_left(cam, -d[:3])
            plus[9:12] += d[3:]
            minus[9:12] -= d[3:]
            num = (residual(plus, X, u, v) - residual(minus, X, u, v)) / (2 * h)
            np.testing.assert_allclose(lin["pose_jacobian"][k][:, col], num, atol=2e-5 * max(1, np.abs(num).max()))
        checked += 1
    assert checked > 10


def test_oracle_solve_recovers_the_survey_frame():
    """Ten targets (sigma 2 cm) fix position, orientation and scale: the converged camera centres
    sit within 8 cm of the truth, where the image-only solve (gauge from the first camera and
    one baseline) is off by decimetres."""
    o = ring_options()
    p = synth.with_control_points(base_ring(), n=10)
    r = O.Oracle(p, o).solve()
    assert r["report"]["status"] == SolveStatus.Success
    err = np.abs(r["cameras"][:, 9:12] - p.truth_cameras[:, 9:12]).max()
    q = base_ring()
    r0 = O.Oracle(q, o).solve()
    err0 = np.abs(r0["cameras"][:, 9:12] - q.truth_cameras[:, 9:12]).max()
    assert err < 0.08 and err < 0.5 * err0, (err, err0)


def test_quality_statistics_whitening_agrees_with_the_oracle():
    """The solver's control-point statistics (RMS uncertainty for the quality gate) whiten the
    constraints as the oracle does."""
    from plabundle_gb300.solver import control_point_rms_uncertainty, control_point_whitening
    p = synth.with_control_points(base_ring(), n=9)
    for _, c in p.controlPoints:
        ok, W = O.control_point_whitening(c.record())
        assert ok
        np.testing.assert_allclose(control_point_whitening(c), W, rtol=1e-12, atol=1e-12)
    o = SolveOptions()
    expect = np.sqrt(np.mean([(np.linalg.inv(O.control_point_whitening(c.record())[1]) ** 2).sum() / c.weight
                              for _, c in p.controlPoints]))
    assert abs(control_point_rms_uncertainty(p, o) - expect) < 1e-12 * expect


def test_unavailable_backend_is_reported_without_running():
    """An explicit backend this build does not provide: BackendUnavailable, no solution, no GPU
    work (src/solver.cpp:450-467; the build has no CPU fallback to run instead)."""
    from plabundle_gb300.problem import Backend
    from plabundle_gb300.solver import Solver
    o = SolveOptions()
    o.backend.requested = Backend.PlaMatrixCpu
    r = Solver().solve(base_ring(), o)
    assert r.status == SolveStatus.BackendUnavailable
    assert not r.solutionUsable and r.usedBackend == Backend.PlaMatrixCpu
    assert "not provided" in r.backendMessage
