"""CPU tests of the FP64 oracle: analytic Jacobians against central differences, the
reference's qualitative online-Schur test, and end-to-end convergence on the ring workload.

Parity of the oracle against the reference is unpinned (the reference cannot be built and
has no golden vectors); these tests pin its internal consistency instead.
"""
import numpy as np
import pytest

import oracle as O
from plabundle_gb300 import synth
from plabundle_gb300.problem import (GaugePolicy, ImageRobustLoss, Problem, SolveOptions, SolveStatus)

D = np.diag([1.0, -1.0, -1.0])


def euler(d):
    sx, cx = np.sin(d[0]), np.cos(d[0])
    sy, cy = np.sin(d[1]), np.cos(d[1])
    sz, cz = np.sin(d[2]), np.cos(d[2])
    rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return rx @ ry @ rz


def retract_camera(cam, d):
    """Pose retraction of BundleAdjustPlaMatrixAssembly.cpp:130-179."""
    out = cam.copy()
    R = cam[0:9].reshape(3, 3)
    out[0:9] = (D @ euler(d[:3]).T @ D @ R).reshape(9)
    out[9:12] = cam[9:12] + d[3:6]
    return out


def point_scale(X):
    n = np.linalg.norm(X) / 1000.0
    return 1.0 if n == 0 else n / np.arctan(n)


def residual(cam, X, u, v):
    px, ok = synth.project(cam[None], np.zeros(1, int), X[None])
    assert ok[0]
    return px[0] - np.array([u, v])


def small_ring(seed=3, n_cameras=6, n_points=40):
    return synth.ring_problem(seed=seed, n_cameras=n_cameras, n_points=n_points, outlier_frac=0.0)


def test_analytic_jacobians_match_central_differences():
    p = small_ring()
    opts = SolveOptions()
    orc = O.Oracle(p, opts)
    lin = orc.linearize_observations()
    info = orc.info()
    act = orc.active()
    rng = np.random.default_rng(0)
    checked = 0
    for k in rng.choice(p.n_obs, size=40, replace=False):
        if not lin["valid"][k]:
            continue
        t = int(np.searchsorted(p.track_offsets, k, side="right") - 1)
        c = int(p.obs_camera[k])
        cam, X = p.cameras[c], p.points[t]
        u, v = p.obs_u[k], p.obs_v[k]
        # point columns (scaled point parameterisation)
        for col in range(3):
            h = 1e-6
            e = np.zeros(3)
            e[col] = h * point_scale(X)
            num = (residual(cam, X + e, u, v) - residual(cam, X - e, u, v)) / (2 * h)
            np.testing.assert_allclose(lin["point_jacobian"][k][:, col], num, atol=2e-5 * max(1, np.abs(num).max()))
        if act["camera_block"][c] < 0 or c == info["gauge_scale"]:
            continue
        for col in range(6):
            h = 1e-7 if col >= 3 else 1e-6
            d = np.zeros(6)
            d[col] = h
            num = (residual(retract_camera(cam, d), X, u, v) - residual(retract_camera(cam, -d), X, u, v)) / (2 * h)
            np.testing.assert_allclose(lin["pose_jacobian"][k][:, col], num, atol=2e-5 * max(1, np.abs(num).max()))
        checked += 1
    assert checked > 10


def test_gauge_tangent_columns_match_retraction():
    p = small_ring(seed=5)
    orc = O.Oracle(p, SolveOptions())
    info = orc.info()
    lin = orc.linearize_observations()
    a, s, base = info["gauge_anchor"], info["gauge_scale"], info["gauge_baseline"]
    assert a == 0 and s > 0
    np.testing.assert_allclose(np.linalg.norm(p.cameras[s, 9:12] - p.cameras[a, 9:12]), base)
    origin = D @ p.cameras[a, 9:12]
    centre = D @ p.cameras[s, 9:12]
    unit = (centre - origin) / np.linalg.norm(centre - origin)
    axis_index = 1 if abs(unit[0]) > abs(unit[1]) else 0
    if abs(unit[axis_index]) > abs(unit[2]):
        axis_index = 2
    ax = np.zeros(3)
    ax[axis_index] = 1
    second = np.cross(ax, unit)
    second /= np.linalg.norm(second)
    basis = [np.cross(unit, second), second]

    def tangent_step(cam, da, db):
        tent = centre + basis[0] * da + basis[1] * db
        direction = tent - origin
        new = origin + direction / np.linalg.norm(direction) * base
        out = cam.copy()
        out[9:12] = D @ new
        return out

    ks = np.nonzero((p.obs_camera == s) & (lin["valid"] == 1))[0][:6]
    assert ks.size > 0
    for k in ks:
        t = int(np.searchsorted(p.track_offsets, k, side="right") - 1)
        X = p.points[t]
        for j in range(2):
            h = 1e-7
            dp = [0.0, 0.0]
            dm = [0.0, 0.0]
            dp[j], dm[j] = h, -h
            num = (residual(tangent_step(p.cameras[s], *dp), X, p.obs_u[k], p.obs_v[k])
                   - residual(tangent_step(p.cameras[s], *dm), X, p.obs_u[k], p.obs_v[k])) / (2 * h)
            np.testing.assert_allclose(lin["pose_jacobian"][k][:, 3 + j], num, atol=2e-5 * max(1, np.abs(num).max()))
        assert np.all(lin["pose_jacobian"][k][:, 5] == 0.0)


def native_problem():
    """The three-camera / 24-track problem of test/test_native_problem.cpp:51-94."""
    cams = []
    for cx in (0.0, 1.0, 2.0):
        cams.append(synth.make_camera(np.eye(3), [cx, 0.0, 0.0], 100.0, 100.0, 50.0, 50.0, width=100, height=100))
    truth = np.array(cams)
    init = truth.copy()
    init[2] = synth.make_camera(synth.rotation_from_axis_angle(np.zeros(3)), [2.0, 0, 0], 100, 100, 50, 50,
                                width=100, height=100)
    # applyPoseDelta({0.001, -0.001, 0.0005, 0.02, -0.01, 0.005}) on camera 2
    dR = synth.rotation_from_axis_angle(np.array([0.001, -0.001, 0.0005]))
    init[2, 0:9] = (dR @ truth[2, 0:9].reshape(3, 3)).reshape(9)
    init[2, 9:12] = truth[2, 9:12] + np.array([0.02, -0.01, 0.005])
    pts, offs, cam_idx, us, vs = [], [0], [], [], []
    for i in range(24):
        X = np.array([0.5 * (i % 4) - 0.75, 0.3 * ((i // 4) % 3) - 0.3, 5.0 + 0.2 * (i % 5)])
        pts.append(X + np.array([0.03, -0.02, 0.04]))
        px, ok = synth.project(truth, np.arange(3), np.repeat(X[None], 3, 0))
        assert ok.all()
        cam_idx += [0, 1, 2]
        us += list(px[:, 0])
        vs += list(px[:, 1])
        offs.append(offs[-1] + 3)
    n = len(cam_idx)
    prob = Problem(cameras=init, points=np.array(pts), track_offsets=np.array(offs), obs_camera=np.array(cam_idx),
                   obs_u=np.array(us), obs_v=np.array(vs), obs_weight=np.ones(n), obs_scale=np.ones(n),
                   fixedCameraIndices=[0, 1]).normalized()
    prob.gauge.policy = GaugePolicy.RequireExplicitGauge
    return prob


def native_options():
    opts = SolveOptions()
    opts.solver.useReferenceOnlineSchur = True
    opts.solver.maxIterations = 8
    opts.solver.numThreads = 1
    opts.solver.enablePointFilter = False
    return opts


def test_reference_online_schur_native_problem_decreases_cost():
    orc = O.Oracle(native_problem(), native_options(), num_threads=1)
    assert orc.status == 0
    r = orc.solve()["report"]
    assert r["status"] in (SolveStatus.Success, SolveStatus.NoConvergence)
    assert r["solution_usable"]
    assert r["final_cost"] < r["initial_cost"]


def test_require_explicit_gauge_without_two_fixed_cameras_is_unsupported():
    p = native_problem()
    p.fixedCameraIndices = [0]
    orc = O.Oracle(p, native_options())
    assert orc.status == SolveStatus.UnsupportedConfiguration


@pytest.mark.parametrize("threads", [1, 3])
def test_ring_solve_converges_and_is_thread_count_stable(threads):
    p = synth.ring_problem(seed=7, n_points=600)
    opts = SolveOptions()
    opts.solver.imageRobustLoss = ImageRobustLoss.Huber
    opts.solver.imageRobustLossScalePixels = 1.5
    r = O.Oracle(p, opts, num_threads=threads).solve()
    rep = r["report"]
    assert rep["status"] == SolveStatus.Success
    assert rep["final_cost"] < 0.01 * rep["initial_cost"]
    assert rep["mean_rms_after"] < 0.6
    ref = O.Oracle(p, opts, num_threads=2).solve()
    np.testing.assert_allclose(r["report"]["final_cost"], ref["report"]["final_cost"], rtol=1e-9)


def test_reduced_system_matches_dense_elimination():
    """The online point Schur equals the dense Schur complement of the full normal equations."""
    p = small_ring(seed=9, n_cameras=5, n_points=25)
    orc = O.Oracle(p, SolveOptions())
    orc.build(0.0)
    S, red = orc.dense_reduced()
    lin = orc.linearize_observations()
    act = orc.active()
    info = orc.info()
    P, nt = info["primary"], info["track_blocks"]
    nc = P * 13
    J = np.zeros((2 * p.n_obs, nc + 3 * nt))
    r = np.zeros(2 * p.n_obs)
    w = np.zeros(2 * p.n_obs)
    for k in range(p.n_obs):
        if not lin["valid"][k]:
            continue
        t = int(np.searchsorted(p.track_offsets, k, side="right") - 1)
        if not act["active_track"][t]:
            continue
        c = p.obs_camera[k]
        cb = act["camera_block"][c]
        if cb >= 0:
            J[2 * k:2 * k + 2, cb * 13:(cb + 1) * 13] = lin["pose_jacobian"][k]
        tb = act["track_block"][t]
        J[2 * k:2 * k + 2, nc + 3 * tb:nc + 3 * tb + 3] = lin["point_jacobian"][k]
        r[2 * k:2 * k + 2] = lin["residual"][k]
        w[2 * k:2 * k + 2] = lin["normal_weight"][k]
    H = J.T @ (w[:, None] * J)
    g = J.T @ (w * r)
    Hcc, Hcp, Hpp = H[:nc, :nc], H[:nc, nc:], H[nc:, nc:]
    Sd = Hcc - Hcp @ np.linalg.solve(Hpp, Hcp.T)
    gd = g[:nc] - Hcp @ np.linalg.solve(Hpp, g[nc:])
    live = np.array([i for i in range(nc) if abs(Sd[i, i]) > 0])
    np.testing.assert_allclose(S[np.ix_(live, live)], Sd[np.ix_(live, live)], rtol=1e-9,
                               atol=1e-9 * np.abs(Sd).max())
    np.testing.assert_allclose(red["gradient"][live], gd[live], rtol=1e-9, atol=1e-9 * np.abs(gd).max())
