"""Rig problems (Problem::rig): captures and shared sensor extrinsics chained to the cameras.

The reference chains a rig camera's pose Jacobian to its capture and sensor blocks
(cameraPosePrimaryTerms, BundleAdjustPlaMatrixAssembly.cpp:207-284), numbers the blocks captures
first, then sensors (prepareActiveProblem, BundleAdjustPlaMatrixProblem.cpp:156-199), updates
captures and sensors with the plain pose delta and composes the cameras again (:1152-1209).

CPU tests: the oracle's chained gradient against central differences of its objective, the host
planner's rig model (blocks, pairs, composed cameras, fixed cameras, sensor groups) against the
oracle bit for bit, the rig term lists by brute force, and the rejected topologies.  GPU tests:
the FP64 path follows the oracle iteration for iteration on the online and general paths (also
with control points and scale bars), the mixed path reaches the oracle's fixed point, and the
reduced system over the rig blocks equals the oracle's.
"""
import copy
import ctypes as C
import dataclasses

import numpy as np
import pytest

import oracle as O
from plabundle_gb300 import native, synth
from plabundle_gb300.problem import (GaugePolicy, ImageRobustLoss, Precision, SolveOptions, SolveStatus)


def rig_block(seed=21, n_along=5, n_lines=3, n_points=2500, **kw):
    kw.setdefault("rot_sigma", 0.001)
    kw.setdefault("centre_sigma", 0.02)
    return synth.rig_grid_problem(seed=seed, n_along=n_along, n_lines=n_lines, n_points=n_points, **kw)


def rig_options(mixed=False, general=False, intrinsics=False, iterations=20, poses=True):
    o = SolveOptions()
    o.calibration.refineCameraPose = poses
    o.solver.imageRobustLoss = ImageRobustLoss.Huber
    o.solver.imageRobustLossScalePixels = 1.5
    o.solver.useReferenceOnlineSchur = not general
    o.solver.maxIterations = iterations
    o.backend.enablePlaMatrixMixedPrecision = mixed
    if intrinsics:
        o.calibration.refineSharedFocalLength = True
        o.calibration.refineSharedPrincipalPoint = True
    return o


def rig_with_groups():
    """Two explicit calibration groups (nadir, obliques) with intrinsics refined."""
    p = rig_block(seed=23)
    p.cameraCalibrationGroupIds = np.array([0 if c % 5 == 0 else 1 for c in range(p.n_cameras)], np.int32)
    return p


def rig_survey():
    """The block with control points and scale bars: general path, promoted bar points."""
    p = synth.with_control_points(rig_block(seed=25), n=12, seed=3)
    return synth.with_scale_bars(p, n=4, seed=5)


def rig_fixed_capture():
    """A fixed capture pose and an explicit two-camera gauge."""
    p = rig_block(seed=27)
    p.rig.captures[3] = dataclasses.replace(p.rig.captures[3], fixedPose=True)
    p.fixedCameraIndices = [0, 10]
    p.gauge.policy = GaugePolicy.RequireExplicitGauge
    return p


def rig_intrinsics_only():
    """Poses held (CalibrationOptions::refineCameraPose = false): no capture or sensor blocks,
    only the two calibration groups are refined."""
    return rig_with_groups()


HOST_CASES = [("auto", rig_block, {}), ("groups", rig_with_groups, {"intrinsics": True}),
              ("survey", rig_survey, {"general": True}), ("fixed", rig_fixed_capture, {}),
              ("poses_held", rig_intrinsics_only, {"intrinsics": True, "poses": False})]


def host_rig(L, problem, options):
    desc, keep = native.problem_desc(problem)
    o = native.solve_options(options, problem)
    out = np.zeros(8, np.int32)
    kb = np.zeros(len(problem.rig.captures), np.int32)
    sb = np.zeros(len(problem.rig.sensors), np.int32)
    pairs = np.zeros((100000, 2), np.int32)
    cams = np.zeros((problem.n_cameras, 32))
    fixed = np.zeros(problem.n_cameras, np.int32)
    groups = np.zeros(problem.n_cameras, np.int32)
    rc = L.probe_rig(C.byref(desc), C.byref(o), out.ctypes.data, kb.ctypes.data, sb.ctypes.data, pairs.ctypes.data,
                     pairs.shape[0], cams.ctypes.data, fixed.ctypes.data, groups.ctypes.data)
    del keep
    return rc, {"ncapb": out[1], "nsenb": out[2], "primary": out[3], "pairs": pairs[:out[4]], "camera_blocks": out[5],
                "fixed": fixed[:out[6]], "ref_param": out[7], "capture_block": kb, "sensor_block": sb,
                "cameras": cams, "groups": groups}


@pytest.mark.parametrize("name,make,kw", HOST_CASES)
def test_host_rig_model_matches_oracle(host_probe, name, make, kw):
    p = make()
    opts = rig_options(**kw)
    rc, h = host_rig(host_probe, p, opts)
    assert rc == 0, host_probe.probe_message().decode()
    orc = O.Oracle(p, opts)
    assert orc.status == 0
    info = orc.info()
    r = orc.rig()
    assert np.array_equal(h["capture_block"], r["capture_block"])
    assert np.array_equal(h["sensor_block"], r["sensor_block"])
    assert h["ncapb"] + h["nsenb"] == info["camera_blocks"]
    assert h["primary"] == info["primary"]
    assert h["ref_param"] == info["ref_param"] == 0
    orc.build(0.0) if not kw.get("general") else orc.general_equations()
    if not kw.get("general"):
        assert np.array_equal(h["pairs"], orc.reduced()["pairs"])
    # the composed input cameras: R_rig R_sensor and C_rig + R_rig c_sensor, the same arithmetic
    a = orc.active()
    assert np.array_equal(a["camera_block"], np.full(p.n_cameras, -1))
    want = np.zeros((p.n_cameras, 12))
    for b in p.rig.cameraBindings:
        Rc = np.array(p.rig.captures[b.captureId].rigToWorldRotation).reshape(3, 3)
        Cc = np.array(p.rig.captures[b.captureId].rigCenterInWorld)
        Rs = np.array(p.rig.sensors[b.sensorId].cameraToRigRotation).reshape(3, 3)
        ts = np.array(p.rig.sensors[b.sensorId].cameraCenterInRig)
        want[b.cameraIndex, :9] = (Rc @ Rs).reshape(9)
        want[b.cameraIndex, 9:12] = Cc + Rc @ ts
    np.testing.assert_allclose(h["cameras"][:, :12], want, rtol=0, atol=1e-12)
    assert info["fixed_cameras"] == h["fixed"].size
    if opts.calibration.refineSharedFocalLength:
        assert np.array_equal(h["groups"] >= 0, np.ones(p.n_cameras, bool))


def test_sensors_share_intrinsic_groups_without_explicit_groups(host_probe):
    """makeSolverOptions (Conversion.cpp:83-98): without explicit calibration groups the cameras of
    one sensor form one group; five sensors exceed the four groups of the dense border and the
    problem is refused as unsupported, with explicit groups it is accepted."""
    p = rig_block()
    rc, _ = host_rig(host_probe, p, rig_options(intrinsics=True))
    assert rc == SolveStatus.UnsupportedConfiguration
    p3 = rig_block(n_obliques=2)
    rc, h = host_rig(host_probe, p3, rig_options(intrinsics=True))
    assert rc == 0
    want = np.array([c % 3 for c in range(p3.n_cameras)])
    assert np.array_equal(h["groups"], want)


@pytest.mark.parametrize("name,make,kw", HOST_CASES)
def test_host_rig_term_lists(host_probe, name, make, kw):
    p = make()
    desc, keep = native.problem_desc(p)
    o = native.solve_options(rig_options(**kw), p)
    assert host_probe.probe_rig_terms(C.byref(desc), C.byref(o)) == 0


def bad(kind):
    p = rig_block(n_along=3, n_lines=2, n_points=500)
    if kind == "no_fixed_sensor":
        p.rig.sensors[0] = dataclasses.replace(p.rig.sensors[0], fixedExtrinsic=False)
    elif kind == "other_rig":
        p.rig.sensors[2] = dataclasses.replace(p.rig.sensors[2], rigId=7)
        p.rig.sensors.append(dataclasses.replace(p.rig.sensors[0], rigId=7, sensorId=99))
    elif kind == "not_rotation":
        R = np.array(p.rig.captures[1].rigToWorldRotation) * 1.01
        p.rig.captures[1] = dataclasses.replace(p.rig.captures[1], rigToWorldRotation=tuple(R))
    elif kind == "unbound":
        p.rig.cameraBindings = p.rig.cameraBindings[:-1]
    return p


@pytest.mark.parametrize("kind", ["no_fixed_sensor", "other_rig", "not_rotation", "unbound"])
def test_invalid_rig_topologies_are_rejected(host_probe, kind):
    p = bad(kind)
    rc, _ = host_rig(host_probe, p, rig_options())
    assert rc == SolveStatus.InvalidInput
    assert O.Oracle(p, rig_options()).status == SolveStatus.InvalidInput


def test_oracle_rig_gradient_matches_central_differences():
    """The chained capture and sensor columns of the oracle's general equations equal central
    differences (h = 1e-6) of its objective under the pose delta R' = Exp(h e_a) R, C' = C + h e_a
    of one capture or sensor (the reference's own Jacobian check pattern, test_linescan.cpp:83-132:
    tolerance 2e-5 relative)."""
    p = rig_block(n_along=4, n_lines=2, n_points=800, outlier_frac=0.0)
    opts = rig_options(general=True)
    o = O.Oracle(p, opts)
    g = o.general_equations()["g"]
    r = o.rig()

    def cost_with(kind, idx, col, h):
        q = copy.deepcopy(p)
        rec = q.rig.captures[idx] if kind == "cap" else q.rig.sensors[idx]
        R = np.array(rec.rigToWorldRotation if kind == "cap" else rec.cameraToRigRotation).reshape(3, 3)
        Cn = np.array(rec.rigCenterInWorld if kind == "cap" else rec.cameraCenterInRig, float)
        if col < 3:
            e = np.zeros(3)
            e[col] = h
            R = synth.rotation_from_axis_angle(e) @ R
        else:
            Cn[col - 3] += h
        if kind == "cap":
            q.rig.captures[idx] = dataclasses.replace(rec, rigToWorldRotation=tuple(R.reshape(9)),
                                                      rigCenterInWorld=tuple(Cn))
        else:
            q.rig.sensors[idx] = dataclasses.replace(rec, cameraToRigRotation=tuple(R.reshape(9)),
                                                     cameraCenterInRig=tuple(Cn))
        return O.Oracle(q, opts).cost()

    h = 1e-6
    for kind, idx in (("cap", 1), ("cap", 4), ("sen", 1), ("sen", 3)):
        blk = r["capture_block"][idx] if kind == "cap" else r["sensor_block"][idx]
        assert blk >= 0
        an = g[13 * blk:13 * blk + 6]
        fd = np.array([(cost_with(kind, idx, c, h) - cost_with(kind, idx, c, -h)) / (2 * h) for c in range(6)])
        assert np.abs(fd - an).max() <= 2e-5 * np.abs(an).max(), (kind, idx, fd, an)


# ---- GPU ------------------------------------------------------------------------------------

GPU_CASES = [("online", rig_block, {}), ("general", rig_block, {"general": True}),
             ("groups", rig_with_groups, {"intrinsics": True}), ("survey", rig_survey, {"general": True}),
             ("fixed", rig_fixed_capture, {}), ("poses_held", rig_intrinsics_only, {"intrinsics": True, "poses": False})]


def gpu(problem, options):
    from plabundle_gb300.device import Gb300Context
    ctx = Gb300Context(0)
    st = ctx.upload(problem, options)
    assert st == 0, ctx.L.pb_gpu_last_error(ctx.ctx)
    return ctx


def scene_scale(cams):
    C = cams[:, 9:12]
    return np.linalg.norm(C - C.mean(0), axis=1).max()


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,kw", GPU_CASES)
def test_rig_blocks_and_pairs_match_oracle(name, make, kw):
    p = make()
    opts = rig_options(**kw)
    ctx = gpu(p, opts)
    orc = O.Oracle(p, opts)
    r, o = ctx.rig(), orc.rig()
    assert np.array_equal(r["capture_block"], o["capture_block"])
    assert np.array_equal(r["sensor_block"], o["sensor_block"])
    a, b = ctx.active(), orc.active()
    for k in ("active_track", "camera_block", "intrinsic_block", "track_block"):
        assert np.array_equal(a[k], b[k]), k
    if not kw.get("general"):
        orc.build(0.0)
        assert np.array_equal(ctx.pairs(), orc.reduced()["pairs"])


@pytest.mark.gpu
@pytest.mark.parametrize("damping", [0.0, 1e-3])
def test_rig_reduced_system_matches_oracle(damping):
    """The camera-block system mapped onto the rig blocks equals the oracle's reduced system
    assembled with the chained Jacobians (FP64 path, 1e-9 of the diagonal scaling)."""
    p = rig_with_groups()
    opts = rig_options(intrinsics=True)
    ctx = gpu(p, opts)
    orc = O.Oracle(p, opts)
    cg, sg = ctx.linearize_schur(damping, Precision.Fp64)
    co, so = orc.build(damping)
    assert sg == so
    np.testing.assert_allclose(cg, co, rtol=1e-12)
    S, rhs, _ = ctx.reduced()
    So, red = orc.dense_reduced()
    # the solve of that system: the rig step satisfies S x = rhs (FP64 path, CG to 2e-10)
    step, cv, _, rr = ctx.solve_reduced()
    assert cv and step.size == S.shape[0]
    assert np.linalg.norm(S @ step - rhs) <= 1e-8 * np.linalg.norm(rhs)
    s = ctx.sizes()
    nrb, ng, ni = s["camera_blocks"], s["intrinsic_blocks"], s["ni"]
    cols = [q for q in range(9) if (int(ctx.copts.intrinsic_mask) >> q) & 1]
    m = np.array([13 * i + a for i in range(nrb) for a in range(6)] +
                 [13 * (nrb + g) + cols[c] for g in range(ng) for c in range(ni)])
    Sm = So[np.ix_(m, m)]
    d = np.sqrt(np.abs(np.diag(Sm)))
    assert np.abs((S - Sm) / np.outer(d, d)).max() < 1e-9
    assert np.abs((rhs + red["gradient"][m]) / d).max() < 1e-9 * max(1.0, np.abs(red["gradient"][m] / d).max())


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,kw", GPU_CASES)
def test_rig_fp64_follows_the_oracle(name, make, kw):
    """FP64 path: the oracle's LM trajectory iteration for iteration (20-iteration budget), the
    refined captures, sensors and composed cameras."""
    p = make()
    opts = rig_options(**kw)
    ref = O.Oracle(p, opts).solve()
    ctx = gpu(p, opts)
    rep = ctx.solve()
    out = ctx.download()
    rig = ctx.rig()
    rr = ref["report"]
    assert rep["status"] == rr["status"]
    assert rep["iterations"] == rr["iterations"]
    assert rep["accepted_steps"] == rr["accepted_steps"]
    assert rep["camera_blocks"] == rep["rig_capture_blocks"] + rep["rig_sensor_blocks"]
    np.testing.assert_allclose(rep["initial_cost"], rr["initial_cost"], rtol=1e-12)
    assert abs(rep["final_cost"] - rr["final_cost"]) / rr["final_cost"] < 1e-9
    scale = scene_scale(ref["cameras"])
    assert np.abs(out["cameras"][:, 9:12] - ref["cameras"][:, 9:12]).max() / scale < 1e-8
    assert np.abs(out["cameras"][:, :9] - ref["cameras"][:, :9]).max() < 1e-8
    assert np.abs(rig["captures"][:, 9:12] - ref["captures"][:, 9:12]).max() / scale < 1e-8
    assert np.abs(rig["sensors"] - ref["sensors"]).max() < 1e-7
    assert np.array_equal(out["valid"], ref["valid"])
    if ref["intrinsics"].size:
        np.testing.assert_allclose(out["intrinsics"], ref["intrinsics"], rtol=1e-6, atol=1e-7)


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,kw", [c for c in GPU_CASES if c[0] in ("online", "survey")])
def test_rig_mixed_reaches_the_oracle_fixed_point(name, make, kw):
    """Mixed path: both solves to convergence; 1e-6 relative final cost, 1e-5 relative camera
    centres and capture centres, identical inliers."""
    p = make()
    o_ref, o_mix = rig_options(iterations=150, **kw), rig_options(mixed=True, iterations=150, **kw)
    ref = O.Oracle(p, o_ref).solve()
    ctx = gpu(p, o_mix)
    rep = ctx.solve()
    out = ctx.download()
    rig = ctx.rig()
    rr = ref["report"]
    assert rr["status"] == SolveStatus.Success
    assert rep["status"] == SolveStatus.Success
    assert abs(rep["final_cost"] - rr["final_cost"]) / rr["final_cost"] < 1e-6
    scale = scene_scale(ref["cameras"])
    assert np.abs(out["cameras"][:, 9:12] - ref["cameras"][:, 9:12]).max() / scale < 1e-5
    assert np.abs(rig["captures"][:, 9:12] - ref["captures"][:, 9:12]).max() / scale < 1e-5
    assert np.array_equal(out["valid"], ref["valid"])


@pytest.mark.gpu
def test_public_solve_publishes_the_refined_rig():
    """Solver.solve: Result.refinedRig carries the accepted captures and sensors, and
    refinedCameras their composition."""
    from plabundle_gb300.solver import Solver
    p = rig_block()
    res = Solver().solve(p, rig_options())
    assert res.status in (SolveStatus.Success, SolveStatus.NoConvergence)
    rig = res.refinedRig
    assert rig is not None and len(rig.captures) == len(p.rig.captures)
    for b in rig.cameraBindings:
        Rc = np.array(rig.captures[b.captureId].rigToWorldRotation).reshape(3, 3)
        Cc = np.array(rig.captures[b.captureId].rigCenterInWorld)
        Rs = np.array(rig.sensors[b.sensorId].cameraToRigRotation).reshape(3, 3)
        ts = np.array(rig.sensors[b.sensorId].cameraCenterInRig)
        cam = res.refinedCameras[b.cameraIndex]
        np.testing.assert_allclose(cam[:9], (Rc @ Rs).reshape(9), atol=1e-12)
        np.testing.assert_allclose(cam[9:12], Cc + Rc @ ts, atol=1e-9)
    assert np.array_equal(np.array(rig.sensors[0].cameraToRigRotation), np.array(p.rig.sensors[0].cameraToRigRotation))
