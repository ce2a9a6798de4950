"""GPU parity of the sm_103a kernels against the CPU FP64 oracle, through the C ABI.

Integer work (active tracks, block numbering, reduced pattern, inlier masks) must match bit for
bit.  Floating point tolerances are written in each test: FP64 path to FP64 rounding of a
different summation order; mixed path (FP32 Jacobians/Schur/PCG with compensated sums and FP64
cost / refinement) to the benchmark spec's targets, 1e-6 relative final cost and 1e-5 relative camera
centre error.
"""
import numpy as np
import pytest

import oracle as O
from plabundle_gb300 import synth
from plabundle_gb300.device import Gb300Context
from plabundle_gb300.problem import ImageRobustLoss, Precision, SolveOptions, SolveStatus

pytestmark = pytest.mark.gpu


def ring(seed=5, n_cameras=8, n_points=300, **kw):
    return synth.ring_problem(seed=seed, n_cameras=n_cameras, n_points=n_points, **kw)


def ring_options(mixed=False):
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Huber
    o.solver.imageRobustLossScalePixels = 1.5
    o.backend.enablePlaMatrixMixedPrecision = mixed
    return o


def aerial(n_along=5, n_lines=4, n_points=3000, seed=3):
    return synth.aerial_grid_problem(seed=seed, n_along=n_along, n_lines=n_lines, n_points=n_points)


def aerial_options(mixed=False):
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Cauchy
    o.solver.imageRobustLossScalePixels = 1.5
    o.calibration.refineSharedFocalLength = True
    o.calibration.refineSharedPrincipalPoint = True
    o.calibration.refineSharedRadialDistortion = True
    o.backend.enablePlaMatrixMixedPrecision = mixed
    return o


def gpu(problem, options):
    ctx = Gb300Context(0)
    st = ctx.upload(problem, options)
    assert st == 0, ctx.L.pb_gpu_last_error(ctx.ctx)
    return ctx


def index_map(ctx, orc):
    """GPU compact reduced index -> oracle 13-padded index."""
    s = ctx.sizes()
    ncb, ng, ni = s["camera_blocks"], s["intrinsic_blocks"], s["ni"]
    cols = [p for p in range(9) if (int(ctx.copts.intrinsic_mask) >> p) & 1]
    assert len(cols) == ni
    idx = [13 * i + a for i in range(ncb) for a in range(6)]
    idx += [13 * (ncb + g) + cols[c] for g in range(ng) for c in range(ni)]
    return np.array(idx)


def ring_gcp():
    """The ring with ten survey targets (sigma 2 cm, the three uncertainty forms): complete
    control-point gauge, plain parameterisation, Huber control-point terms in both branches."""
    return synth.with_control_points(ring(), n=10, seed=2)


def aerial_gcp():
    """The aerial block with 16 ground control points and shared intrinsics refined."""
    return synth.with_control_points(aerial(), n=16, seed=4)


CASES = [("ring", ring, ring_options), ("aerial", aerial, aerial_options), ("ring_gcp", ring_gcp, ring_options),
         ("aerial_gcp", aerial_gcp, aerial_options)]


@pytest.mark.parametrize("name,make,opts", CASES)
def test_active_problem_pattern_and_gauge_are_identical(name, make, opts):
    p = make()
    ctx = gpu(p, opts())
    orc = O.Oracle(p, opts())
    a, b = ctx.active(), orc.active()
    for k in ("active_track", "camera_block", "intrinsic_block", "track_block"):
        assert np.array_equal(a[k], b[k]), k
    orc.build(0.0)
    assert np.array_equal(ctx.pairs(), orc.reduced()["pairs"])
    s, i = ctx.sizes(), orc.info()
    assert (s["gauge_anchor"], s["gauge_scale"]) == (i["gauge_anchor"], i["gauge_scale"])
    assert s["gauge_baseline"] == i["gauge_baseline"]
    assert s["active_tracks"] == i["active_tracks"] and s["observation_count"] == i["observation_count"]
    assert s["rejected_initial_tracks"] == i["rejected_initial_tracks"]


@pytest.mark.parametrize("name,make,opts", CASES)
@pytest.mark.parametrize("precision", [Precision.Fp64, Precision.Mixed])
def test_observation_linearization_matches_oracle(name, make, opts, precision):
    p = make()
    ctx = gpu(p, opts())
    g = ctx.linearize_observations(precision)
    r = O.Oracle(p, opts()).linearize_observations()
    act = ctx.active()["active_track"]
    trk = np.repeat(np.arange(p.n_tracks), np.diff(p.track_offsets))
    sel = (act[trk] == 1) & (r["valid"] == 1)
    assert np.array_equal(g["valid"][sel], r["valid"][sel])
    tol = 1e-10 if precision == Precision.Fp64 else 2e-6
    rtol_r = 1e-12 if precision == Precision.Fp64 else 1e-6
    np.testing.assert_allclose(g["residual"][sel], r["residual"][sel], rtol=rtol_r, atol=1e-9)
    np.testing.assert_allclose(g["cost"][sel], r["cost"][sel], rtol=1e-12, atol=1e-12)
    for key in ("point_jacobian", "pose_jacobian", "intrinsic_jacobian"):
        scale = np.abs(r[key][sel]).max(axis=(1, 2), keepdims=True) + 1e-300
        err = np.abs(g[key][sel] - r[key][sel]) / scale
        assert err.max() < tol, (key, err.max())
    np.testing.assert_allclose(g["normal_weight"][sel], r["normal_weight"][sel], rtol=tol)


def normalized_error(Sg, So):
    d = np.sqrt(np.abs(np.diag(So)))
    d[d == 0] = 1.0
    return np.abs((Sg - So) / np.outer(d, d)).max()


@pytest.mark.parametrize("name,make,opts", CASES)
@pytest.mark.parametrize("precision", [Precision.Fp64, Precision.Mixed])
@pytest.mark.parametrize("damping", [0.0, 1e-3])
def test_reduced_system_matches_oracle(name, make, opts, precision, damping):
    p = make()
    ctx = gpu(p, opts())
    orc = O.Oracle(p, opts())
    cg, sg = ctx.linearize_schur(damping, precision)
    co, so = orc.build(damping)
    assert sg == so
    np.testing.assert_allclose(cg, co, rtol=1e-12)
    S, rhs, direct = ctx.reduced()
    So, red = orc.dense_reduced()
    m = index_map(ctx, orc)
    tol = 1e-9 if precision == Precision.Fp64 else 2e-4
    assert normalized_error(S, So[np.ix_(m, m)]) < tol
    d = np.sqrt(np.abs(np.diag(So[np.ix_(m, m)])))
    assert np.abs((rhs + red["gradient"][m]) / d).max() < tol * max(1.0, np.abs(red["gradient"][m] / d).max())
    assert np.abs((direct - red["direct_rhs"][m]) / d).max() < tol * max(1.0, np.abs(red["direct_rhs"][m] / d).max())


@pytest.mark.parametrize("name,make,opts", CASES)
@pytest.mark.parametrize("precision", [Precision.Fp64, Precision.Mixed])
def test_reduced_solve_and_back_substitution_match_oracle(name, make, opts, precision):
    """Camera step, point steps and the predicted decrease of one LM step against the oracle's
    dense FP64 solve.  FP64 path: 1e-7 relative.  Mixed path: the FP32 rounding of the Jacobians
    perturbs the matrix by ~1e-7 relative, which a condition number of ~1e7 amplifies in the
    weakest modes; the step is therefore checked in the matrix's own energy norm (1e-4), the
    predicted decrease to 1e-6 and the point steps to 2e-2."""
    p = make()
    ctx = gpu(p, opts())
    orc = O.Oracle(p, opts(), linear_solver=1)
    ctx.linearize_schur(0.0, precision)
    orc.build(0.0)
    step, cv, it, rr = ctx.solve_reduced()
    assert cv and rr <= 2e-10
    ostep, ocv, _ = orc.solve_linear()
    m = index_map(ctx, orc)
    So, _ = orc.dense_reduced()
    So = So[np.ix_(m, m)]
    ost = ostep[m]
    elim, dd, ok = ctx.back_substitute()
    oelim, odd, ook = orc.back_substitute(ostep)
    assert ok and ook
    if precision == Precision.Fp64:
        rel = np.linalg.norm(step - ost) / np.linalg.norm(ost)
        assert rel < 1e-7, rel
        assert np.linalg.norm(elim - oelim) / np.linalg.norm(oelim) < 1e-7
        assert abs(dd - odd) / abs(odd) < 1e-7
    else:
        d = step - ost
        energy = np.sqrt(abs(d @ So @ d) / abs(ost @ So @ ost))
        assert energy < 1e-4, energy
        assert abs(dd - odd) / abs(odd) < 1e-6, (dd, odd)
        assert np.linalg.norm(elim - oelim) / np.linalg.norm(oelim) < 2e-2


@pytest.mark.parametrize("name,make,opts", CASES)
def test_full_solve_matches_oracle(name, make, opts):
    """FP64 path: the LM trajectory of the oracle, iteration for iteration (20-iteration budget)."""
    p = make()
    ref = O.Oracle(p, opts()).solve()
    ctx = gpu(p, opts(False))
    rep = ctx.solve()
    out = ctx.download()
    rr = ref["report"]
    assert rep["status"] == rr["status"]
    assert rr["status"] in (SolveStatus.Success, SolveStatus.NoConvergence)
    rel_cost = abs(rep["final_cost"] - rr["final_cost"]) / rr["final_cost"]
    assert rel_cost < 1e-9, rel_cost
    np.testing.assert_allclose(rep["initial_cost"], rr["initial_cost"], rtol=1e-12)
    C_ref = ref["cameras"][:, 9:12]
    scale = np.linalg.norm(C_ref - C_ref.mean(0), axis=1).max()
    cerr = np.abs(out["cameras"][:, 9:12] - C_ref).max() / scale
    assert cerr < 1e-8, cerr
    assert np.array_equal(out["valid"], ref["valid"])
    assert rep["iterations"] == rr["iterations"]
    assert rep["accepted_steps"] == rr["accepted_steps"]
    # the solves stop once the step RMS is below 1e-6; the final states agree to that level
    np.testing.assert_allclose(out["rms_after"][ref["valid"]], ref["rms_after"][ref["valid"]], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(out["rms_before"], ref["rms_before"], rtol=1e-12)
    if ref["intrinsics"].size:
        np.testing.assert_allclose(out["intrinsics"], ref["intrinsics"], rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("name,make,opts", CASES)
def test_mixed_solve_converges_to_the_oracle_fixed_point(name, make, opts):
    """Mixed path (FP32 Jacobians, float-float Schur assembly, FP32-factor preconditioned CG on
    the FP64 system, FP64 cost and gain ratio): both solves run to convergence (step RMS below
    1e-6) and must agree to the targets: 1e-6 relative final cost, 1e-5 relative camera-centre
    error (relative to the scene extent), intrinsics to 2e-5 relative, identical inlier sets."""
    p = make()
    o_ref, o_mix = opts(False), opts(True)
    o_ref.solver.maxIterations = o_mix.solver.maxIterations = 80
    ref = O.Oracle(p, o_ref).solve()
    ctx = gpu(p, o_mix)
    rep = ctx.solve()
    out = ctx.download()
    rr = ref["report"]
    assert rr["status"] == SolveStatus.Success
    assert rep["status"] == SolveStatus.Success
    rel_cost = abs(rep["final_cost"] - rr["final_cost"]) / rr["final_cost"]
    assert rel_cost < 1e-6, rel_cost
    np.testing.assert_allclose(rep["initial_cost"], rr["initial_cost"], rtol=1e-12)
    C_ref = ref["cameras"][:, 9:12]
    scale = np.linalg.norm(C_ref - C_ref.mean(0), axis=1).max()
    cerr = np.abs(out["cameras"][:, 9:12] - C_ref).max() / scale
    assert cerr < 1e-5, cerr
    assert np.array_equal(out["valid"], ref["valid"])
    np.testing.assert_allclose(out["rms_before"], ref["rms_before"], rtol=1e-12)
    if ref["intrinsics"].size:
        np.testing.assert_allclose(out["intrinsics"], ref["intrinsics"], rtol=2e-5, atol=1e-7)


@pytest.mark.parametrize("mixed", [False, True])
def test_block_jacobi_pcg_solve_matches_oracle(mixed):
    """The block-Jacobi PCG path (used above 16384 reduced unknowns), forced on the ring: the LM
    solve with the PCG to the reference's 2e-10 relative residual reaches the oracle's solution."""
    p = ring()
    o = ring_options(mixed)
    o.solver.maxIterations = 40
    o.backend.linearSolver = 2
    o_ref = ring_options(False)
    o_ref.solver.maxIterations = 40
    ref = O.Oracle(p, o_ref).solve()
    ctx = gpu(p, o)
    rep = ctx.solve()
    out = ctx.download()
    rr = ref["report"]
    assert rep["status"] == rr["status"] == SolveStatus.Success
    assert abs(rep["final_cost"] - rr["final_cost"]) / rr["final_cost"] < 1e-8
    C_ref = ref["cameras"][:, 9:12]
    scale = np.linalg.norm(C_ref - C_ref.mean(0), axis=1).max()
    assert np.abs(out["cameras"][:, 9:12] - C_ref).max() / scale < 1e-6
    assert np.array_equal(out["valid"], ref["valid"])


@pytest.mark.parametrize("name,make,opts", CASES)
def test_parity_report_of_the_public_solve(name, make, opts):
    """Solver.solve on the GPU (FP64) against the oracle, through the reference's outcome
    comparison (plabundle_gb300/parity.py): id-keyed camera and track differences, identical
    valid masks, matching termination status."""
    from plabundle_gb300.parity import PhotoAlignmentComparisonTolerance, compare_outcomes, make_outcome
    from plabundle_gb300.problem import QualitySummary, RefinedPoint, Result
    from plabundle_gb300.solver import Solver
    p = make()
    o = opts(False)
    got = Solver().solve(p, o)
    ref = O.Oracle(p, opts()).solve()
    rr = ref["report"]
    oracle_result = Result(status=SolveStatus(rr["status"]), solutionUsable=bool(rr["solution_usable"]),
                           quality=QualitySummary(meanRmsBefore=rr["mean_rms_before"], meanRmsAfter=rr["mean_rms_after"]),
                           points=RefinedPoint(valid=ref["valid"], converged=True, point=ref["points"],
                                               rmsBefore=ref["rms_before"], rmsAfter=ref["rms_after"], iterations=0),
                           refinedCameras=ref["cameras"], backendMessage=got.backendMessage)
    # the rotation angle is acos((trace - 1) / 2) as in the reference: for equal rotations the
    # rounding of the trace alone gives ~sqrt(2 eps) rad, about 1e-6 degrees
    tol = PhotoAlignmentComparisonTolerance(rms=1e-6, cameraCenterMeters=1e-6, cameraRotationDegrees=1e-5,
                                            pointMeters=1e-4)
    c = compare_outcomes(make_outcome(oracle_result), make_outcome(got), tol)
    assert c.comparable
    assert c.validTrackMaskMismatchIds == []
    assert c.terminationStatusMatches
    assert c.equivalent, (c.maximumCameraCenterDifferenceMeters, c.maximumCameraRotationDifferenceDegrees,
                          c.maximumPointDifferenceMeters, c.rmsAfterDifference)
    if p.controlPoints:
        # control-point statistics of the result (BundleAdjustQuality.cpp:179-211, :282-289)
        q = got.quality
        assert q.controlPointConstraintCount == sum(1 for t, _ in p.controlPoints if ref["valid"][t])
        assert q.controlPointRmsAfterMeters < q.controlPointRmsBeforeMeters
        assert not got.qualityGateRejected


def test_backward_pass_rejects_control_point_problems():
    """The exact-Hessian adjoint is written for the charts of image-only problems; a problem with
    control points (plain parameterisation) is refused with an unsupported status."""
    p = ring_gcp()
    ctx = gpu(p, ring_options())
    ctx.solve()
    g = np.zeros((p.n_cameras, 6))
    with pytest.raises(RuntimeError, match="image-only"):
        ctx.backward(grad_cameras=g)


@pytest.mark.parametrize("name,make,opts", CASES)
def test_mixed_weight_and_gradient_chain_match_fp64(name, make, opts):
    """The mixed path evaluates the robust weight and the gradient chain -J^T w r in float-float
    from the FP64 projection and residual.  Against the FP64 path at the same state: normal
    weights within 1e-10 relative (measured ~1e-10 at the 500-camera block), the direct gradient
    (before point elimination, the image terms only) within 1e-10 of its largest entry (measured
    3e-12); the residual is the FP64 one."""
    p = make()
    ctx = gpu(p, opts())
    a = ctx.linearize_observations(Precision.Fp64)
    b = ctx.linearize_observations(Precision.Mixed)
    sel = (a["valid"] == 1) & (b["valid"] == 1)
    assert np.array_equal(a["valid"], b["valid"])
    # the FP64 residual, to a few ulps of the pixel coordinate (the compiler contracts the
    # projection into FMAs differently at different call sites) and the 48 bits of its
    # float-float copy
    np.testing.assert_allclose(b["residual"][sel], a["residual"][sel], rtol=1e-13, atol=2e-12)
    wrel = np.abs(b["normal_weight"][sel] - a["normal_weight"][sel]) / a["normal_weight"][sel]
    assert wrel.max() < 1e-10, wrel.max()
    ctx.linearize_schur(0.0, Precision.Fp64)
    _, _, d64 = ctx.reduced()
    ctx.linearize_schur(0.0, Precision.Mixed)
    _, _, d32 = ctx.reduced()
    err = np.abs(d32 - d64).max() / np.abs(d64).max()
    assert err < 1e-10, err
