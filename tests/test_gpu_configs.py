"""GPU parity at the two workloads the time-to-converge metric is quoted on, against the CPU FP64
oracle, through the C ABI.

* The 20-camera ring exactly as specified (`synth.ring_problem()` defaults: 20 cameras on a
  circle, 2 000 points, 9 019 observations, Huber 1.5 px, AutoAnchor, a 20-iteration budget), in
  both precisions and with the FP64 path's factor kept across LM iterations.
* The 500-camera / 200 k-point aerial grid (two calibration groups, Cauchy 1.5 px, run to
  convergence), against the committed fixture of the oracle's converged solve
  (tests/golden/make_c1_fixture.py).  The problem is regenerated from its seed; the test skips
  when the generator does not reproduce the fixture's problem (integer arrays bit for bit,
  sampled floating-point entries to 1e-10).  The oracle's solves there are direct and accepted
  without a post-solve gate, the semantics of the GPU paths' CG (see the fixture script).

Tolerances: the FP64 path reproduces the oracle's LM trajectory (same iterations and accepted
steps, final cost to 1e-9 relative); the mixed path and the FP64 path with a kept factor reach
the oracle's fixed point to 1e-6 relative final cost and 1e-5 camera-centre error relative to
the scene extent, with identical inlier sets.
"""
import numpy as np
import pytest

import oracle as O
from plabundle_gb300 import synth
from plabundle_gb300.device import Gb300Context
from plabundle_gb300.problem import ImageRobustLoss, SolveOptions, SolveStatus

pytestmark = pytest.mark.gpu


def ring_c0_options(mixed=False, factor_reuse=0):
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Huber
    o.solver.imageRobustLossScalePixels = 1.5
    assert o.solver.maxIterations == 20
    o.backend.enablePlaMatrixMixedPrecision = mixed
    o.backend.factorReuse = factor_reuse
    return o


def solve_gpu(problem, options):
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


@pytest.fixture(scope="module")
def ring_c0():
    p = synth.ring_problem()
    assert (p.n_cameras, p.n_tracks) == (20, 2000)
    ref = O.Oracle(p, ring_c0_options()).solve()
    assert ref["report"]["status"] == SolveStatus.Success
    return p, ref


def test_ring_c0_fp64_path_follows_the_oracle_trajectory(ring_c0):
    p, ref = ring_c0
    rep, out = solve_gpu(p, ring_c0_options(False))
    rr = ref["report"]
    assert rep["status"] == rr["status"]
    assert rep["iterations"] == rr["iterations"] and rep["accepted_steps"] == rr["accepted_steps"]
    assert abs(rep["final_cost"] - rr["final_cost"]) / rr["final_cost"] < 1e-9
    np.testing.assert_allclose(rep["initial_cost"], rr["initial_cost"], rtol=1e-12)
    assert centre_error(out, ref) < 1e-8
    assert np.array_equal(out["valid"], ref["valid"])
    np.testing.assert_allclose(out["rms_before"], ref["rms_before"], rtol=1e-12)
    np.testing.assert_allclose(out["rms_after"][ref["valid"]], ref["rms_after"][ref["valid"]], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("mixed,factor_reuse", [(True, 0), (False, 1)])
def test_ring_c0_converges_to_the_oracle_fixed_point(ring_c0, mixed, factor_reuse):
    p, ref = ring_c0
    rep, out = solve_gpu(p, ring_c0_options(mixed, factor_reuse))
    rr = ref["report"]
    assert rep["status"] == SolveStatus.Success
    assert abs(rep["final_cost"] - rr["final_cost"]) / rr["final_cost"] < 1e-6
    np.testing.assert_allclose(rep["initial_cost"], rr["initial_cost"], rtol=1e-12)
    assert centre_error(out, ref) < 1e-5
    assert np.array_equal(out["valid"], ref["valid"])
    np.testing.assert_allclose(out["rms_before"], ref["rms_before"], rtol=1e-12)


@pytest.fixture(scope="module")
def aerial_c1():
    from golden import make_c1_fixture as FX
    fx = FX.load_fixture()
    if fx is None:
        pytest.skip("the 500-camera oracle fixture is absent")
    prob, opts = FX.c1_workload()
    why = FX.problem_mismatch(fx[0], fx[1], prob)
    if why:
        pytest.skip("the generator does not reproduce the fixture's problem on this machine: " + why)
    return FX, fx, prob, opts


@pytest.mark.parametrize("mixed", [True, False])
def test_aerial_c1_reaches_the_oracle_solution(aerial_c1, mixed):
    """Mixed path, and the FP64 path with a kept factor: the 500-camera solve run to
    convergence against the oracle's converged solve of the same problem."""
    FX, (meta, arrays), prob, opts = aerial_c1
    opts.backend.enablePlaMatrixMixedPrecision = mixed
    opts.backend.factorReuse = 0 if mixed else 1
    rep, out = solve_gpu(prob, opts)
    assert rep["status"] == SolveStatus.Success
    cmp = FX.compare(meta, arrays, out["cameras"], out["intrinsics"], out["valid"], out["rms_after"], out["points"],
                     rep["final_cost"], rep["filter_threshold"])
    assert cmp["final_cost_rel_err"] < 1e-6, cmp
    assert cmp["camera_centre_rel_err"] < 1e-5, cmp
    assert cmp["intrinsics_rel_err"] < 2e-5, cmp
    assert cmp["point_sample_rel_err"] < 1e-5, cmp
    # identical inliers, except a track whose after-RMS sits within 1e-6 px of the threshold
    assert all(abs(m) < 1e-6 for m in cmp["flip_margins_px"]) and cmp["inlier_mask_flips"] <= 2, cmp
    np.testing.assert_allclose(rep["initial_cost"], meta["report"]["initial_cost"], rtol=1e-12)


@pytest.mark.gpu
def test_cost_history_of_a_solve():
    """pb_gpu_get_history: the initial cost, then one entry per accepted step, costs decreasing,
    the last entry the final cost, host times increasing."""
    from plabundle_gb300.device import Gb300Context
    p = synth.ring_problem(seed=7)
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Huber
    o.solver.imageRobustLossScalePixels = 1.5
    ctx = Gb300Context(0)
    assert ctx.upload(p, o) == 0
    rep = ctx.solve()
    h = ctx.history()
    assert h["cost"].size == rep["accepted_steps"] + 1
    assert h["iterations"][0] == 0 and h["cost"][0] == rep["initial_cost"]
    assert h["cost"][-1] == rep["final_cost"]
    assert np.all(np.diff(h["cost"]) < 0) and np.all(np.diff(h["ms"]) >= 0)
    assert np.all(np.diff(h["iterations"]) > 0)


@pytest.fixture(scope="module")
def rig_block():
    from golden import make_rig_fixture as FX
    fx = FX.load_fixture()
    if fx is None:
        pytest.skip("the rig-block oracle fixture is absent")
    prob, opts = FX.rig_workload()
    why = FX.problem_mismatch(fx[0], fx[1], prob)
    if why:
        pytest.skip("the generator does not reproduce the fixture's problem on this machine: " + why)
    return FX, fx, prob, opts


def test_rig_block_reaches_the_oracle_solution(rig_block):
    """The large oblique survey configuration (600 five-camera rig captures, 1.5 M points, 40
    control points, 10 scale bars; general path), mixed path run to convergence, against the
    oracle's converged CPU FP64 solve of the same problem: 1e-6 relative final cost, 1e-5 relative
    camera and capture centres and sampled points, sensor parameters to 1e-6, identical inliers."""
    FX, (meta, arrays), prob, opts = rig_block
    opts.backend.enablePlaMatrixMixedPrecision = True
    ctx = Gb300Context(0)
    assert ctx.upload(prob, opts) == 0, ctx.L.pb_gpu_last_error(ctx.ctx)
    rep = ctx.solve()
    out = ctx.download()
    rig = ctx.rig()
    ctx.close()
    assert rep["status"] == SolveStatus.Success
    cmp = FX.compare(meta, arrays, out["cameras"], rig["captures"], rig["sensors"], out["valid"], out["rms_after"],
                     out["points"], rep["final_cost"], rep["filter_threshold"])
    assert cmp["final_cost_rel_err"] < 1e-6, cmp
    assert cmp["camera_centre_rel_err"] < 1e-5, cmp
    assert cmp["capture_centre_rel_err"] < 1e-5, cmp
    assert cmp["point_sample_rel_err"] < 1e-5, cmp
    assert cmp["sensor_max_abs_err"] < 1e-6, cmp
    assert all(abs(m) < 1e-6 for m in cmp["flip_margins_px"]) and cmp["inlier_mask_flips"] <= 2, cmp
    np.testing.assert_allclose(rep["initial_cost"], meta["report"]["initial_cost"], rtol=1e-12)
