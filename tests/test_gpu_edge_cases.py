"""Edge cases of the input on the GPU path against the oracle (FP64, the full LM solve through the
C ABI): unusable observations (non-finite pixels, camera indices out of range, zero, negative or
infinite weights, non-positive measurement scales), fixed tracks and cameras under an explicit
gauge, the least-squares and Cauchy losses, the initial-RMS track gate, ragged tracks (empty and
single-observation tracks), and a problem with no usable observation.  The FP64 path follows the oracle's LM trajectory iteration for iteration; the
mixed path reaches the oracle's fixed point."""
import numpy as np
import pytest

import oracle as O
from edge_problems import CASES, no_usable_observation, options
from plabundle_gb300.device import Gb300Context
from plabundle_gb300.problem import SolveStatus

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,make,opts", CASES, ids=[c[0] for c in CASES])
def test_edge_case_solve_matches_oracle(name, make, opts):
    p, o = make(), opts()
    ref = O.Oracle(p, o).solve()
    ctx = Gb300Context(0)
    assert ctx.upload(p, o) == 0, ctx.L.pb_gpu_last_error(ctx.ctx)
    a, b = ctx.active(), O.Oracle(p, o).active()
    for key in ("active_track", "camera_block", "track_block"):
        assert np.array_equal(a[key], b[key]), key
    rep = ctx.solve()
    out = ctx.download()
    rr = ref["report"]
    assert rep["status"] == rr["status"]
    assert rep["iterations"] == rr["iterations"]
    assert rep["accepted_steps"] == rr["accepted_steps"]
    assert abs(rep["final_cost"] - rr["final_cost"]) <= 1e-9 * rr["final_cost"]
    np.testing.assert_allclose(rep["initial_cost"], rr["initial_cost"], rtol=1e-12)
    assert np.array_equal(out["valid"], ref["valid"])
    np.testing.assert_allclose(out["rms_before"], ref["rms_before"], rtol=1e-12)
    C_ref = ref["cameras"][:, 9:12]
    scale = np.linalg.norm(C_ref - C_ref.mean(0), axis=1).max()
    assert np.abs(out["cameras"][:, 9:12] - C_ref).max() / scale < 1e-8


def test_no_usable_observation_is_invalid_input():
    p = no_usable_observation()
    ctx = Gb300Context(0)
    assert ctx.upload(p, options()) == 0, ctx.L.pb_gpu_last_error(ctx.ctx)
    assert ctx.sizes()["observation_count"] == 0
    assert ctx.solve()["status"] == SolveStatus.InvalidInput


# every case whose FP64 solve converges within 80 iterations (the fixed-track case does not: its
# fixed points keep the noise of their initial triangulation)
MIXED = [c for c in CASES if c[0] != "fixed_tracks_and_cameras"]


@pytest.mark.parametrize("name,make,opts", MIXED, ids=[c[0] for c in MIXED])
def test_mixed_edge_case_solve_reaches_the_oracle_fixed_point(name, make, opts):
    """Mixed path (float-float weights and gradient, FP32 Jacobians, FP64 residual and cost) on the
    same inputs: 1e-6 relative final cost, 1e-5 relative camera-centre error, identical inliers."""
    p = make()
    o_ref, o_mix = opts(), opts()
    o_mix.backend.enablePlaMatrixMixedPrecision = True
    o_ref.solver.maxIterations = o_mix.solver.maxIterations = 80
    ref = O.Oracle(p, o_ref).solve()
    assert ref["report"]["status"] == SolveStatus.Success
    ctx = Gb300Context(0)
    assert ctx.upload(p, o_mix) == 0, ctx.L.pb_gpu_last_error(ctx.ctx)
    rep = ctx.solve()
    out = ctx.download()
    assert rep["status"] == SolveStatus.Success
    rr = ref["report"]
    assert abs(rep["final_cost"] - rr["final_cost"]) <= 1e-6 * rr["final_cost"]
    C_ref = ref["cameras"][:, 9:12]
    scale = np.linalg.norm(C_ref - C_ref.mean(0), axis=1).max()
    assert np.abs(out["cameras"][:, 9:12] - C_ref).max() / scale < 1e-5
    assert np.array_equal(out["valid"], ref["valid"])
