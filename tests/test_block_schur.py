"""The internal block-Schur interface of the general path (BlockNormalEquations +
solveDampedSchurComplement, src/internal/BundleAdjustPlaMatrix.cpp:311-357) and the general LM path,
against the oracle's restatement.

CPU: the host container (pb_bne_*) filled from the oracle's per-observation linearisation, the way
the reference's addObservation fills it (BundleAdjustPlaMatrixAssembly.cpp:381-440), must equal the
oracle's own buildNormalEquations (to FP64 summation order); merges, shards, transposed Hessian
blocks and finalizePrimaryDiagonal follow their stated semantics.
GPU: the device damped Schur solve of that container matches the oracle's dense FP64 solve, and the
general LM path (useReferenceOnlineSchur = false) follows the oracle's general path on the 20-camera
ring (20 cameras, 2 000 points, Huber 1.5 px) and a 20-camera aerial block with shared intrinsics.
"""
import numpy as np
import pytest

import oracle as O
from plabundle_gb300 import synth
from plabundle_gb300.problem import ImageRobustLoss, SolveOptions, SolveStatus
from plabundle_gb300.schur import (BlockNormalEquations, SchurComplementSolverOptions, SchurSolveError,
                                   solve_damped_schur_complement)

KP = 13


def ring_options(mixed=False):
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Huber
    o.solver.imageRobustLossScalePixels = 1.5
    o.solver.useReferenceOnlineSchur = False
    o.backend.enablePlaMatrixMixedPrecision = mixed
    return o


def aerial_options(mixed=False):
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Cauchy
    o.solver.imageRobustLossScalePixels = 1.5
    o.calibration.refineSharedFocalLength = True
    o.calibration.refineSharedPrincipalPoint = True
    o.calibration.refineSharedRadialDistortion = True
    o.solver.useReferenceOnlineSchur = False
    o.solver.maxIterations = 60
    o.backend.enablePlaMatrixMixedPrecision = mixed
    return o


def ring_c0():
    return synth.ring_problem()


def aerial_small():
    return synth.aerial_grid_problem(seed=3, n_along=5, n_lines=4, n_points=3000)


def equations_from_oracle_linearization(problem, orc):
    """A host container filled observation by observation from the oracle's linearisation at the
    initial state: camera pose term, intrinsic group term and the track's point, as addObservation
    hands them to addResidualBlocks."""
    p = problem.normalized()
    info, act, lin = orc.info(), orc.active(), orc.linearize_observations()
    eq = BlockNormalEquations(info["primary"], info["track_blocks"], KP, 3)
    trk = np.repeat(np.arange(p.n_tracks), np.diff(p.track_offsets))
    for k in range(p.n_obs):
        t = trk[k]
        if not act["active_track"][t] or not lin["valid"][k]:
            continue
        cam = p.obs_camera[k]
        prim, jac = [], []
        if act["camera_block"][cam] >= 0:
            prim.append(act["camera_block"][cam])
            jac.append(lin["pose_jacobian"][k])
        if act["intrinsic_block"][cam] >= 0:
            prim.append(act["intrinsic_block"][cam])
            jac.append(lin["intrinsic_jacobian"][k])
        eq.addResidualBlocks(prim, jac, int(act["track_block"][t]), lin["point_jacobian"][k], lin["residual"][k],
                             lin["normal_weight"][k])
    return eq


def close(a, b, rtol):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / scale < rtol


def test_host_container_equals_the_oracle_general_equations():
    p = ring_c0()
    orc = O.Oracle(p, ring_options())
    ref = orc.general_equations()
    got = equations_from_oracle_linearization(p, orc).export()
    assert close(got["H"], ref["H"], 1e-13)
    assert close(got["g"], ref["g"], 1e-12)
    assert close(got["Hee"], ref["Hee"], 1e-13)
    assert close(got["ge"], ref["ge"], 1e-12)
    # couplings: same (eliminated, primary) set and values
    gi = {tuple(k): i for i, k in enumerate(got["coupling_index"])}
    assert set(gi) == {tuple(k) for k in ref["coupling_index"]}
    W = np.stack([got["W"][gi[tuple(k)]] for k in ref["coupling_index"]])
    assert close(W, ref["W"], 1e-13)


def test_container_merge_shard_transpose_and_finalize_semantics():
    rng = np.random.default_rng(1)
    P, E, n = 4, 6, 5
    full = BlockNormalEquations(P, E, n, 3)
    shards = [BlockNormalEquations(P, 3, n, 3), BlockNormalEquations(P, 3, n, 3)]
    H = np.zeros((P * n + E * 3,) * 2)
    g = np.zeros(P * n + E * 3)
    for _ in range(40):
        prim = sorted(rng.choice(P, size=rng.integers(1, 3), replace=False).tolist())
        e = int(rng.integers(0, E))
        rows = int(rng.integers(1, 4))
        jac = [rng.normal(size=(rows, n)) for _ in prim]
        je = rng.normal(size=(rows, 3))
        r = rng.normal(size=rows)
        w = float(rng.uniform(0.5, 2.0))
        full.addResidualBlocks(prim, jac, e, je, r, w)
        shards[e // 3].addResidualBlocks(prim, jac, e % 3, je, r, w)
        J = np.zeros((rows, H.shape[0]))
        for b, jb in zip(prim, jac):
            J[:, b * n:(b + 1) * n] = jb
        J[:, P * n + 3 * e:P * n + 3 * e + 3] = je
        H += w * J.T @ J
        g += w * J.T @ r
    a = full.export()
    assert close(a["H"], H[:P * n, :P * n], 1e-13)
    assert close(a["g"], g[:P * n], 1e-13)
    assert close(a["Hee"], np.stack([H[P * n + 3 * e:P * n + 3 * e + 3, P * n + 3 * e:P * n + 3 * e + 3]
                                     for e in range(E)]), 1e-13)
    for (e, b), W in zip(a["coupling_index"], a["W"]):
        assert close(W, H[b * n:(b + 1) * n, P * n + 3 * e:P * n + 3 * e + 3], 1e-13)
    merged = BlockNormalEquations(P, E, n, 3)
    merged.mergeEliminatedShardFrom(shards[0], 0)
    merged.mergeEliminatedShardFrom(shards[1], 3)
    m = merged.export()
    for k in ("H", "g", "Hee", "ge"):
        assert close(m[k], a[k], 1e-13), k
    # a lower Hessian block is stored as the transpose of its upper mirror
    blk = rng.normal(size=(n, n))
    t = BlockNormalEquations(P, 0, n, 3)
    t.addPrimaryHessianBlock(2, 0, blk)
    np.testing.assert_array_equal(t.export()["H"][0:n, 2 * n:3 * n], blk.T)
    # finalizePrimaryDiagonal: non-zero entries scaled, zero entries set to `add`
    t.addPrimaryHessianBlock(1, 1, np.diag(np.r_[2.0, np.zeros(n - 1)]))
    t.finalizePrimaryDiagonal(1.5, 1.0)
    d = np.diag(t.export()["H"])[n:2 * n]
    np.testing.assert_array_equal(d, np.r_[3.0, np.ones(n - 1)])
    t.clearValues()
    assert not t.export()["H"].any()


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_device_damped_schur_solve_matches_the_oracle(mixed):
    from plabundle_gb300.device import Gb300Context
    p = ring_c0()
    orc = O.Oracle(p, ring_options())
    orc.general_equations()
    eq = equations_from_oracle_linearization(p, orc)
    ctx = Gb300Context(0)
    opts = SchurComplementSolverOptions(useMixedPrecision=mixed)
    for i, damping in enumerate((0.0, 1e-3, 1e-1)):
        x_ref, y_ref, cv = orc.general_solve(damping)
        assert cv
        x, y, rep = solve_damped_schur_complement(ctx, eq, damping, opts)
        assert rep["converged"] == 1 and rep["relative_residual"] <= 1e-11, rep
        assert rep["schur_pattern_reused"] == (1 if i > 0 else 0)
        assert rep["mixed_precision_used"] == int(mixed)
        # solutions of the same system to the 1e-12 relative residual (condition ~1e6 here)
        assert close(x, x_ref, 1e-6), np.abs(x - x_ref).max()
        assert close(y, y_ref, 1e-6), np.abs(y - y_ref).max()
    # warm start from the solution: converges at once to the same step
    x_ref, y_ref, _ = orc.general_solve(1e-3)
    x, y, rep = solve_damped_schur_complement(ctx, eq, 1e-3, SchurComplementSolverOptions(useInitialGuess=True),
                                              initial_guess=x_ref)
    assert rep["converged"] == 1 and rep["iterations"] <= 2 and close(x, x_ref, 1e-9)
    ctx.close()


@pytest.mark.gpu
def test_device_damped_schur_solve_reports_a_singular_point_block():
    from plabundle_gb300.device import Gb300Context
    eq = BlockNormalEquations(1, 1, 6, 3)
    J = np.eye(6)[:2]
    eq.addResidualBlocks([0], [J], 0, np.array([[1.0, 0, 0], [0, 1.0, 0]]), np.ones(2), 1.0)  # rank-2 point block
    eq.addPrimaryResidualBlock(0, np.eye(6), np.ones(6), 1.0)
    ctx = Gb300Context(0)
    with pytest.raises(SchurSolveError, match="numerically SPD"):
        solve_damped_schur_complement(ctx, eq, 0.0)
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,opts", [("ring", ring_c0, ring_options), ("aerial", aerial_small, aerial_options)])
def test_general_path_follows_the_oracle_general_path(name, make, opts):
    """FP64: the oracle's general-path trajectory (iterations, accepted steps, status, final cost
    to 1e-9, identical inliers); mixed: the same fixed point to 1e-6 in cost and 1e-5 in camera
    centres."""
    from plabundle_gb300.device import Gb300Context
    p = make()
    # the GPU's CG stops on its recursive residual: the oracle accepts its refined direct solves
    # likewise (no post-solve gate at the 1e-12 tolerance, which the FP64 residual floor can miss)
    ref = O.Oracle(p, opts(), residual_gate=False).solve()
    rr = ref["report"]
    assert rr["status"] == SolveStatus.Success
    C_ref = ref["cameras"][:, 9:12]
    scale = np.linalg.norm(C_ref - C_ref.mean(0), axis=1).max()
    for mixed in (False, True):
        ctx = Gb300Context(0)
        assert ctx.upload(p, opts(mixed)) == 0
        rep = ctx.solve()
        out = ctx.download()
        ctx.close()
        assert rep["status"] == SolveStatus.Success
        rel = abs(rep["final_cost"] - rr["final_cost"]) / rr["final_cost"]
        cerr = np.abs(out["cameras"][:, 9:12] - C_ref).max() / scale
        np.testing.assert_allclose(rep["initial_cost"], rr["initial_cost"], rtol=1e-12)
        assert np.array_equal(out["valid"], ref["valid"])
        if not mixed and name == "ring":
            assert rep["iterations"] == rr["iterations"] and rep["accepted_steps"] == rr["accepted_steps"]
            assert rep["linearizations"] == rr["linearizations"]
            assert rel < 1e-9 and cerr < 1e-8, (rel, cerr)
        elif not mixed:
            # Cauchy aerial block: the last iterations take steps whose cost change, and the forward-
            # difference directional decrease, sit at the FP64 rounding floor of the cost, so the
            # stopping iteration depends on the last bits; both solves end at the same fixed point
            assert abs(rep["iterations"] - rr["iterations"]) <= 4, (rep["iterations"], rr["iterations"])
            assert rel < 1e-9 and cerr < 1e-6, (rel, cerr)
        else:
            assert rel < 1e-6 and cerr < 1e-5, (rel, cerr)
