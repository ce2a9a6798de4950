"""The CPU implicit-differentiation reference (oracle/orc_adjoint.py) against finite differences.

Both sides work in one fixed chart around the solution: the finite differences perturb a datum
(an observation, the gauge baseline, the anchor camera's pose), re-converge the free variables by
Newton's method in that chart, and difference the camera-centre loss.  This pins the chart
formulas (rotation generators, gauge sphere, point scale, group intrinsics), the hyper-dual
second derivatives and the implicit-function-theorem algebra that the GPU backward pass is
checked against.
"""
import numpy as np
import pytest

import oracle as O
import orc_adjoint as A
from plabundle_gb300 import synth
from plabundle_gb300.problem import ImageRobustLoss, SolveOptions


def _options(loss=ImageRobustLoss.Cauchy):
    o = SolveOptions()
    o.solver.imageRobustLoss = loss
    o.solver.imageRobustLossScalePixels = 1.5
    o.calibration.refineSharedFocalLength = True
    o.calibration.refineSharedPrincipalPoint = True
    o.calibration.refineSharedRadialDistortion = True
    o.solver.maxIterations = 100
    return o


def _problem():
    return synth.aerial_grid_problem(seed=5, n_along=4, n_lines=3, n_points=300)


def _setup(loss=ImageRobustLoss.Cauchy):
    p = _problem()
    orc = O.Oracle(p, _options(loss))
    r = orc.solve()
    assert r["report"]["status"] == 1
    adj = A.AdjointOracle(orc, r["cameras"], r["points"], r["intrinsics"])
    z = adj.polish(np.zeros(adj.n_vars))
    return p, adj, z


def _fd(adj, z, vid, h, T):
    vals = []
    for sgn in (1.0, -1.0):
        zz = z.copy()
        zz[vid] += sgn * h
        zz = adj.polish(zz)
        vals.append(adj.centre_loss(zz, T)[0])
    return (vals[0] - vals[1]) / (2.0 * h)


@pytest.mark.parametrize("loss", [ImageRobustLoss.Cauchy, ImageRobustLoss.Huber])
def test_implicit_gradient_matches_finite_differences(loss):
    p, adj, z = _setup(loss)
    _, g, _ = adj.system(z)
    assert np.abs(g[adj.free]).max() < 1e-5  # polished to the fixed point
    T = A.centre_targets(p.truth_cameras, 0.1, seed=3)
    _, dL = adj.centre_loss(z, T)
    tot, _ = adj.implicit(dL, z)
    go = adj.observation_gradient(tot, p.n_obs)
    rng = np.random.default_rng(0)
    cand = np.nonzero(np.abs(go).sum(1) > 0)[0]
    # a Huber residual near its kink makes the central difference straddle a jump of rho''
    atol = 1e-5 * np.abs(go).max()
    for k in rng.choice(cand, 3, replace=False):
        for a in range(2):
            fd = _fd(adj, z, adj.base_o + 2 * k + a, 1e-3, T)
            assert abs(fd - go[k, a]) <= 1e-5 * abs(fd) + atol, (k, a, fd, go[k, a])
    # gauge data: the baseline, the anchor's centre and rotation (the anchor is fixed)
    for vid, h in [(adj.id_b, 1e-4), (6 * adj.anchor + 4, 1e-4), (6 * adj.anchor + 1, 1e-7)]:
        fd = _fd(adj, z, vid, h, T)
        assert abs(fd - tot[vid]) <= 2e-5 * abs(fd) + 1e-9, (vid, fd, tot[vid])


def test_hyper_dual_gradient_is_the_oracle_gradient():
    """First derivatives of the chart cost equal the oracle's analytic linearisation (J^T w r)."""
    p = _problem()
    orc = O.Oracle(p, _options())
    lin = orc.linearize_observations()  # at the initial state, which is the oracle's state now
    adj0 = A.AdjointOracle(orc, p.cameras, p.points, None)
    ids, val, grad, hess, _ = adj0.local()
    # observation order of orc_adjoint_local: usable observations of active tracks
    act = orc.active()["active_track"].astype(bool)
    trk = np.repeat(np.arange(p.n_tracks), np.diff(p.track_offsets))
    obs = np.nonzero(act[trk] & (lin["valid"] > 0))[0]
    assert obs.size == ids.shape[0]
    r = lin["residual"][obs]
    w = lin["normal_weight"][obs]
    jp = lin["point_jacobian"][obs]          # 2 x 3, in the point chart
    g_pt = np.einsum("n,nrc,nr->nc", w, jp, r)   # J^T w r
    # the point variables sit after the rotation (3) and centre (3, or 6 for the gauge camera)
    pos = np.array([np.nonzero((ids[i] >= 6 * p.n_cameras) & (ids[i] < 6 * p.n_cameras + 3 * p.n_tracks))[0][0]
                    for i in range(ids.shape[0])])
    hd_pt = np.stack([grad[i, pos[i]:pos[i] + 3] for i in range(ids.shape[0])])
    np.testing.assert_allclose(hd_pt, g_pt, rtol=1e-9, atol=1e-9 * np.abs(g_pt).max())
