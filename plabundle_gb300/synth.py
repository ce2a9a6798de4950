"""Seeded synthetic bundle-adjustment problems with the shapes of the benchmark workloads.

No public dataset is involved: every workload is generated from a seed.

* ``ring_problem``    -- 20 frame cameras on a circle (r=10 m, z=2 m) looking at the origin,
  4000x3000 px, f=3500, Brown k1=-0.05, k2=0.01, p1=p2=1e-4, 2 000 points in [-2,2]^3, each
  seen by a random 3..6 of the cameras that see it; 0.5 px noise, 2 % outliers, pose noise
  N(0, 0.01 rad) / N(0, 0.05 m), point noise N(0, 0.05 m).
* ``aerial_grid_problem`` -- 500 nadir cameras in a 25x20 grid at 100 m with 80 %/60 %
  forward/side overlap, 6000x4000 px, f=4000 px, 200 000 points on a sum-of-8-sinusoids
  terrain (20 m amplitude), 3..12 observations per track (~1.2 M), two shared calibration
  groups, 0.5 px noise, 3 % outliers.
* ``window_problems`` -- independent local windows generated like ``ring_problem`` with
  their own seeds, camera counts in 10..60 and point counts in 1k..20k.

The projector is the frame-pinhole Brown-Conrady model of
src/internal/BundleAdjustProjection.h:58-91 in the reference.
"""
from __future__ import annotations

import numpy as np

from .problem import (CAMERA_STRIDE, ControlPointConstraint, ControlPointUncertainty, Gauge, GaugePolicy,
                      Problem)


def look_at_rotation(centre: np.ndarray, target: np.ndarray, up=(0.0, 0.0, 1.0)) -> np.ndarray:
    """Camera-to-world rotation whose columns are the camera x (right), y (down), z (forward)."""
    f = np.asarray(target, float) - np.asarray(centre, float)
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, float))
    if np.linalg.norm(r) < 1e-9:
        r = np.cross(f, np.array([0.0, 1.0, 0.0]))
    r /= np.linalg.norm(r)
    d = np.cross(f, r)
    return np.stack([r, d, f], axis=1)


def make_camera(R, C, fx, fy, cx, cy, k=(0.0, 0.0, 0.0), p=(0.0, 0.0), width=0.0, height=0.0,
                u_sign=1.0, v_sign=1.0, flip=0.0) -> np.ndarray:
    cam = np.zeros(CAMERA_STRIDE)
    cam[0:9] = np.asarray(R, float).reshape(9)
    cam[9:12] = C
    cam[12:16] = (fx, fy, cx, cy)
    cam[16:19] = k
    cam[19:21] = p
    cam[21:26] = (u_sign, v_sign, flip, width, height)
    return cam


def project(cameras: np.ndarray, cam_idx: np.ndarray, X: np.ndarray):
    """Vectorised projection; returns (pixels [n,2], valid [n])."""
    cams = cameras[cam_idx]
    R = cams[:, 0:9].reshape(-1, 3, 3)
    d = X - cams[:, 9:12]
    xc = np.einsum("nij,ni->nj", R, d)
    z = xc[:, 2]
    fwd = np.where(cams[:, 23] != 0, -z, z)
    valid = fwd > 1e-9
    zs = np.where(valid, z, 1.0)
    x = xc[:, 0] / zs
    y = xc[:, 1] / zs
    r2 = x * x + y * y
    k1, k2, k3, p1, p2 = (cams[:, 16 + i] for i in range(5))
    radial = 1 + k1 * r2 + k2 * r2 * r2 + k3 * r2 ** 3
    xd = x * radial + p1 * 2 * x * y + p2 * (r2 + 2 * x * x)
    yd = y * radial + p1 * (r2 + 2 * y * y) + p2 * 2 * x * y
    u = cams[:, 21] * cams[:, 12] * xd + cams[:, 14]
    v = cams[:, 22] * cams[:, 13] * yd + cams[:, 15]
    return np.stack([u, v], axis=1), valid


def _project_one(cam: np.ndarray, X: np.ndarray):
    """`project` of all points X [n, 3] with one camera record (no per-point gather)."""
    R = cam[0:9].reshape(3, 3)
    xc = (X - cam[9:12]) @ R
    z = xc[:, 2]
    valid = (-z if cam[23] != 0 else z) > 1e-9
    zs = np.where(valid, z, 1.0)
    x = xc[:, 0] / zs
    y = xc[:, 1] / zs
    r2 = x * x + y * y
    k1, k2, k3, p1, p2 = cam[16:21]
    radial = 1 + k1 * r2 + k2 * r2 * r2 + k3 * r2 ** 3
    xd = x * radial + p1 * 2 * x * y + p2 * (r2 + 2 * x * x)
    yd = y * radial + p1 * (r2 + 2 * y * y) + p2 * 2 * x * y
    return np.stack([cam[21] * cam[12] * xd + cam[14], cam[22] * cam[13] * yd + cam[15]], axis=1), valid


def rotation_from_axis_angle(w: np.ndarray) -> np.ndarray:
    th = np.linalg.norm(w)
    if th < 1e-15:
        return np.eye(3)
    k = w / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K


def perturb_cameras(cameras: np.ndarray, rng, rot_sigma: float, centre_sigma: float) -> np.ndarray:
    out = cameras.copy()
    for i in range(out.shape[0]):
        dR = rotation_from_axis_angle(rng.normal(0.0, rot_sigma, 3))
        out[i, 0:9] = (dR @ out[i, 0:9].reshape(3, 3)).reshape(9)
        out[i, 9:12] += rng.normal(0.0, centre_sigma, 3)
    return out


def _choose_views_vectorized(visible_mask, rng, min_views, max_views):
    """Per point, a uniformly random subset of min(k, visible) of its visible cameras with
    k ~ U{min_views..max_views}, in camera order; vectorised over points (random keys, keep the
    k smallest)."""
    n_pts, n_c = visible_mask.shape
    k = rng.integers(min_views, max_views + 1, n_pts)
    keys = np.where(visible_mask, rng.random((n_pts, n_c)), np.inf)
    rank = np.argsort(np.argsort(keys, axis=1), axis=1)
    chosen = visible_mask & (rank < k[:, None])
    counts = chosen.sum(1).astype(np.int64)
    cam_idx = np.nonzero(chosen)[1].astype(np.int32)  # row-major: per point, cameras ascending
    return counts, cam_idx


def _assemble(cameras_true, cameras_init, X_true, X_init, visible_lists, rng, noise, outlier_frac,
              min_views, max_views, visible_mask=None):
    """Picks views per point, projects, adds noise and outliers; returns track-CSR arrays.
    With `visible_mask` ([points, cameras] bool) the views are drawn vectorised."""
    n_pts = X_true.shape[0]
    if visible_mask is not None:
        counts, cam_idx = _choose_views_vectorized(visible_mask, rng, min_views, max_views)
    else:
        counts = np.zeros(n_pts, np.int64)
        chosen = []
        for t in range(n_pts):
            vis = visible_lists[t]
            k = int(rng.integers(min_views, max_views + 1))
            if vis.size > k:
                vis = np.sort(rng.choice(vis, size=k, replace=False))
            chosen.append(vis)
            counts[t] = vis.size
        cam_idx = np.concatenate(chosen).astype(np.int32) if n_pts else np.zeros(0, np.int32)
    offsets = np.zeros(n_pts + 1, np.int64)
    np.cumsum(counts, out=offsets[1:])
    pt_idx = np.repeat(np.arange(n_pts), counts)
    px, _ = project(cameras_true, cam_idx, X_true[pt_idx])
    px = px + rng.normal(0.0, noise, px.shape)
    n_obs = cam_idx.size
    out_mask = rng.random(n_obs) < outlier_frac
    w = cameras_true[cam_idx, 24]
    h = cameras_true[cam_idx, 25]
    px[out_mask, 0] = rng.random(out_mask.sum()) * w[out_mask]
    px[out_mask, 1] = rng.random(out_mask.sum()) * h[out_mask]
    return offsets, cam_idx, px


def _problem(cameras_init, X_init, offsets, cam_idx, px, **kw) -> Problem:
    n_obs = cam_idx.size
    return Problem(cameras=cameras_init, points=X_init, track_offsets=offsets, obs_camera=cam_idx,
                   obs_u=px[:, 0].copy(), obs_v=px[:, 1].copy(), obs_weight=np.ones(n_obs),
                   obs_scale=np.ones(n_obs), **kw).normalized()


def _visible(cameras, X, margin=0.0, as_mask=False):
    """Per point, the sorted indices of the cameras that see it in front and in frame (or the
    [points, cameras] visibility mask with `as_mask`)."""
    n_c = cameras.shape[0]
    if as_mask:
        # camera by camera: all points against one camera record, no per-pair gather
        mask = np.zeros((X.shape[0], n_c), bool)
        for c in range(n_c):
            px, valid = _project_one(cameras[c], X)
            mask[:, c] = valid & (px[:, 0] >= margin) & (px[:, 0] < cameras[c, 24] - margin) \
                & (px[:, 1] >= margin) & (px[:, 1] < cameras[c, 25] - margin)
        return mask
    lists, masks = [], []
    chunk = max(1, 4_000_000 // max(1, n_c))
    for s in range(0, X.shape[0], chunk):
        Xs = X[s:s + chunk]
        m = Xs.shape[0]
        ci = np.tile(np.arange(n_c), m)
        pi = np.repeat(np.arange(m), n_c)
        px, valid = project(cameras, ci, Xs[pi])
        inside = valid & (px[:, 0] >= margin) & (px[:, 0] < cameras[ci, 24] - margin) \
            & (px[:, 1] >= margin) & (px[:, 1] < cameras[ci, 25] - margin)
        inside = inside.reshape(m, n_c)
        if as_mask:
            masks.append(inside)
        else:
            lists.extend(np.nonzero(row)[0] for row in inside)
    if as_mask:
        return np.concatenate(masks) if masks else np.zeros((0, n_c), bool)
    return lists


def ring_problem(seed: int = 7, n_cameras: int = 20, n_points: int = 2000, noise: float = 0.5,
                 outlier_frac: float = 0.02, rot_sigma: float = 0.01, centre_sigma: float = 0.05,
                 point_sigma: float = 0.05, min_views: int = 3, max_views: int = 6,
                 vectorized_views: bool = False) -> Problem:
    """The ring of cameras around a point cloud.  `vectorized_views` draws the views of all points
    at once (same distribution, another random stream; used for large batches of windows)."""
    rng = np.random.default_rng(seed)
    cams = []
    for i in range(n_cameras):
        a = 2 * np.pi * i / n_cameras
        C = np.array([10 * np.cos(a), 10 * np.sin(a), 2.0])
        R = look_at_rotation(C, np.zeros(3))
        cams.append(make_camera(R, C, 3500.0, 3500.0, 2000.0, 1500.0, k=(-0.05, 0.01, 0.0), p=(1e-4, 1e-4),
                                width=4000.0, height=3000.0))
    cams = np.array(cams)
    X = rng.uniform(-2.0, 2.0, (n_points, 3))
    if vectorized_views:
        mask = _visible(cams, X, as_mask=True)
        offsets, cam_idx, px = _assemble(cams, None, X, None, None, rng, noise, outlier_frac, min_views, max_views,
                                         visible_mask=mask)
    else:
        vis = _visible(cams, X)
        offsets, cam_idx, px = _assemble(cams, None, X, None, vis, rng, noise, outlier_frac, min_views, max_views)
    cams0 = perturb_cameras(cams, rng, rot_sigma, centre_sigma)
    X0 = X + rng.normal(0.0, point_sigma, X.shape)
    prob = _problem(cams0, X0, offsets, cam_idx, px)
    prob.truth_cameras = cams
    prob.truth_points = X
    return prob


def _terrain(rng, n_waves=8, amplitude=20.0):
    k = rng.uniform(0.003, 0.03, (n_waves, 2)) * rng.choice([-1.0, 1.0], (n_waves, 2))
    ph = rng.uniform(0, 2 * np.pi, n_waves)
    a = rng.uniform(0.5, 1.5, n_waves)
    a *= amplitude / a.sum()

    def height(x, y):
        return (a[None, :] * np.sin(x[:, None] * k[None, :, 0] + y[:, None] * k[None, :, 1] + ph[None, :])).sum(1)

    return height


def aerial_grid_problem(seed: int = 11, n_along: int = 25, n_lines: int = 20, n_points: int = 200_000,
                        altitude: float = 100.0, width: float = 6000.0, height: float = 4000.0,
                        focal: float = 4000.0, forward_overlap: float = 0.8, side_overlap: float = 0.6,
                        noise: float = 0.5, outlier_frac: float = 0.03, rot_sigma: float = 0.01,
                        centre_sigma: float = 0.05, point_sigma: float = 0.05, min_views: int = 3,
                        max_views: int = 12, n_groups: int = 2, intrinsic_error: bool = True) -> Problem:
    rng = np.random.default_rng(seed)
    foot_x = width / focal * altitude     # image x along world x
    foot_y = height / focal * altitude    # image y along world -y (flight direction)
    step_along = (1 - forward_overlap) * foot_y
    step_side = (1 - side_overlap) * foot_x
    truth_models = []
    for g in range(n_groups):
        truth_models.append(dict(f=focal * (1 + 0.002 * g), cx=width / 2 + 3.0 * g, cy=height / 2 - 2.0 * g,
                                 k=(-0.04 + 0.005 * g, 0.008, -0.001), p=(1e-4, -1e-4)))
    R = look_at_rotation(np.zeros(3), np.array([0.0, 0.0, -1.0]), up=(0.0, 1.0, 0.0))
    cams, groups = [], []
    for line in range(n_lines):
        for j in range(n_along):
            g = line % n_groups
            m = truth_models[g]
            C = np.array([line * step_side, j * step_along, altitude])
            cams.append(make_camera(R, C, m["f"], m["f"], m["cx"], m["cy"], k=m["k"], p=m["p"],
                                    width=width, height=height))
            groups.append(g)
    cams = np.array(cams)
    groups = np.array(groups, np.int32)
    hfun = _terrain(rng)
    xs = rng.uniform(-0.35 * foot_x, (n_lines - 1) * step_side + 0.35 * foot_x, n_points)
    ys = rng.uniform(-0.35 * foot_y, (n_along - 1) * step_along + 0.35 * foot_y, n_points)
    X = np.stack([xs, ys, hfun(xs, ys)], axis=1)
    vis = _visible_grid(cams, X, foot_x, foot_y)
    offsets, cam_idx, px = _assemble(cams, None, X, None, vis, rng, noise, outlier_frac, min_views, max_views)
    keep = np.diff(offsets) >= 2
    if not keep.all():
        X, offsets, cam_idx, px = _drop_tracks(X, offsets, cam_idx, px, keep)
    cams0 = perturb_cameras(cams, rng, rot_sigma, centre_sigma)
    if intrinsic_error:
        for g in range(n_groups):
            sel = groups == g
            cams0[sel, 12] *= 1.0 + 0.003 * (1 if g == 0 else -1)
            cams0[sel, 13] = cams0[sel, 12]
            cams0[sel, 14] += 4.0
            cams0[sel, 15] -= 3.0
            cams0[sel, 16] += 0.004
    X0 = X + rng.normal(0.0, point_sigma, X.shape)
    prob = _problem(cams0, X0, offsets, cam_idx, px, cameraCalibrationGroupIds=groups)
    prob.truth_cameras = cams
    prob.truth_points = X
    return prob


def _visible_grid(cams, X, foot_x, foot_y):
    """Visibility for nadir grids: candidate cameras within one footprint, then exact test."""
    C = cams[:, 9:12]
    lists = []
    order = np.argsort(C[:, 0] * 1e6 + C[:, 1])
    chunk = 20000
    for s in range(0, X.shape[0], chunk):
        Xs = X[s:s + chunk]
        near = (np.abs(Xs[:, None, 0] - C[None, :, 0]) < 0.6 * foot_x) & \
               (np.abs(Xs[:, None, 1] - C[None, :, 1]) < 0.6 * foot_y)
        pi, ci = np.nonzero(near)
        px, valid = project(cams, ci, Xs[pi])
        ok = valid & (px[:, 0] >= 0) & (px[:, 0] < cams[ci, 24]) & (px[:, 1] >= 0) & (px[:, 1] < cams[ci, 25])
        pi, ci = pi[ok], ci[ok]
        split = np.searchsorted(pi, np.arange(Xs.shape[0] + 1))
        for t in range(Xs.shape[0]):
            lists.append(np.sort(ci[split[t]:split[t + 1]]))
    del order
    return lists


def _drop_tracks(X, offsets, cam_idx, px, keep):
    counts = np.diff(offsets)
    obs_keep = np.repeat(keep, counts)
    counts = counts[keep]
    new_off = np.zeros(counts.size + 1, np.int64)
    np.cumsum(counts, out=new_off[1:])
    return X[keep], new_off, cam_idx[obs_keep], px[obs_keep]


def window_problems(n_windows: int = 256, seed: int = 1234, cameras=(10, 60), points=(1000, 20000)):
    rng = np.random.default_rng(seed)
    out = []
    for w in range(n_windows):
        nc = int(rng.integers(cameras[0], cameras[1] + 1))
        npt = int(rng.integers(points[0], points[1] + 1))
        out.append(ring_problem(seed=seed * 1000 + w, n_cameras=nc, n_points=npt, vectorized_views=True))
    return out


def with_gauge(problem: Problem, policy=GaugePolicy.AutoAnchor) -> Problem:
    problem.gauge = Gauge(policy=policy)
    return problem


def with_scale_bars(problem: Problem, n: int = 10, sigma: float = 0.005, seed: int = 0,
                    max_length: float = 20.0, weights=(1.0, 0.5, 2.0)) -> Problem:
    """Scale bars between `n` disjoint pairs of tracks seen by two distinct cameras, their true
    points at most `max_length` apart (the closest candidate to a random track): measured
    distance = true distance + N(0, sigma), sigma and the weights cycling as given."""
    from .problem import ScaleBarConstraint
    rng = np.random.default_rng(seed)
    off = np.asarray(problem.track_offsets)
    cams = np.asarray(problem.obs_camera)
    truth = getattr(problem, "truth_points", None)
    truth = problem.points if truth is None else truth
    eligible = np.array([t for t in range(problem.n_tracks) if np.unique(cams[off[t]:off[t + 1]]).size >= 2])
    used = set()
    bars = []
    for t in rng.permutation(eligible):
        if len(bars) >= n:
            break
        if t in used:
            continue
        d = np.linalg.norm(truth[eligible] - truth[t], axis=1)
        order = np.argsort(d)
        for j in order[1:]:
            u = int(eligible[j])
            if u in used or u == t or d[j] <= 0.5 or d[j] > max_length:
                continue
            used.update((int(t), u))
            length = float(np.linalg.norm(truth[u] - truth[t])) + rng.normal(0.0, sigma)
            bars.append(ScaleBarConstraint(trackIndexA=int(t), trackIndexB=u, measuredDistanceMeters=length,
                                           sigmaMeters=sigma, weight=weights[len(bars) % len(weights)],
                                           sourceIndex=len(bars)))
            break
    problem.scaleBarConstraints = bars
    return problem


def with_control_points(problem: Problem, n: int = 12, sigma: float = 0.02, seed: int = 0,
                        kinds=(0, 1, 2), weights=(1.0, 0.5, 2.0)) -> Problem:
    """Survey control points on `n` tracks seen by two distinct cameras: the true point plus
    Gaussian noise (0.1 sigma on every other target, so that both Huber branches occur), with
    the uncertainty cycling through isotropic sigma, a correlated covariance and the matching
    upper-triangular square-root information (kinds 0, 1, 2)."""
    rng = np.random.default_rng(seed)
    off = np.asarray(problem.track_offsets)
    cams = np.asarray(problem.obs_camera)
    eligible = [t for t in range(problem.n_tracks) if np.unique(cams[off[t]:off[t + 1]]).size >= 2]
    pick = np.sort(rng.choice(np.array(eligible), size=min(n, len(eligible)), replace=False))
    truth = getattr(problem, "truth_points", None)
    truth = problem.points if truth is None else truth
    cps = []
    for i, t in enumerate(pick):
        scale = sigma * (0.1 if i % 2 else 1.0)
        target = truth[t] + rng.normal(0.0, scale, 3)
        kind = kinds[i % len(kinds)]
        B = rng.normal(0.0, 0.4, (3, 3))
        cov = sigma * sigma * (np.eye(3) + B @ B.T)
        c = ControlPointConstraint(point=tuple(target), sigmaMeters=sigma, weight=weights[i % len(weights)],
                                   uncertainty=ControlPointUncertainty(kind))
        if kind == 1:
            c.uncertaintyMatrix = tuple(cov.reshape(9))
        elif kind == 2:
            c.uncertaintyMatrix = tuple(np.linalg.cholesky(np.linalg.inv(cov)).T.reshape(9))
        cps.append((int(t), c))
    problem.controlPoints = cps
    return problem



def _visible_pairs(cams: np.ndarray, X: np.ndarray, zlo: float, zhi: float, cell: float = 25.0):
    """(point, camera) pairs of every camera that sees a point in front and in frame, sorted by
    point then camera.  Candidates per camera come from the cells of a ground grid that cover the
    camera's footprint between the heights zlo and zhi."""
    x0, y0 = X[:, 0].min(), X[:, 1].min()
    nx = int((X[:, 0].max() - x0) // cell) + 1
    ny = int((X[:, 1].max() - y0) // cell) + 1
    cx = np.clip(((X[:, 0] - x0) // cell).astype(np.int64), 0, nx - 1)
    cy = np.clip(((X[:, 1] - y0) // cell).astype(np.int64), 0, ny - 1)
    cid = cy * nx + cx
    order = np.argsort(cid, kind="stable")
    start = np.searchsorted(cid[order], np.arange(nx * ny + 1))
    pis, cis = [], []
    for c in range(cams.shape[0]):
        cam = cams[c]
        R = cam[0:9].reshape(3, 3)
        C = cam[9:12]
        w, h = cam[24], cam[25]
        corners = np.array([[0, 0], [w, 0], [0, h], [w, h]], float)
        rays = np.stack([(corners[:, 0] - cam[14]) / cam[12], (corners[:, 1] - cam[15]) / cam[13],
                         np.ones(4)], axis=1) @ R.T
        if np.any(rays[:, 2] >= -1e-6):
            continue  # a corner ray does not reach the ground: not an aerial view
        pts = []
        for z in (zlo, zhi):
            t = (z - C[2]) / rays[:, 2]
            pts.append(C[None, :2] + t[:, None] * rays[:, :2])
        pts = np.concatenate(pts)
        gx0 = max(0, int((pts[:, 0].min() - x0) // cell))
        gx1 = min(nx - 1, int((pts[:, 0].max() - x0) // cell))
        gy0 = max(0, int((pts[:, 1].min() - y0) // cell))
        gy1 = min(ny - 1, int((pts[:, 1].max() - y0) // cell))
        if gx1 < gx0 or gy1 < gy0:
            continue
        cand = np.concatenate([order[start[gy * nx + gx0]:start[gy * nx + gx1 + 1]] for gy in range(gy0, gy1 + 1)])
        if cand.size == 0:
            continue
        px, valid = _project_one(cam, X[cand])
        ok = valid & (px[:, 0] >= 0) & (px[:, 0] < w) & (px[:, 1] >= 0) & (px[:, 1] < h)
        pis.append(cand[ok])
        cis.append(np.full(int(ok.sum()), c, np.int32))
    pi = np.concatenate(pis) if pis else np.zeros(0, np.int64)
    ci = np.concatenate(cis) if cis else np.zeros(0, np.int32)
    # the pairs are grouped by ascending camera: a stable sort by point gives (point, camera) order
    o = np.argsort(pi, kind="stable")
    return pi[o], ci[o]


def _choose_views_sparse(pi, ci, n_pts, rng, min_views, max_views):
    """Per point, a uniformly random subset of min(k, visible) of its visible cameras with
    k ~ U{min_views..max_views}, in camera order; from sorted (point, camera) pairs."""
    k = rng.integers(min_views, max_views + 1, n_pts)
    keys = rng.random(pi.size)
    # order by point, then by the random key (the point index plus a key in [0, 1) is exact in
    # FP64 for the point counts used here)
    o = np.argsort(pi.astype(np.float64) + keys)
    start = np.searchsorted(pi[o], np.arange(n_pts + 1))
    rank = np.arange(pi.size) - np.repeat(start[:-1], np.diff(start))
    keep = np.zeros(pi.size, bool)
    keep[o[rank < k[pi[o]]]] = True
    pi, ci = pi[keep], ci[keep]          # still sorted by (point, camera)
    counts = np.bincount(pi, minlength=n_pts).astype(np.int64)
    return counts, ci.astype(np.int32)


def rig_grid_problem(seed: int = 21, n_along: int = 30, n_lines: int = 20, n_points: int = 1_500_000,
                     altitude: float = 100.0, width: float = 6000.0, height: float = 4000.0,
                     nadir_focal: float = 4000.0, oblique_focal: float = 8000.0, tilt_deg: float = 45.0,
                     forward_overlap: float = 0.8, side_overlap: float = 0.6, noise: float = 0.7,
                     outlier_frac: float = 0.05, rot_sigma: float = 0.01, centre_sigma: float = 0.05,
                     point_sigma: float = 0.05, sensor_rot_sigma: float = 0.003, sensor_centre_sigma: float = 0.01,
                     min_views: int = 3, max_views: int = 8, n_obliques: int = 4):
    """Oblique block of 5-camera rigs: captures on a flight grid at `altitude` (nadir overlap
    80 %/60 %), each with a nadir camera (the rig's fixed body-frame sensor) and `n_obliques`
    cameras tilted `tilt_deg` forward, backward, left and right, whose extrinsics (rotation and
    lever arm) are refined.  Points on a sum-of-sinusoids terrain, each observed by a random
    3..`max_views` of the cameras that see it; pixel noise `noise`, `outlier_frac` outliers.
    Initial captures are perturbed by N(0, rot_sigma) / N(0, centre_sigma), initial free sensors
    are the nominal extrinsics (the truth differs by N(0, sensor_rot_sigma) / N(0,
    sensor_centre_sigma)), initial points by N(0, point_sigma)."""
    from .problem import RigCameraBinding, RigCapture, RigSensor, RigTopology
    rng = np.random.default_rng(seed)
    foot_x = width / nadir_focal * altitude
    foot_y = height / nadir_focal * altitude
    step_along = (1 - forward_overlap) * foot_y
    step_side = (1 - side_overlap) * foot_x
    tilt = np.deg2rad(tilt_deg)
    dirs = [np.array([1.0, 0.0]), np.array([-1.0, 0.0]), np.array([0.0, 1.0]), np.array([0.0, -1.0])][:n_obliques]
    # nominal sensors: nadir (fixed) and obliques, camera-to-rig rotations and lever arms
    nominal = [(look_at_rotation(np.zeros(3), np.array([0.0, 0.0, -1.0]), up=(0.0, 1.0, 0.0)), np.zeros(3))]
    for d in dirs:
        f = np.array([d[0] * np.sin(tilt), d[1] * np.sin(tilt), -np.cos(tilt)])
        nominal.append((look_at_rotation(np.zeros(3), f, up=(0.0, 0.0, 1.0)),
                        np.array([0.12 * d[0], 0.12 * d[1], -0.05])))
    n_sen = len(nominal)
    truth_sen, init_sen = [], []
    for s, (Rn, tn) in enumerate(nominal):
        if s == 0:
            truth_sen.append((Rn, tn))
        else:
            dR = rotation_from_axis_angle(rng.normal(0.0, sensor_rot_sigma, 3))
            truth_sen.append((dR @ Rn, tn + rng.normal(0.0, sensor_centre_sigma, 3)))
        init_sen.append((Rn, tn))
    models = [dict(f=nadir_focal, k=(-0.03, 0.006, 0.0), p=(1e-4, -1e-4))]
    models += [dict(f=oblique_focal, k=(-0.02, 0.004, 0.0), p=(-1e-4, 1e-4)) for _ in dirs]
    truth_cap, cap_pos = [], []
    for line in range(n_lines):
        for j in range(n_along):
            yaw = rng.normal(0.0, 0.02)
            truth_cap.append((rotation_from_axis_angle(np.array([0.0, 0.0, yaw])),
                              np.array([line * step_side, j * step_along, altitude])))
    n_cap = len(truth_cap)

    def compose(caps, sens):
        out = []
        for k, (Rc, Cc) in enumerate(caps):
            for s, (Rs, ts) in enumerate(sens):
                m = models[s]
                out.append(make_camera(Rc @ Rs, Cc + Rc @ ts, m["f"], m["f"], width / 2, height / 2, k=m["k"],
                                       p=m["p"], width=width, height=height))
        return np.array(out)

    cams = compose(truth_cap, truth_sen)
    hfun = _terrain(rng)
    margin_x, margin_y = 0.45 * foot_x, 0.45 * foot_y
    xs = rng.uniform(-margin_x, (n_lines - 1) * step_side + margin_x, n_points)
    ys = rng.uniform(-margin_y, (n_along - 1) * step_along + margin_y, n_points)
    X = np.stack([xs, ys, hfun(xs, ys)], axis=1)
    pi, ci = _visible_pairs(cams, X, X[:, 2].min() - 1.0, X[:, 2].max() + 1.0)
    counts, cam_idx = _choose_views_sparse(pi, ci, n_points, rng, min_views, max_views)
    offsets = np.zeros(n_points + 1, np.int64)
    np.cumsum(counts, out=offsets[1:])
    pt_idx = np.repeat(np.arange(n_points), counts)
    px, _ = project(cams, cam_idx, X[pt_idx])
    px = px + rng.normal(0.0, noise, px.shape)
    out_mask = rng.random(cam_idx.size) < outlier_frac
    px[out_mask, 0] = rng.random(out_mask.sum()) * width
    px[out_mask, 1] = rng.random(out_mask.sum()) * height
    keep = counts >= 2
    if not keep.all():
        X, offsets, cam_idx, px = _drop_tracks(X, offsets, cam_idx, px, keep)
    init_cap = []
    for Rc, Cc in truth_cap:
        dR = rotation_from_axis_angle(rng.normal(0.0, rot_sigma, 3))
        init_cap.append((dR @ Rc, Cc + rng.normal(0.0, centre_sigma, 3)))
    cams0 = compose(init_cap, init_sen)
    X0 = X + rng.normal(0.0, point_sigma, X.shape)
    rig = RigTopology(
        captures=[RigCapture(rigId=0, captureId=k, rigToWorldRotation=tuple(R.reshape(9)), rigCenterInWorld=tuple(C))
                  for k, (R, C) in enumerate(init_cap)],
        sensors=[RigSensor(rigId=0, sensorId=s, cameraToRigRotation=tuple(R.reshape(9)), cameraCenterInRig=tuple(t),
                           fixedExtrinsic=(s == 0)) for s, (R, t) in enumerate(init_sen)],
        cameraBindings=[RigCameraBinding(cameraIndex=k * n_sen + s, rigId=0, captureId=k, sensorId=s)
                        for k in range(n_cap) for s in range(n_sen)])
    prob = _problem(cams0, X0, offsets, cam_idx, px, rig=rig)
    prob.truth_cameras = cams
    prob.truth_points = X
    prob.truth_captures = np.array([np.concatenate([R.reshape(9), C]) for R, C in truth_cap])
    prob.truth_sensors = np.array([np.concatenate([R.reshape(9), t]) for R, t in truth_sen])
    return prob
