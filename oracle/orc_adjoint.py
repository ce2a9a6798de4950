"""Implicit-differentiation reference of a converged bundle adjustment (test infrastructure).

Only tests/ and bench.py's checking legs use this module; the product path never imports it.
The reference has no adjoint, so there is nothing to pin it to: it is an independent CPU
statement of the same mathematics, checked by the tests against central finite differences of
a Newton-polished fixed point in the same chart.

At a fixed point z* of the robust objective F(z; d) in local chart variables (z: free cameras,
points and group intrinsics; d: observations, fixed cameras and tracks, the gauge baseline),
the implicit function theorem gives, for a scalar loss L(z, d):

    H_zz mu = dL/dz,        dL/dd (total) = dL/dd (partial) - H_dz mu,

with H the exact Hessian of F (robust-loss second derivatives and residual curvature included,
not Gauss-Newton).  The per-observation blocks of H come from the oracle's hyper-dual
evaluation (`orc_adjoint_local`, exact to rounding); the prior terms of the group intrinsics
add invSigma^2 on their diagonal; H_zz is solved with scipy's sparse LU (SuperLU) and iterative
refinement.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import lib, _ptr  # noqa: F401  (oracle.py is importable as a module from tests)

_KMAX = 24
_P = 13


def _bind(L):
    if getattr(L, "_adjoint_bound", False):
        return L
    L.orc_set_state.argtypes = [C.c_void_p] + [C.c_void_p] * 3
    L.orc_adjoint_layout.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.c_void_p, C.c_void_p]
    L.orc_adjoint_local.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)] + [C.c_void_p] * 5
    L._adjoint_bound = True
    return L


def solve_refined(Hc, b, max_sweeps=30, tol=1e-15):
    """Sparse LU (SuperLU) solve of the Jacobi-scaled system with iterative refinement on the
    FP64 residual.  The Hessians here have Jacobi-scaled condition numbers around 1e10 (and far
    larger unscaled, the variables carry different units): one LU solve leaves a relative
    residual near 1e-6, the refinement sweeps bring it to rounding level."""
    d = np.sqrt(np.abs(Hc.diagonal()))
    d[d == 0] = 1.0
    Di = sp.diags(1.0 / d)
    Hs = (Di @ Hc @ Di).tocsc()
    lu = spla.splu(Hs)
    bs = b / d
    y = lu.solve(bs)
    nb = np.linalg.norm(bs)
    for _ in range(max_sweeps):
        r = bs - Hs @ y
        if np.linalg.norm(r) <= tol * nb:
            break
        dy = lu.solve(r)
        y = y + dy
        if np.linalg.norm(dy) <= tol * np.linalg.norm(y):
            break
    return y / d


class AdjointOracle:
    """Adjoint reference bound to one `oracle.Oracle` instance whose state is the fixed point."""

    def __init__(self, orc, cameras, points, groups=None):
        self.orc = orc
        self.L = _bind(lib())
        p = orc.problem
        self.nc, self.nt = p.n_cameras, p.n_tracks
        cams = np.ascontiguousarray(cameras, np.float64)
        pts = np.ascontiguousarray(points, np.float64)
        grp = None if groups is None else np.ascontiguousarray(groups, np.float64)
        self.L.orc_set_state(orc.h, _ptr(cams), _ptr(pts), None if grp is None else _ptr(grp))
        self.state_cams = cams.copy()
        n = C.c_int64(0)
        self.L.orc_adjoint_layout(orc.h, C.byref(n), None, None)
        self.n_vars = n.value
        self.kind = np.zeros(self.n_vars, np.int8)
        self.geom = np.zeros(17)
        self.L.orc_adjoint_layout(orc.h, C.byref(n), _ptr(self.kind), _ptr(self.geom))
        self.ng = orc.info()["intrinsic_blocks"]
        self.base_g = 6 * self.nc + 3 * self.nt
        self.id_b = self.base_g + _P * self.ng
        self.base_o = self.id_b + 1
        self.free = np.nonzero(self.kind == 1)[0]
        self.param = np.nonzero(self.kind == 2)[0]
        self.anchor = int(self.geom[0])
        self.scale = int(self.geom[1])

    # ---- per-observation blocks and the global Hessian -------------------------------------------
    def local(self, z0=None):
        cnt = C.c_int64(0)
        ph = np.zeros(3 * max(1, self.ng) * _P)
        z = None if z0 is None else np.ascontiguousarray(z0, np.float64)
        self.L.orc_adjoint_local(self.orc.h, None if z is None else _ptr(z), C.byref(cnt), None, None, None, None,
                                 _ptr(ph))
        m = cnt.value
        ids = np.zeros((m, _KMAX), np.int32)
        val = np.zeros(m)
        grad = np.zeros((m, _KMAX))
        hess = np.zeros((m, _KMAX, _KMAX))
        bad = self.L.orc_adjoint_local(self.orc.h, None if z is None else _ptr(z), C.byref(cnt), _ptr(ids), _ptr(val),
                                       _ptr(grad), _ptr(hess), _ptr(ph))
        if bad:
            raise RuntimeError("an observation does not project at this state")
        k = self.ng * _P
        return ids, val, grad, hess, (ph[:k], ph[k:2 * k], ph[2 * k:3 * k])

    def system(self, z0=None):
        """(objective, gradient, sparse Hessian) over all variables at state (+) z0."""
        ids, val, grad, hess, ph = self.local(z0)
        n = self.n_vars
        mask = ids >= 0
        g = np.zeros(n)
        np.add.at(g, ids[mask], grad[mask])
        rows = np.broadcast_to(ids[:, :, None], hess.shape)
        cols = np.broadcast_to(ids[:, None, :], hess.shape)
        m2 = (rows >= 0) & (cols >= 0)
        H = sp.coo_matrix((hess[m2], (rows[m2], cols[m2])), shape=(n, n)).tocsr()
        f = float(val.sum())
        if self.ng:
            # priors 0.5 * (invSigma (theta - prior))^2 in the additive group chart
            ph_h, ph_g, ph_c = ph
            gid = self.base_g + np.arange(self.ng * _P)
            on = ph_h > 0
            H = H + sp.csr_matrix((ph_h[on], (gid[on], gid[on])), shape=(n, n))
            g[gid] += ph_g
            f += float(ph_c.sum())
        return f, g, H

    # ---- camera centres as functions of the chart -------------------------------------------------
    def centres(self, z):
        """Camera centres at state (+) z and their derivatives d C_c / d z as a sparse (3 nc x n) map."""
        nc = self.nc
        Cs = self.state_cams[:, 9:12].copy()
        rows, cols, vals = [], [], []
        for c in range(nc):
            if c == self.scale:
                continue
            Cs[c] += z[6 * c + 3:6 * c + 6]
            for i in range(3):
                rows.append(3 * c + i); cols.append(6 * c + 3 + i); vals.append(1.0)
        if self.scale >= 0:
            s, a = self.scale, self.anchor
            e, B = self.geom[3:6], self.geom[6:12].reshape(2, 3)
            t = z[6 * s + 3:6 * s + 5]
            bl = self.geom[2] + z[self.id_b]
            d = e + t[0] * B[0] + t[1] * B[1]
            ln = np.linalg.norm(d)
            nvec = d / ln
            A = self.geom[12:15] + z[6 * a + 3:6 * a + 6]
            Cs[s] = A + bl * nvec
            for p in range(2):
                dp = bl / ln * (B[p] - nvec * (nvec @ B[p]))
                for i in range(3):
                    rows.append(3 * s + i); cols.append(6 * s + 3 + p); vals.append(dp[i])
            for i in range(3):
                rows.append(3 * s + i); cols.append(self.id_b); vals.append(nvec[i])
                rows.append(3 * s + i); cols.append(6 * a + 3 + i); vals.append(1.0)
        J = sp.csr_matrix((vals, (rows, cols)), shape=(3 * nc, self.n_vars))
        return Cs, J

    def centre_loss(self, z, targets):
        Cs, J = self.centres(z)
        r = (Cs - targets).ravel()
        return float(r @ r), J.T @ (2.0 * r)

    # ---- Newton polish of the free variables (for finite differences) ---------------------------
    def polish(self, z0, iterations=30, tol=1e-15):
        z = np.array(z0, np.float64)
        fr = self.free
        for _ in range(iterations):
            _, g, H = self.system(z)
            step = solve_refined(H[fr][:, fr].tocsc(), g[fr])
            z[fr] -= step
            if np.max(np.abs(step)) <= tol * max(1.0, np.max(np.abs(z[fr]))):
                break
        return z

    # ---- the implicit gradient ---------------------------------------------------------------
    def implicit(self, dLdz, z=None):
        """Total derivative of L w.r.t. every parameter variable, given dL/dz over all variables
        (partial derivatives); returns (dL/d params as a full-length vector, mu over the free
        variables)."""
        z = np.zeros(self.n_vars) if z is None else z
        _, _, H = self.system(z)
        fr, pa = self.free, self.param
        mu = solve_refined(H[fr][:, fr].tocsc(), dLdz[fr])
        out = np.zeros(self.n_vars)
        out[pa] = dLdz[pa] - H[pa][:, fr] @ mu
        return out, mu

    def observation_gradient(self, total, n_obs):
        return total[self.base_o:self.base_o + 2 * n_obs].reshape(n_obs, 2)

    def initial_pose_gradient(self, total, initial_cameras):
        """dL/d(initial camera pose) per camera as (rotation increment, centre): fixed cameras
        directly; the gauge baseline b = |C_scale^0 - C_anchor^0| adds to both centres."""
        g = np.zeros((self.nc, 6))
        for c in range(self.nc):
            if self.kind[6 * c] == 2:
                g[c] = total[6 * c:6 * c + 6]
        if self.scale >= 0:
            d = initial_cameras[self.scale, 9:12] - initial_cameras[self.anchor, 9:12]
            db = total[self.id_b] * d / np.linalg.norm(d)
            g[self.scale, 3:6] += db
            g[self.anchor, 3:6] -= db
        return g


def centre_targets(truth_cameras, sigma=0.1, seed=0):
    """Targets of the camera-centre loss: true centres plus N(0, sigma^2) per axis."""
    rng = np.random.default_rng(seed)
    return truth_cameras[:, 9:12] + rng.normal(0.0, sigma, (truth_cameras.shape[0], 3))
