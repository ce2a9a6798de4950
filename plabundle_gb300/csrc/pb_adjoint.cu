// pb_adjoint.cu -- backward pass: implicit differentiation of the converged LM fixed point.
//
// No counterpart in the reference (it has no adjoint).  At a fixed point z* of the robust
// objective F(z; d) in the solver's own local chart (pose rotation increment C2W' = D E(w)^T D C2W
// with E = Rx Ry Rz, world centre increment or the 2-DoF gauge tangent, point increment
// X + s(X) dX, additive group intrinsics), the implicit function theorem gives for a scalar loss L
//     H mu = dL/dz,    dL/dd = (partial) dL/dd - H_dz mu
// with H the EXACT Hessian of F: per observation
//     H_o = J^T W2 J + sum_k lam_k d2 r_k,   W2 = 2 rho' w I + 4 rho'' w^2 r r^T,  lam = 2 rho' w r,
// i.e. the robust loss's second derivative and the residual curvature are both kept (Gauss-Newton
// drops them; at a Cauchy-weighted fixed point the rho'' term is of the same order as J^T w J).
//
//   k_adj_hessian   one thread per observation: FP64 Jacobian (linearize_obs), W2, and the
//                   curvature lam^T d2 pi: analytic second derivatives of the projection over the
//                   camera-frame point and the intrinsics, composed with the second derivatives
//                   of the camera-frame point in the chart (rotation generators, gauge sphere);
//                   writes one record per observation.
//   k_adj_assemble  one CTA per chunk of the forward path's chunk plan: point blocks V = sum H_pp,
//                   V^-1 (FP64), and the eliminated system -W V^-1 W^T plus the own terms, every
//                   output element owned by one thread (fixed-order sums, no atomics), written
//                   as FP64 chunk partials and summed by the forward reduce kernels into the
//                   reduced system (pose CSR blocks, border, intrinsic block);
//   k_adj_finalize  priors (invSigma^2), empty diagonals;
//   k_adj_rhs       dL/dz of the primary variables added to the reduced right-hand side.
//   (the reduced system is then solved by the forward path's dense Cholesky-preconditioned CG
//    or block-Jacobi PCG)
//   k_adj_gradient  one thread per track: point back-substitution mu_p = V^-1 (b_p - W^T mu_c),
//                   dL/d(u, v) = W2 J mu per observation, cross terms of fixed cameras and
//                   tracks, and the gauge terms (anchor centre, baseline) from the scale camera's
//                   observations in the Euclidean centre chart.
// Every sum of the reduced system and of dL/d(u, v) has a fixed order; only the initial-pose cross
// terms of fixed cameras and of the gauge pair are accumulated with FP64 atomics.
#include <cuda_runtime.h>

#include "pb_kernels.h"

namespace pb {

namespace {

// Gradient gx (3) and Hessian Hm (M x M, M = 3 + ni, row-major) of lam^T pi(x_c, kappa) over the
// camera-frame point x_c and the refined intrinsic columns kappa (group chart: fx, log aspect,
// cx, cy, k1, k2, k3, p1, p2, additive; fy = fx * aspect).  Analytic: derivatives of the
// distorted normalised point (xd, yd) over (x, y) = (X / Z, Y / Z), chained through the
// perspective division; the intrinsics enter bilinearly (focal x distortion), so their own
// block is non-zero only in the focal and aspect rows.
__host__ __device__ __forceinline__ void lam_pixel_derivatives(const DCam& c, const double* xc, double lam0, double lam1, int ni,
                                                      const int* cols, double* gx, double* Hm) {
    const int M = 3 + ni;
    const double iz = 1.0 / xc[2];
    const double x = xc[0] * iz, y = xc[1] * iz;
    const double r2 = x * x + y * y;
    const double R = 1.0 + r2 * (c.k1 + r2 * (c.k2 + r2 * c.k3));
    const double R1 = c.k1 + r2 * (2.0 * c.k2 + 3.0 * c.k3 * r2);
    const double R2 = 2.0 * c.k2 + 6.0 * c.k3 * r2;
    const double p1 = c.p1, p2 = c.p2;
    const double yd = y * R + p1 * (r2 + 2.0 * y * y) + 2.0 * p2 * x * y;
    const double xd_x = R + 2.0 * x * x * R1 + 2.0 * p1 * y + 6.0 * p2 * x;
    const double xd_y = 2.0 * x * y * R1 + 2.0 * p1 * x + 2.0 * p2 * y;
    const double yd_x = xd_y;
    const double yd_y = R + 2.0 * y * y * R1 + 6.0 * p1 * y + 2.0 * p2 * x;
    const double xd_xx = 6.0 * x * R1 + 4.0 * x * x * x * R2 + 6.0 * p2;
    const double xd_xy = 2.0 * y * R1 + 4.0 * x * x * y * R2 + 2.0 * p1;
    const double xd_yy = 2.0 * x * R1 + 4.0 * x * y * y * R2 + 2.0 * p2;
    const double yd_xx = xd_xy;
    const double yd_xy = xd_yy;
    const double yd_yy = 6.0 * y * R1 + 4.0 * y * y * y * R2 + 6.0 * p1;
    const double aspect = c.fx > 0.0 ? c.fy / c.fx : 1.0;
    const double al = lam0 * c.su * c.fx, be = lam1 * c.sv * c.fy;
    const double Px = al * xd_x + be * yd_x, Py = al * xd_y + be * yd_y;
    const double Pxx = al * xd_xx + be * yd_xx, Pxy = al * xd_xy + be * yd_xy, Pyy = al * xd_yy + be * yd_yy;
    const double iz2 = iz * iz;
    gx[0] = iz * Px;
    gx[1] = iz * Py;
    gx[2] = -iz * (x * Px + y * Py);
    // J_n = iz [[1, 0, -x], [0, 1, -y]]; H = J_n^T P'' J_n + Px d2(x) + Py d2(y)
    Hm[0 * M + 0] = iz2 * Pxx;
    Hm[0 * M + 1] = Hm[1 * M + 0] = iz2 * Pxy;
    Hm[1 * M + 1] = iz2 * Pyy;
    Hm[0 * M + 2] = Hm[2 * M + 0] = -iz2 * (x * Pxx + y * Pxy + Px);
    Hm[1 * M + 2] = Hm[2 * M + 1] = -iz2 * (x * Pxy + y * Pyy + Py);
    Hm[2 * M + 2] = iz2 * (x * x * Pxx + 2.0 * x * y * Pxy + y * y * Pyy + 2.0 * (x * Px + y * Py));
    // per intrinsic column: the (x, y)-gradient (kx, ky) of d(lam^T pi)/d kappa, and for the
    // distortion columns the shape (shx, shy) = d(xd, yd)/d kappa that the focal and aspect rows
    // multiply
    double kx[kMaxNI], ky[kMaxNI], shx[kMaxNI], shy[kMaxNI];
    for (int k = 0; k < ni; ++k) {
        double dxd = 0.0, dyd = 0.0, dxd_x = 0.0, dxd_y = 0.0, dyd_x = 0.0, dyd_y = 0.0;
        switch (cols[k]) {
            case 0:  // fx (fy = fx * aspect follows)
                kx[k] = lam0 * c.su * xd_x + lam1 * c.sv * aspect * yd_x;
                ky[k] = lam0 * c.su * xd_y + lam1 * c.sv * aspect * yd_y;
                shx[k] = shy[k] = 0.0;
                continue;
            case 1:  // log aspect: d fy = fy
                kx[k] = be * yd_x;
                ky[k] = be * yd_y;
                shx[k] = shy[k] = 0.0;
                continue;
            case 4: dxd = x * r2; dyd = y * r2; dxd_x = r2 + 2.0 * x * x; dxd_y = 2.0 * x * y; dyd_x = dxd_y;
                    dyd_y = r2 + 2.0 * y * y; break;
            case 5: dxd = x * r2 * r2; dyd = y * r2 * r2; dxd_x = r2 * r2 + 4.0 * x * x * r2; dxd_y = 4.0 * x * y * r2;
                    dyd_x = dxd_y; dyd_y = r2 * r2 + 4.0 * y * y * r2; break;
            case 6: dxd = x * r2 * r2 * r2; dyd = y * r2 * r2 * r2; dxd_x = r2 * r2 * r2 + 6.0 * x * x * r2 * r2;
                    dxd_y = 6.0 * x * y * r2 * r2; dyd_x = dxd_y; dyd_y = r2 * r2 * r2 + 6.0 * y * y * r2 * r2; break;
            case 7: dxd = 2.0 * x * y; dyd = r2 + 2.0 * y * y; dxd_x = 2.0 * y; dxd_y = 2.0 * x; dyd_x = 2.0 * x;
                    dyd_y = 6.0 * y; break;
            case 8: dxd = r2 + 2.0 * x * x; dyd = 2.0 * x * y; dxd_x = 6.0 * x; dxd_y = 2.0 * y; dyd_x = 2.0 * y;
                    dyd_y = 2.0 * x; break;
            default: break;  // cx, cy: constant derivatives
        }
        kx[k] = al * dxd_x + be * dyd_x;
        ky[k] = al * dxd_y + be * dyd_y;
        shx[k] = dxd;
        shy[k] = dyd;
    }
    // intrinsic-intrinsic block: only the focal and log-aspect rows are non-zero
    for (int k = 0; k < ni; ++k)
        for (int l = k; l < ni; ++l) {
            const int ck = cols[k], cl = cols[l];
            const int a = ck < cl ? ck : cl, b = ck < cl ? cl : ck;
            const int kb = ck < cl ? l : k;  // the column of the larger index
            double h = 0.0;
            if (a == 0 && b == 1) h = lam1 * c.sv * aspect * yd;
            else if (a == 1 && b == 1) h = be * yd;
            else if (a == 0 && b >= 4) h = lam0 * c.su * shx[kb] + lam1 * c.sv * aspect * shy[kb];
            else if (a == 1 && b >= 4) h = be * shy[kb];
            Hm[(3 + k) * M + 3 + l] = Hm[(3 + l) * M + 3 + k] = h;
        }
    // point-intrinsic block: J_n^T (kx, ky)
    for (int k = 0; k < ni; ++k) {
        const double h0 = iz * kx[k], h1 = iz * ky[k], h2 = -iz * (x * kx[k] + y * ky[k]);
        Hm[0 * M + 3 + k] = Hm[(3 + k) * M + 0] = h0;
        Hm[1 * M + 3 + k] = Hm[(3 + k) * M + 1] = h1;
        Hm[2 * M + 3 + k] = Hm[(3 + k) * M + 2] = h2;
    }
}

__device__ __forceinline__ int sym6(int a, int b) { return a * 6 - a * (a - 1) / 2 + (b - a); }
__device__ __forceinline__ int sym3(int a, int b) { return a * 3 - a * (a - 1) / 2 + (b - a); }
__device__ __forceinline__ int symn(int n, int a, int b) { return a * n - a * (a - 1) / 2 + (b - a); }

__device__ __forceinline__ void cross3(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// Exact per-observation Hessian record (layout AdjLayout) in the chart of the observation's
// camera: tangent (gauge scale camera, centre columns 3 and 4 along the world basis gb) or
// Euclidean.  nvec / baseline: unit direction anchor -> scale camera and the gauge baseline.
// Returns false on an invalid projection or loss.
__device__ bool adj_obs_hessian(const DCam& c, const double* X, double s, double u, double v, double wobs, int loss,
                                double lscale, bool tangent, const double* gb, const double* nvec, double baseline,
                                int ni, const int* cols, const AdjLayout& Lo, double* rec) {
    Lin<double> L;
    if (!linearize_obs<double>(c, X[0], X[1], X[2], s, u, v, wobs, loss, lscale, tangent, false, gb, ni, cols, true, L))
        return false;
    const double r0 = L.rd0, r1 = L.rd1;
    double d1, d2;
    robust_derivatives(wobs * (r0 * r0 + r1 * r1), loss, lscale, d1, d2);
    const double wa = 2.0 * d1 * wobs, wb = 4.0 * d2 * wobs * wobs;
    const double W00 = wa + wb * r0 * r0, W01 = wb * r0 * r1, W11 = wa + wb * r1 * r1;
    const double lam0 = wa * r0, lam1 = wa * r1;
    // world displacement d = X - C and the camera-frame point x_c = C2W^T d
    const double d[3] = {X[0] - c.C[0], X[1] - c.C[1], X[2] - c.C[2]};
    double xc[3];
    for (int m = 0; m < 3; ++m) xc[m] = c.R[m] * d[0] + c.R[3 + m] * d[1] + c.R[6 + m] * d[2];
    // second derivatives of lam^T pi over (x_c, kappa)
    const int M = 3 + ni;
    double gx[3];
    double Hm[(3 + kMaxNI) * (3 + kMaxNI)];
    lam_pixel_derivatives(c, xc, lam0, lam1, ni, cols, gx, Hm);
    // camera-frame point Jacobian over (w0..2, centre 0..2, dX 0..2), columns of Jx[m][col]
    const double sg[3] = {1.0, -1.0, -1.0};
    double Jx[3][9];
    for (int i = 0; i < 3; ++i) {
        const double e[3] = {i == 0 ? 1.0 : 0.0, i == 1 ? 1.0 : 0.0, i == 2 ? 1.0 : 0.0};
        double a[3];
        cross3(e, d, a);
        for (int m = 0; m < 3; ++m) {
            Jx[m][i] = sg[i] * (c.R[m] * a[0] + c.R[3 + m] * a[1] + c.R[6 + m] * a[2]);
            Jx[m][6 + i] = s * c.R[3 * i + m];
            if (tangent)
                Jx[m][3 + i] = i < 2 ? -(c.R[m] * gb[3 * i] + c.R[3 + m] * gb[3 * i + 1] + c.R[6 + m] * gb[3 * i + 2]) : 0.0;
            else
                Jx[m][3 + i] = -c.R[3 * i + m];
        }
    }
    // g_w = C2W g_x: gradient of lam^T pi w.r.t. the world displacement d
    double gw[3];
    for (int j = 0; j < 3; ++j) gw[j] = c.R[3 * j] * gx[0] + c.R[3 * j + 1] * gx[1] + c.R[3 * j + 2] * gx[2];
    const double gd = gw[0] * d[0] + gw[1] * d[1] + gw[2] * d[2];
    // T: lam^T (d pi / d x_c) d2 x_c over the pose and point columns (upper 9x9)
    double T[9][9];
    for (int a = 0; a < 9; ++a)
        for (int b = 0; b < 9; ++b) T[a][b] = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j)  // d2 E / dw_i dw_j = G_i G_j (i <= j, product order Rx Ry Rz)
            T[i][j] = sg[i] * sg[j] * (gw[j] * d[i] - (i == j ? gd : 0.0));
    for (int i = 0; i < 3; ++i) {
        const double e[3] = {i == 0 ? 1.0 : 0.0, i == 1 ? 1.0 : 0.0, i == 2 ? 1.0 : 0.0};
        double ge[3];  // g_w x e_i, so that g_w . (e_i x b) = b . (g_w x e_i)
        cross3(gw, e, ge);
        for (int k = 0; k < 3; ++k) {
            T[i][6 + k] = s * sg[i] * ge[k];
            if (tangent)
                T[i][3 + k] = k < 2 ? -sg[i] * (ge[0] * gb[3 * k] + ge[1] * gb[3 * k + 1] + ge[2] * gb[3 * k + 2]) : 0.0;
            else
                T[i][3 + k] = -sg[i] * ge[k];
        }
    }
    if (tangent) {
        const double tt = (gw[0] * nvec[0] + gw[1] * nvec[1] + gw[2] * nvec[2]) / baseline;
        T[3][3] = tt;
        T[4][4] = tt;
    }
    // full local Jacobian rows and W2 J
    const int nl = 9 + ni;
    double Jf[2][9 + kMaxNI], WJ[2][9 + kMaxNI];
    for (int r = 0; r < 2; ++r) {
        for (int a = 0; a < 6; ++a) Jf[r][a] = L.Jc[r * 6 + a];
        for (int a = 0; a < 3; ++a) Jf[r][6 + a] = L.Jp[r * 3 + a];
        for (int k = 0; k < ni; ++k) Jf[r][9 + k] = L.Ji[r * kMaxNI + k];
    }
    for (int a = 0; a < nl; ++a) {
        WJ[0][a] = W00 * Jf[0][a] + W01 * Jf[1][a];
        WJ[1][a] = W01 * Jf[0][a] + W11 * Jf[1][a];
    }
    // HJ = Hxx Jx (3 x 9)
    double HJ[3][9];
    for (int m = 0; m < 3; ++m)
        for (int a = 0; a < 9; ++a)
            HJ[m][a] = Hm[m * M + 0] * Jx[0][a] + Hm[m * M + 1] * Jx[1][a] + Hm[m * M + 2] * Jx[2][a];
    auto h99 = [&](int a, int b) {  // a <= b < 9
        return Jf[0][a] * WJ[0][b] + Jf[1][a] * WJ[1][b] + Jx[0][a] * HJ[0][b] + Jx[1][a] * HJ[1][b] +
               Jx[2][a] * HJ[2][b] + T[a][b];
    };
    double* hcc = rec + Lo.hcc();
    double* hcp = rec + Lo.hcp();
    double* hpp = rec + Lo.hpp();
    double* hck = rec + Lo.hck();
    double* hpk = rec + Lo.hpk();
    double* hkk = rec + Lo.hkk();
    for (int a = 0; a < 6; ++a)
        for (int b = a; b < 6; ++b) hcc[sym6(a, b)] = h99(a, b);
    for (int a = 0; a < 6; ++a)
        for (int b = 0; b < 3; ++b) hcp[a * 3 + b] = h99(a, 6 + b);
    for (int a = 0; a < 3; ++a)
        for (int b = a; b < 3; ++b) hpp[sym3(a, b)] = h99(6 + a, 6 + b);
    for (int k = 0; k < ni; ++k) {
        for (int a = 0; a < 9; ++a) {
            const double h = Jf[0][a] * WJ[0][9 + k] + Jf[1][a] * WJ[1][9 + k] + Jx[0][a] * Hm[0 * M + 3 + k] +
                             Jx[1][a] * Hm[1 * M + 3 + k] + Jx[2][a] * Hm[2 * M + 3 + k];
            if (a < 6) hck[a * ni + k] = h;
            else hpk[(a - 6) * ni + k] = h;
        }
        for (int l = k; l < ni; ++l)
            hkk[symn(ni, k, l)] = Jf[0][9 + k] * WJ[0][9 + l] + Jf[1][9 + k] * WJ[1][9 + l] + Hm[(3 + k) * M + 3 + l];
    }
    double* J = rec + Lo.jac();
    for (int r = 0; r < 2; ++r)
        for (int a = 0; a < nl; ++a) J[r * nl + a] = Jf[r][a];
    double* w2 = rec + Lo.w2();
    w2[0] = W00;
    w2[1] = W01;
    w2[2] = W11;
    w2[3] = lam0;
    w2[4] = lam1;
    return true;
}

__device__ __forceinline__ bool is_tangent(const Shape& S, int cam) {
    return cam == S.gauge_scale && S.gauge_anchor >= 0 && S.gauge_baseline > 0.0;
}

// unit vector anchor -> scale camera (world) at the current state
__device__ __forceinline__ void gauge_normal(const Shape& S, const DevPtrs& D, double* n) {
    n[0] = n[1] = n[2] = 0.0;
    if (S.gauge_scale < 0 || S.gauge_anchor < 0) return;
    const double* cs = D.cams_state + static_cast<size_t>(S.gauge_scale) * kCamStride + 9;
    const double* ca = D.cams_state + static_cast<size_t>(S.gauge_anchor) * kCamStride + 9;
    double e[3] = {cs[0] - ca[0], cs[1] - ca[1], cs[2] - ca[2]};
    const double l = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    if (l > 0.0)
        for (int i = 0; i < 3; ++i) n[i] = e[i] / l;
}

__global__ void __launch_bounds__(128) k_adj_hessian(Shape S, DevPtrs D, AdjBuffers B) {
    const long long o = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (o >= S.nop) return;
    const int cam = D.obs_cam[o], trk = D.obs_trk[o];
    DCam c;
    load_cam(D.cams_eff + static_cast<size_t>(cam) * kCamStride, c);
    const bool tangent = is_tangent(S, cam);
    double n[3];
    gauge_normal(S, D, n);
    double* rec = B.rec + static_cast<size_t>(o) * B.lay.stride;
    if (!adj_obs_hessian(c, D.points + static_cast<size_t>(trk) * 3, D.pscale[trk], D.obs_u[o], D.obs_v[o], D.obs_w[o],
                         S.loss, S.loss_scale, tangent, D.gauge_basis, n, S.gauge_baseline, S.ni, S.int_cols, B.lay,
                         rec)) {
        for (int i = 0; i < B.lay.stride; ++i) rec[i] = 0.0;
        atomicOr(B.flags, 2);
    }
}

// dL/dz of the primary variables added to the reduced right-hand side (which holds the point
// terms after the reduction).  One thread per camera, then one per intrinsic column.
__global__ void k_adj_rhs(Shape S, DevPtrs D, AdjBuffers B, double* __restrict__ rhs) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < S.nc) {
        const int b = D.cam_block[t];
        if (b < 0) return;
        const double* g = B.gcam + static_cast<size_t>(t) * 6;
        double* r = rhs + 6 * b;
        r[0] += g[0];
        r[1] += g[1];
        r[2] += g[2];
        if (is_tangent(S, t)) {
            const double* gb = D.gauge_basis;
            r[3] += g[3] * gb[0] + g[4] * gb[1] + g[5] * gb[2];
            r[4] += g[3] * gb[3] + g[4] * gb[4] + g[5] * gb[5];
        } else {
            r[3] += g[3];
            r[4] += g[4];
            r[5] += g[5];
        }
        return;
    }
    const int q = t - S.nc;
    if (q < S.nb) {
        const int g = q / S.ni, k = q - g * S.ni;
        rhs[6 * S.ncb + q] += B.gint[static_cast<size_t>(g) * kP + S.int_cols[k]];
    }
}

__device__ __forceinline__ int csr_find(const DevPtrs& D, int row, int col) {
    int lo = D.row_ptr[row], hi = D.row_ptr[row + 1] - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int v = D.col_idx[mid];
        if (v == col) return mid;
        if (v < col) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// full 3x3 inverse of a symmetric matrix given by its upper triangle; false when singular
// relative to its scale
__device__ __forceinline__ bool sym3_inverse(const double* u, double* inv) {
    const double a = u[0], b = u[1], c = u[2], d = u[3], e = u[4], f = u[5];
    const double A = d * f - e * e, Bc = c * e - b * f, Cc = b * e - c * d;
    const double det = a * A + b * Bc + c * Cc;
    const double scale = fabs(a) * fabs(d) * fabs(f) + 1e-300;
    if (!(fabs(det) > 1e-14 * scale) || !isfinite(det)) return false;
    const double id = 1.0 / det;
    inv[0] = A * id;
    inv[1] = Bc * id;
    inv[2] = Cc * id;
    inv[3] = Bc * id;
    inv[4] = (a * f - c * c) * id;
    inv[5] = (b * c - a * e) * id;
    inv[6] = Cc * id;
    inv[7] = (b * c - a * e) * id;
    inv[8] = (a * d - b * b) * id;
    return true;
}

// Right-hand side of a track's point block: s(X) dL/dX (backward pass), or in Newton mode the
// descent direction -grad F = -sum_o Jp_o^T lam_o over its observations (point chart).
__device__ __forceinline__ void track_rhs(const Shape& S, const DevPtrs& D, const AdjBuffers& B, int trk, double* bp) {
    if (B.newton) {
        bp[0] = bp[1] = bp[2] = 0.0;
        const int nl = 9 + S.ni;
        for (int o = D.trk_obs_begin[trk]; o < D.trk_obs_begin[trk + 1]; ++o) {
            const double* rec = B.rec + static_cast<size_t>(o) * B.lay.stride;
            const double* J = rec + B.lay.jac();
            const double l0 = rec[B.lay.w2() + 3], l1 = rec[B.lay.w2() + 4];
            for (int i = 0; i < 3; ++i) bp[i] -= J[6 + i] * l0 + J[nl + 6 + i] * l1;
        }
        return;
    }
    const double sp = D.pscale[trk];
    for (int i = 0; i < 3; ++i) bp[i] = sp * B.gpt[static_cast<size_t>(trk) * 3 + i];
}

constexpr int kAdjThreads = 256;

template <typename U>
__device__ __forceinline__ U* carve(char*& ptr, size_t count) {
    U* out = reinterpret_cast<U*>(ptr);
    ptr += (count * sizeof(U) + 15) & ~static_cast<size_t>(15);
    return out;
}

// Point elimination of the exact Hessian over the forward path's chunk plan: one CTA per chunk
// of consecutive tracks, every output element owned by one thread that sums its terms over the
// host-built item lists in a fixed order (deterministic, no atomics), written as FP64 chunk
// partials in the layout of the forward assembly and summed by the forward reduce kernels:
//   pose block (a, b):  sum_o H_cc(o) (own items)  -  sum_(oa, ob) Y_oa W_ob^T,  Y = W V^-1
//   border (c, g):      sum_(o in c, g) H_ck(o)  -  sum_(o in c) Y_o K_(t(o), g)
//   intrinsic (g, g'):  sum_(o in g) H_kk(o)  -  sum_t K_(t,g)^T V_t^-1 K_(t,g')
//   rhs:                -sum_(o in c) Y_o b_t  and  -sum_t K_(t,g)^T V_t^-1 b_t
// with W = H_cp (pose-point), K_(t,g) = sum over the track's observations of group g of H_pk,
// V_t = sum H_pp and b_t = s(X) dL/dX of the track.
__global__ void __launch_bounds__(kAdjThreads, 2)
    k_adj_assemble(Shape S, DevPtrs D, AdjBuffers B, double* __restrict__ part_pair, double* __restrict__ part_cam,
                   double* __restrict__ part_chunk) {
    extern __shared__ __align__(16) char smem[];
    const AdjLayout& Lo = B.lay;
    const int chunk = blockIdx.x, tid = threadIdx.x;
    const int MO = S.max_obs, MT = S.max_tracks;
    const int ng = S.ng, ni = S.ni, nb = S.nb;
    char* ptr = smem;
    double* s_W = carve<double>(ptr, static_cast<size_t>(MO) * 18);     // H_cp per observation
    double* s_Vi = carve<double>(ptr, static_cast<size_t>(MT) * 12);    // V^-1 (9) and q = V^-1 b (3) per track
    double* s_K = carve<double>(ptr, static_cast<size_t>(MT) * nb * 3);  // K[(t, g*ni + c), j]
    int* s_info = carve<int>(ptr, MO);                                  // group + 1 | elim << 4 | slot << 8
    int* s_tfirst = carve<int>(ptr, MT + 1);
    int* s_flag = carve<int>(ptr, 1);
    const int obs0 = D.ch_obs_begin[chunk], nobs = D.ch_obs_begin[chunk + 1] - obs0;
    const int trk0 = D.obs_trk[obs0];
    const int ntc = D.obs_trk[obs0 + nobs - 1] - trk0 + 1;
    if (tid == 0) s_flag[0] = ntc > MT ? 1 : 0;
    __syncthreads();
    if (s_flag[0]) {
        if (tid == 0) atomicOr(B.flags, 4);
        return;
    }
    // per observation: H_cp into shared memory, group / elimination / track slot
    if (tid < nobs) {
        const int o = obs0 + tid;
        const double* rec = B.rec + static_cast<size_t>(o) * Lo.stride + Lo.hcp();
        for (int i = 0; i < 18; ++i) s_W[tid * 18 + i] = rec[i];
        const int cam = D.obs_cam[o], trk = D.obs_trk[o];
        const int g = ng > 0 ? D.cam_group[cam] : -1;
        const int elim = D.trk_block[trk] >= 0 ? 1 : 0;
        const int slot = trk - trk0;
        s_info[tid] = (g + 1) | (elim << 4) | (slot << 8);
        if (o == D.trk_obs_begin[trk]) s_tfirst[slot] = tid;
    }
    if (tid == 0) s_tfirst[ntc] = nobs;
    __syncthreads();
    // per track: V^-1 and q (FP64), also kept for the gradient kernel
    if (tid < ntc) {
        const int trk = trk0 + tid;
        double Vi[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, q[3] = {0, 0, 0};
        if (D.trk_block[trk] >= 0) {
            double V[6] = {0, 0, 0, 0, 0, 0};
            for (int o = D.trk_obs_begin[trk]; o < D.trk_obs_begin[trk + 1]; ++o) {
                const double* h = B.rec + static_cast<size_t>(o) * Lo.stride + Lo.hpp();
                for (int i = 0; i < 6; ++i) V[i] += h[i];
            }
            if (!sym3_inverse(V, Vi)) {
                atomicOr(B.flags, 1);
                for (int i = 0; i < 9; ++i) Vi[i] = 0.0;
            }
            double bp[3];
            track_rhs(S, D, B, trk, bp);
            for (int i = 0; i < 3; ++i) q[i] = Vi[i * 3] * bp[0] + Vi[i * 3 + 1] * bp[1] + Vi[i * 3 + 2] * bp[2];
        }
        for (int i = 0; i < 9; ++i) {
            s_Vi[tid * 12 + i] = Vi[i];
            B.vinv[static_cast<size_t>(trk) * 9 + i] = Vi[i];
        }
        for (int i = 0; i < 3; ++i) s_Vi[tid * 12 + 9 + i] = q[i];
    }
    // per track and group: K = sum of H_pk over the track's observations of the group
    if (nb > 0) {
        const int per = nb * 3;
        for (int it = tid; it < ntc * per; it += blockDim.x) {
            const int t = it / per, r = it - t * per;
            const int gc = r / 3, j = r - gc * 3;
            const int g = gc / ni, c = gc - g * ni;
            double acc = 0.0;
            for (int ob = s_tfirst[t]; ob < s_tfirst[t + 1]; ++ob) {
                if ((s_info[ob] & 15) - 1 != g) continue;
                acc += B.rec[static_cast<size_t>(obs0 + ob) * Lo.stride + Lo.hpk() + j * ni + c];
            }
            s_K[it] = acc;
        }
    }
    __syncthreads();
    // owner gathers
    const int pair0 = D.ch_pair_begin[chunk], npairs = D.ch_pair_begin[chunk + 1] - pair0;
    const int cam0 = D.ch_cam_begin[chunk], ncams = D.ch_cam_begin[chunk + 1] - cam0;
    const int camrec = 12 + ng * 6 * ni;
    const int crow = 2 + ng * ni;
    const int chrec = nb * nb + 2 * nb;
    const int w_pair = npairs * 6, w_cam = ncams * crow;
    const int w_total = w_pair + w_cam + chrec;
    // row x of Y_o = W_o V_t^-1
    auto yrow = [&](int ob, int x, double* y) {
        const int info = s_info[ob];
        if (!((info >> 4) & 1)) {
            y[0] = y[1] = y[2] = 0.0;
            return;
        }
        const double* Vi = s_Vi + (info >> 8) * 12;
        const double* w = s_W + ob * 18 + 3 * x;
        for (int j = 0; j < 3; ++j) y[j] = w[0] * Vi[j] + w[1] * Vi[3 + j] + w[2] * Vi[6 + j];
    };
    for (int wk = tid; wk < w_total; wk += blockDim.x) {
        if (wk < w_pair) {
            const int sl = wk / 6, x = wk - sl * 6;
            const int pk = D.ch_pairs[pair0 + sl];
            const bool diag = (pk & 0xFFFF) == (pk >> 16);
            double acc[6] = {0, 0, 0, 0, 0, 0};
            const int i1 = D.slot_item_begin[pair0 + sl + 1];
            for (int it = D.slot_item_begin[pair0 + sl]; it < i1; ++it) {
                const unsigned item = D.slot_items[it];
                const int oa = item & 0xFF, ob = item >> 8;
                double y[3];
                yrow(oa, x, y);
                const double* wb = s_W + ob * 18;
                if (oa == ob) {
                    const double* h = B.rec + static_cast<size_t>(obs0 + oa) * Lo.stride + Lo.hcc();
                    for (int q2 = 0; q2 < 6; ++q2) acc[q2] += h[x <= q2 ? sym6(x, q2) : sym6(q2, x)];
                }
                for (int q2 = 0; q2 < 6; ++q2) acc[q2] -= y[0] * wb[3 * q2] + y[1] * wb[3 * q2 + 1] + y[2] * wb[3 * q2 + 2];
            }
            double* out = part_pair + static_cast<size_t>(pair0 + sl) * 36;
            for (int q2 = 0; q2 < 6; ++q2) {
                if (!diag) {
                    out[x * 6 + q2] = acc[q2];
                } else if (q2 >= x) {
                    out[x * 6 + q2] = acc[q2];
                    out[q2 * 6 + x] = acc[q2];
                }
            }
        } else if (wk < w_pair + w_cam) {
            const int r = wk - w_pair;
            const int l = r / crow, row = r - l * crow;
            const int b0 = D.lcam_obs_begin[cam0 + l], b1 = D.lcam_obs_begin[cam0 + l + 1];
            double* out = part_cam + static_cast<size_t>(cam0 + l) * camrec;
            double acc[6] = {0, 0, 0, 0, 0, 0};
            if (row == 0) {
                // reduced right-hand side: -Y_o b_t = -W_o q_t, and in Newton mode the camera's
                // own descent direction -J_c^T lam
                for (int it = b0; it < b1; ++it) {
                    const int ob = D.lcam_obs[it];
                    const int info = s_info[ob];
                    if (B.newton) {
                        const double* rec = B.rec + static_cast<size_t>(obs0 + ob) * Lo.stride;
                        const double* J = rec + Lo.jac();
                        const double l0 = rec[Lo.w2() + 3], l1 = rec[Lo.w2() + 4];
                        for (int a = 0; a < 6; ++a) acc[a] -= J[a] * l0 + J[9 + ni + a] * l1;
                    }
                    if (!((info >> 4) & 1)) continue;
                    const double* q = s_Vi + (info >> 8) * 12 + 9;
                    const double* w = s_W + ob * 18;
                    for (int a = 0; a < 6; ++a) acc[a] -= w[3 * a] * q[0] + w[3 * a + 1] * q[1] + w[3 * a + 2] * q[2];
                }
                for (int a = 0; a < 6; ++a) out[a] = acc[a];
            } else if (row == 1) {
                for (int a = 0; a < 6; ++a) out[6 + a] = 0.0;
            } else {
                const int gc = row - 2, g = gc / ni, c2 = gc - g * ni;
                for (int it = b0; it < b1; ++it) {
                    const int ob = D.lcam_obs[it];
                    const int info = s_info[ob];
                    if ((info & 15) - 1 == g) {
                        const double* h = B.rec + static_cast<size_t>(obs0 + ob) * Lo.stride + Lo.hck();
                        for (int a = 0; a < 6; ++a) acc[a] += h[a * ni + c2];
                    }
                    if ((info >> 4) & 1) {
                        const double* Kt = s_K + (static_cast<size_t>(info >> 8) * nb + gc) * 3;
                        for (int a = 0; a < 6; ++a) {
                            double y[3];
                            yrow(ob, a, y);
                            acc[a] -= y[0] * Kt[0] + y[1] * Kt[1] + y[2] * Kt[2];
                        }
                    }
                }
                for (int a = 0; a < 6; ++a) out[12 + (g * 6 + a) * ni + c2] = acc[a];
            }
        } else {
            const int e = wk - w_pair - w_cam;
            double* out = part_chunk + static_cast<size_t>(chunk) * chrec;
            double acc = 0.0;
            if (e < nb * nb) {
                const int i = e / nb, j = e - i * nb;
                if (i > j) continue;
                const int g1 = i / ni, c1 = i - g1 * ni, g2 = j / ni, c2 = j - g2 * ni;
                if (g1 == g2)
                    for (int ob = 0; ob < nobs; ++ob) {
                        if ((s_info[ob] & 15) - 1 != g1) continue;
                        const double* h = B.rec + static_cast<size_t>(obs0 + ob) * Lo.stride + Lo.hkk();
                        acc += h[c1 <= c2 ? symn(ni, c1, c2) : symn(ni, c2, c1)];
                    }
                for (int t = 0; t < ntc; ++t) {
                    if (!((s_info[s_tfirst[t]] >> 4) & 1)) continue;
                    const double* K1 = s_K + (static_cast<size_t>(t) * nb + i) * 3;
                    const double* K2 = s_K + (static_cast<size_t>(t) * nb + j) * 3;
                    const double* Vi = s_Vi + t * 12;
                    for (int r = 0; r < 3; ++r)
                        acc -= K1[r] * (Vi[r * 3] * K2[0] + Vi[r * 3 + 1] * K2[1] + Vi[r * 3 + 2] * K2[2]);
                }
                out[e] = acc;
                if (i != j) out[j * nb + i] = acc;
            } else if (e < nb * nb + nb) {
                const int col = e - nb * nb;
                if (B.newton) {
                    const int g = col / ni, c = col - g * ni;
                    for (int ob = 0; ob < nobs; ++ob) {
                        if ((s_info[ob] & 15) - 1 != g) continue;
                        const double* rec = B.rec + static_cast<size_t>(obs0 + ob) * Lo.stride;
                        const double* J = rec + Lo.jac();
                        acc -= J[9 + c] * rec[Lo.w2() + 3] + J[9 + ni + 9 + c] * rec[Lo.w2() + 4];
                    }
                }
                for (int t = 0; t < ntc; ++t) {
                    if (!((s_info[s_tfirst[t]] >> 4) & 1)) continue;
                    const double* K1 = s_K + (static_cast<size_t>(t) * nb + col) * 3;
                    const double* q = s_Vi + t * 12 + 9;
                    acc -= K1[0] * q[0] + K1[1] * q[1] + K1[2] * q[2];
                }
                out[e] = acc;
            } else {
                out[e] = 0.0;
            }
        }
    }
}

// Priors on the intrinsic diagonal (0.5 (invSigma (theta - prior))^2 has Hessian invSigma^2) and
// structurally empty diagonals set to 1 (their right-hand side is zero).
__global__ void k_adj_finalize(Shape S, DevPtrs D, RedOut<double> R, int newton) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nd = 6 * S.ncb;
    if (t < nd) {
        const int b = t / 6, a = t - b * 6;
        double* d = R.vals + static_cast<size_t>(D.diag_pos[b]) * 36 + a * 7;
        if (*d == 0.0) *d = 1.0;
    } else if (t < nd + S.nb) {
        const int q = t - nd, g = q / S.ni, k = q - g * S.ni;
        const double* G = D.groups + static_cast<size_t>(g) * kGroupRec;
        const int p = S.int_cols[k];
        const double w = G[2 * kP + p];
        double* d = R.Cm + static_cast<size_t>(q) * S.nb + q;
        const double v = *d + w * w;
        *d = v != 0.0 ? v : 1.0;
        if (newton) R.rhs[nd + q] -= w * w * (G[p] - G[kP + p]);
    }
}

__global__ void __launch_bounds__(128) k_adj_gradient(Shape S, DevPtrs D, AdjBuffers B, const double* __restrict__ mu) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.ntp) return;
    const AdjLayout& Lo = B.lay;
    const int ni = S.ni, nl = 9 + ni;
    const int ob = D.trk_obs_begin[t], oe = D.trk_obs_begin[t + 1];
    const bool free_pt = D.trk_block[t] >= 0;
    const double* mk_base = mu + 6 * S.ncb;
    // point part of mu: V^-1 (b_p - sum_o (Hcp^T mu_c + Hpk mu_k))
    double mp[3] = {0.0, 0.0, 0.0};
    if (free_pt) {
        double acc[3];
        track_rhs(S, D, B, t, acc);
        for (int o = ob; o < oe; ++o) {
            const double* rec = B.rec + static_cast<size_t>(o) * Lo.stride;
            const int cam = D.obs_cam[o];
            const int b = D.cam_block[cam], g = S.ng > 0 ? D.cam_group[cam] : -1;
            if (b >= 0) {
                const double* mc = mu + 6 * b;
                const double* h = rec + Lo.hcp();
                for (int a = 0; a < 6; ++a)
                    for (int i = 0; i < 3; ++i) acc[i] -= h[a * 3 + i] * mc[a];
            }
            if (g >= 0) {
                const double* h = rec + Lo.hpk();
                for (int i = 0; i < 3; ++i)
                    for (int k = 0; k < ni; ++k) acc[i] -= h[i * ni + k] * mk_base[g * ni + k];
            }
        }
        const double* Vi = B.vinv + static_cast<size_t>(t) * 9;
        for (int i = 0; i < 3; ++i) mp[i] = Vi[i * 3] * acc[0] + Vi[i * 3 + 1] * acc[1] + Vi[i * 3 + 2] * acc[2];
        for (int i = 0; i < 3; ++i) B.mu_p[static_cast<size_t>(t) * 3 + i] = mp[i];
    }
    double fixed_pt[3] = {0.0, 0.0, 0.0};
    for (int o = ob; o < oe; ++o) {
        const double* rec = B.rec + static_cast<size_t>(o) * Lo.stride;
        const int cam = D.obs_cam[o];
        const int b = D.cam_block[cam], g = S.ng > 0 ? D.cam_group[cam] : -1;
        double mloc[9 + kMaxNI];  // mu over the observation's local variables
        for (int a = 0; a < 6; ++a) mloc[a] = b >= 0 ? mu[6 * b + a] : 0.0;
        for (int i = 0; i < 3; ++i) mloc[6 + i] = mp[i];
        for (int k = 0; k < ni; ++k) mloc[9 + k] = g >= 0 ? mk_base[g * ni + k] : 0.0;
        const double* J = rec + Lo.jac();
        double j0 = 0.0, j1 = 0.0;
        for (int a = 0; a < nl; ++a) {
            j0 += J[a] * mloc[a];
            j1 += J[nl + a] * mloc[a];
        }
        const double* w2 = rec + Lo.w2();
        B.grad_obs[2 * static_cast<size_t>(o)] = w2[0] * j0 + w2[1] * j1;
        B.grad_obs[2 * static_cast<size_t>(o) + 1] = w2[1] * j0 + w2[2] * j1;
        if (b < 0) {
            // fixed camera: -(H_c,pt mu_p + H_c,k mu_k)
            const double* hcp = rec + Lo.hcp();
            const double* hck = rec + Lo.hck();
            for (int a = 0; a < 6; ++a) {
                double v = hcp[a * 3] * mp[0] + hcp[a * 3 + 1] * mp[1] + hcp[a * 3 + 2] * mp[2];
                for (int k = 0; k < ni; ++k) v += hck[a * ni + k] * mloc[9 + k];
                if (v != 0.0) atomicAdd(B.grad_fixed_cam + static_cast<size_t>(cam) * 6 + a, -v);
            }
        }
        if (!free_pt) {
            // fixed track: -(H_pt,c mu_c + H_pt,k mu_k) in the scaled point chart
            const double* hcp = rec + Lo.hcp();
            const double* hpk = rec + Lo.hpk();
            for (int i = 0; i < 3; ++i) {
                double v = 0.0;
                for (int a = 0; a < 6; ++a) v += hcp[a * 3 + i] * mloc[a];
                for (int k = 0; k < ni; ++k) v += hpk[i * ni + k] * mloc[9 + k];
                fixed_pt[i] -= v;
            }
        }
        if (is_tangent(S, cam) && b >= 0) {
            // gauge terms: the scale camera's observation in the Euclidean centre chart, with mu
            // lifted to it (centre step = tangent basis * mu_t)
            double frec[kAdjMaxStride];
            DCam c;
            load_cam(D.cams_eff + static_cast<size_t>(cam) * kCamStride, c);
            double n[3];
            gauge_normal(S, D, n);
            if (!adj_obs_hessian(c, D.points + static_cast<size_t>(t) * 3, D.pscale[t], D.obs_u[o], D.obs_v[o], D.obs_w[o],
                                 S.loss, S.loss_scale, false, D.gauge_basis, n, S.gauge_baseline, ni, S.int_cols, Lo,
                                 frec)) {
                atomicOr(B.flags, 2);
                continue;
            }
            const double* gb = D.gauge_basis;
            double ml[9 + kMaxNI];
            for (int i = 0; i < 3; ++i) ml[i] = mloc[i];
            for (int i = 0; i < 3; ++i) ml[3 + i] = gb[i] * mloc[3] + gb[3 + i] * mloc[4];
            for (int i = 0; i < 3 + ni; ++i) ml[6 + i] = mloc[6 + i];
            // hC = H[C rows, all] * ml
            const double* hcc = frec + Lo.hcc();
            const double* hcp = frec + Lo.hcp();
            const double* hck = frec + Lo.hck();
            double hC[3];
            for (int i = 0; i < 3; ++i) {
                const int r = 3 + i;
                double v = 0.0;
                for (int a = 0; a < 6; ++a) v += hcc[r <= a ? sym6(r, a) : sym6(a, r)] * ml[a];
                for (int j = 0; j < 3; ++j) v += hcp[r * 3 + j] * ml[6 + j];
                for (int k = 0; k < ni; ++k) v += hck[r * ni + k] * ml[9 + k];
                hC[i] = v;
            }
            // gC = d phi / dC = lam^T J_C
            const double* fJ = frec + Lo.jac();
            const double* fw = frec + Lo.w2();
            double gC[3];
            for (int i = 0; i < 3; ++i) gC[i] = fw[3] * fJ[3 + i] + fw[4] * fJ[nl + 3 + i];
            const double gt = gC[0] * ml[3] + gC[1] * ml[4] + gC[2] * ml[5];
            for (int i = 0; i < 3; ++i) atomicAdd(B.gauge + i, -hC[i]);
            atomicAdd(B.gauge + 3, -(n[0] * hC[0] + n[1] * hC[1] + n[2] * hC[2]) - gt / S.gauge_baseline);
        }
    }
    if (!free_pt) {
        const double s = D.pscale[t];
        for (int i = 0; i < 3; ++i) B.grad_fixed_pt[static_cast<size_t>(t) * 3 + i] = fixed_pt[i] / s;
    }
}

}  // namespace

void launch_adjoint_hessian(const Shape& S, const DevPtrs& D, const AdjBuffers& B, cudaStream_t st) {
    if (S.nop <= 0) return;
    k_adj_hessian<<<static_cast<unsigned>((S.nop + 127) / 128), 128, 0, st>>>(S, D, B);
}

void launch_adjoint_rhs(const Shape& S, const DevPtrs& D, const AdjBuffers& B, const RedOut<double>& R, cudaStream_t st) {
    const int n = S.nc + S.nb;
    k_adj_rhs<<<(n + 127) / 128, 128, 0, st>>>(S, D, B, R.rhs);
}

size_t adjoint_assemble_smem(const Shape& S) {
    const auto up = [](size_t b) { return (b + 15) & ~static_cast<size_t>(15); };
    return up(static_cast<size_t>(S.max_obs) * 18 * sizeof(double)) + up(static_cast<size_t>(S.max_tracks) * 12 * sizeof(double)) +
           up(static_cast<size_t>(S.max_tracks) * S.nb * 3 * sizeof(double)) + up(static_cast<size_t>(S.max_obs) * sizeof(int)) +
           up(static_cast<size_t>(S.max_tracks + 1) * sizeof(int)) + up(sizeof(int));
}

void launch_adjoint_schur(const Shape& S, const DevPtrs& D, const AdjBuffers& B, const AsmOut& part,
                          const RedOut<double>& R, cudaStream_t st) {
    if (S.nchunks > 0) {
        const size_t smem = adjoint_assemble_smem(S);
        cudaFuncSetAttribute(k_adj_assemble, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        k_adj_assemble<<<S.nchunks, kAdjThreads, smem, st>>>(S, D, B, static_cast<double*>(part.part_pair_v),
                                                              static_cast<double*>(part.part_cam_v),
                                                              static_cast<double*>(part.part_chunk_v));
    }
    launch_reduce_sums64(S, D, part, R, st);
    const int n = 6 * S.ncb + S.nb;
    k_adj_finalize<<<(n + 127) / 128, 128, 0, st>>>(S, D, R, B.newton);
}

void launch_adjoint_gradient(const Shape& S, const DevPtrs& D, const AdjBuffers& B, const double* mu, cudaStream_t st) {
    if (S.ntp <= 0) return;
    k_adj_gradient<<<(S.ntp + 127) / 128, 128, 0, st>>>(S, D, B, mu);
}

}  // namespace pb
