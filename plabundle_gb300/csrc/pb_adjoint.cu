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
//                   curvature lam^T d2 pi: second derivatives of the projection over the camera-
//                   frame point and the intrinsics by hyper-dual numbers (exact), composed with
//                   the analytic second derivatives of the camera-frame point in the chart
//                   (rotation generators, gauge sphere); writes one record per observation.
//   k_adj_rhs       dL/dz of the primary variables into the reduced right-hand side.
//   k_adj_schur     one thread per track: point blocks V = sum H_pp, V^-1 (FP64), and the
//                   eliminated terms -W V^-1 W^T scattered into the reduced system of the forward
//                   path (pose CSR blocks, border, intrinsic block) with FP64 atomics; intrinsic
//                   terms are first summed in shared memory per thread block.
//   k_adj_finalize  priors (invSigma^2), empty diagonals, border transpose.
//   (the reduced system is then solved by the forward path's dense Cholesky-preconditioned CG
//    or block-Jacobi PCG)
//   k_adj_gradient  one thread per track: point back-substitution mu_p = V^-1 (b_p - W^T mu_c),
//                   dL/d(u, v) = W2 J mu per observation, cross terms of fixed cameras and
//                   tracks, and the gauge terms (anchor centre, baseline) from the scale camera's
//                   observations in the Euclidean centre chart.
// The FP64 atomics make the reduced sums' order (and their last bits) vary from run to run.
#include <cuda_runtime.h>

#include "pb_kernels.h"

namespace pb {

namespace {

// ---------------------------------------------------------------- hyper-dual numbers
// v + a e1 + b e2 + ab e1 e2 with e1^2 = e2^2 = 0: one evaluation gives f, df/dx_i, df/dx_j and
// d2f/dx_i dx_j exactly.
struct HD {
    double v, a, b, ab;
};
__device__ __forceinline__ HD hd(double x) { return {x, 0.0, 0.0, 0.0}; }
__device__ __forceinline__ HD operator+(HD x, HD y) { return {x.v + y.v, x.a + y.a, x.b + y.b, x.ab + y.ab}; }
__device__ __forceinline__ HD operator*(HD x, HD y) {
    return {x.v * y.v, fma(x.v, y.a, x.a * y.v), fma(x.v, y.b, x.b * y.v),
            fma(x.v, y.ab, fma(x.a, y.b, fma(x.b, y.a, x.ab * y.v)))};
}
__device__ __forceinline__ HD operator*(double s, HD x) { return {s * x.v, s * x.a, s * x.b, s * x.ab}; }
__device__ __forceinline__ HD operator+(double s, HD x) { return {s + x.v, x.a, x.b, x.ab}; }
__device__ __forceinline__ HD hd_recip(HD x) {
    const double i = 1.0 / x.v, i2 = i * i;
    return {i, -i2 * x.a, -i2 * x.b, -i2 * x.ab + 2.0 * i2 * i * x.a * x.b};
}
__device__ __forceinline__ HD hd_exp(HD x) {
    const double e = exp(x.v);
    return {e, e * x.a, e * x.b, e * (x.ab + x.a * x.b)};
}

// lam^T pi(x_c + dx, kappa + dk) - the pixel projection weighted by lam - as a hyper-dual
// function of the camera-frame point and the refined intrinsic columns (group chart: fx, log
// aspect, cx, cy, k1, k2, k3, p1, p2 additive; fy = fx * aspect).
__device__ __forceinline__ HD lam_pixel(const DCam& c, const HD* xv, const HD* kv, int ni, const int* cols,
                                        double lam0, double lam1) {
    HD fx = hd(c.fx), la = hd(0.0), cx = hd(c.cx), cy = hd(c.cy);
    HD k1 = hd(c.k1), k2 = hd(c.k2), k3 = hd(c.k3), p1 = hd(c.p1), p2 = hd(c.p2);
    for (int k = 0; k < ni; ++k) {
        switch (cols[k]) {
            case 0: fx = fx + kv[k]; break;
            case 1: la = la + kv[k]; break;
            case 2: cx = cx + kv[k]; break;
            case 3: cy = cy + kv[k]; break;
            case 4: k1 = k1 + kv[k]; break;
            case 5: k2 = k2 + kv[k]; break;
            case 6: k3 = k3 + kv[k]; break;
            case 7: p1 = p1 + kv[k]; break;
            case 8: p2 = p2 + kv[k]; break;
            default: break;
        }
    }
    const double aspect = c.fx > 0.0 ? c.fy / c.fx : 1.0;
    const HD fy = fx * (aspect * hd_exp(la));
    const HD iz = hd_recip(xv[2]);
    const HD x = xv[0] * iz, y = xv[1] * iz;
    const HD r2 = x * x + y * y;
    const HD radial = 1.0 + r2 * (k1 + r2 * (k2 + r2 * k3));
    const HD xy2 = 2.0 * (x * y);
    const HD xd = x * radial + p1 * xy2 + p2 * (r2 + 2.0 * (x * x));
    const HD yd = y * radial + p1 * (r2 + 2.0 * (y * y)) + p2 * xy2;
    const HD pu = (c.su * fx) * xd + cx;
    const HD pv = (c.sv * fy) * yd + cy;
    return lam0 * pu + lam1 * pv;
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
    if (!linearize_obs<double>(c, X[0], X[1], X[2], s, u, v, wobs, loss, lscale, tangent, gb, ni, cols, true, L))
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
    // second derivatives of lam^T pi over (x_c, kappa): M = 3 + ni hyper-dual passes per row
    const int M = 3 + ni;
    double gx[3];
    double Hm[(3 + kMaxNI) * (3 + kMaxNI)];
    for (int i = 0; i < M; ++i)
        for (int j = i; j < M; ++j) {
            HD xv[3], kv[kMaxNI];
            for (int m = 0; m < 3; ++m) xv[m] = {xc[m], i == m ? 1.0 : 0.0, j == m ? 1.0 : 0.0, 0.0};
            for (int k = 0; k < ni; ++k) kv[k] = {0.0, i == 3 + k ? 1.0 : 0.0, j == 3 + k ? 1.0 : 0.0, 0.0};
            const HD f = lam_pixel(c, xv, kv, ni, cols, lam0, lam1);
            Hm[i * M + j] = Hm[j * M + i] = f.ab;
            if (i == j && i < 3) gx[i] = f.a;
        }
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

// Reduced right-hand side: dL/dz of the primary variables (point terms are subtracted by the
// Schur kernel).  One thread per camera, then one per intrinsic column.
__global__ void k_adj_rhs(Shape S, DevPtrs D, AdjBuffers B, double* __restrict__ rhs) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < S.nc) {
        const int b = D.cam_block[t];
        if (b < 0) return;
        const double* g = B.gcam + static_cast<size_t>(t) * 6;
        double* r = rhs + 6 * b;
        r[0] = g[0];
        r[1] = g[1];
        r[2] = g[2];
        if (is_tangent(S, t)) {
            const double* gb = D.gauge_basis;
            r[3] = g[3] * gb[0] + g[4] * gb[1] + g[5] * gb[2];
            r[4] = g[3] * gb[3] + g[4] * gb[4] + g[5] * gb[5];
            r[5] = 0.0;
        } else {
            r[3] = g[3];
            r[4] = g[4];
            r[5] = g[5];
        }
        return;
    }
    const int q = t - S.nc;
    if (q < S.nb) {
        const int g = q / S.ni, k = q - g * S.ni;
        rhs[6 * S.ncb + q] = B.gint[static_cast<size_t>(g) * kP + S.int_cols[k]];
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

constexpr int kSchurThreads = 128;

__global__ void __launch_bounds__(kSchurThreads) k_adj_schur(Shape S, DevPtrs D, AdjBuffers B, RedOut<double> R) {
    extern __shared__ double s_k[];  // nb * nb intrinsic block, then nb rhs
    const int nb = S.nb, ni = S.ni;
    for (int i = threadIdx.x; i < nb * nb + nb; i += blockDim.x) s_k[i] = 0.0;
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const AdjLayout& Lo = B.lay;
    if (t < S.ntp) {
        const int ob = D.trk_obs_begin[t], oe = D.trk_obs_begin[t + 1];
        // own terms
        for (int o = ob; o < oe; ++o) {
            const double* rec = B.rec + static_cast<size_t>(o) * Lo.stride;
            const int cam = D.obs_cam[o];
            const int b = D.cam_block[cam], g = S.ng > 0 ? D.cam_group[cam] : -1;
            if (b >= 0) {
                double* blk = R.vals + static_cast<size_t>(D.diag_pos[b]) * 36;
                const double* h = rec + Lo.hcc();
                for (int a = 0; a < 6; ++a)
                    for (int q = 0; q < 6; ++q) atomicAdd(blk + a * 6 + q, h[a <= q ? sym6(a, q) : sym6(q, a)]);
                if (g >= 0) {
                    const double* hk = rec + Lo.hck();
                    for (int a = 0; a < 6; ++a)
                        for (int k = 0; k < ni; ++k)
                            atomicAdd(R.border + static_cast<size_t>(6 * b + a) * nb + g * ni + k, hk[a * ni + k]);
                }
            }
            if (g >= 0) {
                const double* hk = rec + Lo.hkk();
                for (int k = 0; k < ni; ++k)
                    for (int l = 0; l < ni; ++l)
                        atomicAdd(s_k + (g * ni + k) * nb + g * ni + l, hk[k <= l ? symn(ni, k, l) : symn(ni, l, k)]);
            }
        }
        if (D.trk_block[t] >= 0) {
            double V[6] = {0, 0, 0, 0, 0, 0};
            for (int o = ob; o < oe; ++o) {
                const double* h = B.rec + static_cast<size_t>(o) * Lo.stride + Lo.hpp();
                for (int i = 0; i < 6; ++i) V[i] += h[i];
            }
            double Vi[9];
            if (!sym3_inverse(V, Vi)) {
                atomicOr(B.flags, 1);
                for (int i = 0; i < 9; ++i) Vi[i] = 0.0;
            }
            for (int i = 0; i < 9; ++i) B.vinv[static_cast<size_t>(t) * 9 + i] = Vi[i];
            // dL/d(point chart) = s(X) dL/dX
            const double sp = D.pscale[t];
            const double bp[3] = {sp * B.gpt[static_cast<size_t>(t) * 3], sp * B.gpt[static_cast<size_t>(t) * 3 + 1],
                                  sp * B.gpt[static_cast<size_t>(t) * 3 + 2]};
            double q[3];
            for (int i = 0; i < 3; ++i) q[i] = Vi[i * 3] * bp[0] + Vi[i * 3 + 1] * bp[1] + Vi[i * 3 + 2] * bp[2];
            for (int o1 = ob; o1 < oe; ++o1) {
                const double* rec1 = B.rec + static_cast<size_t>(o1) * Lo.stride;
                const int cam1 = D.obs_cam[o1];
                const int b1 = D.cam_block[cam1], g1 = S.ng > 0 ? D.cam_group[cam1] : -1;
                const double* hcp1 = rec1 + Lo.hcp();
                const double* hpk1 = rec1 + Lo.hpk();
                // Y1 = Hcp1 V^-1 (6 x 3), K1 = Hpk1^T V^-1 (ni x 3)
                double Y1[18], K1[3 * kMaxNI];
                for (int a = 0; a < 6; ++a)
                    for (int j = 0; j < 3; ++j)
                        Y1[a * 3 + j] = hcp1[a * 3] * Vi[j] + hcp1[a * 3 + 1] * Vi[3 + j] + hcp1[a * 3 + 2] * Vi[6 + j];
                for (int k = 0; k < ni; ++k)
                    for (int j = 0; j < 3; ++j)
                        K1[k * 3 + j] = hpk1[k] * Vi[j] + hpk1[ni + k] * Vi[3 + j] + hpk1[2 * ni + k] * Vi[6 + j];
                if (b1 >= 0)
                    for (int a = 0; a < 6; ++a)
                        atomicAdd(R.rhs + 6 * b1 + a, -(hcp1[a * 3] * q[0] + hcp1[a * 3 + 1] * q[1] + hcp1[a * 3 + 2] * q[2]));
                if (g1 >= 0)
                    for (int k = 0; k < ni; ++k)
                        atomicAdd(s_k + nb * nb + g1 * ni + k,
                                  -(hpk1[k] * q[0] + hpk1[ni + k] * q[1] + hpk1[2 * ni + k] * q[2]));
                for (int o2 = ob; o2 < oe; ++o2) {
                    const double* rec2 = B.rec + static_cast<size_t>(o2) * Lo.stride;
                    const int cam2 = D.obs_cam[o2];
                    const int b2 = D.cam_block[cam2], g2 = S.ng > 0 ? D.cam_group[cam2] : -1;
                    const double* hcp2 = rec2 + Lo.hcp();
                    const double* hpk2 = rec2 + Lo.hpk();
                    if (b1 >= 0 && b2 >= 0) {
                        const int pos = csr_find(D, b1, b2);
                        if (pos < 0) {
                            atomicOr(B.flags, 4);
                        } else {
                            double* blk = R.vals + static_cast<size_t>(pos) * 36;
                            for (int a = 0; a < 6; ++a)
                                for (int q2 = 0; q2 < 6; ++q2)
                                    atomicAdd(blk + a * 6 + q2, -(Y1[a * 3] * hcp2[q2 * 3] + Y1[a * 3 + 1] * hcp2[q2 * 3 + 1] +
                                                                  Y1[a * 3 + 2] * hcp2[q2 * 3 + 2]));
                        }
                    }
                    if (b1 >= 0 && g2 >= 0)
                        for (int a = 0; a < 6; ++a)
                            for (int k = 0; k < ni; ++k)
                                atomicAdd(R.border + static_cast<size_t>(6 * b1 + a) * nb + g2 * ni + k,
                                          -(Y1[a * 3] * hpk2[k] + Y1[a * 3 + 1] * hpk2[ni + k] + Y1[a * 3 + 2] * hpk2[2 * ni + k]));
                    if (g1 >= 0 && g2 >= 0)
                        for (int k = 0; k < ni; ++k)
                            for (int l = 0; l < ni; ++l)
                                atomicAdd(s_k + (g1 * ni + k) * nb + g2 * ni + l,
                                          -(K1[k * 3] * hpk2[l] + K1[k * 3 + 1] * hpk2[ni + l] + K1[k * 3 + 2] * hpk2[2 * ni + l]));
                }
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb * nb; i += blockDim.x)
        if (s_k[i] != 0.0) atomicAdd(R.Cm + i, s_k[i]);
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
        if (s_k[nb * nb + i] != 0.0) atomicAdd(R.rhs + 6 * S.ncb + i, s_k[nb * nb + i]);
}

// Priors on the intrinsic diagonal (0.5 (invSigma (theta - prior))^2 has Hessian invSigma^2),
// structurally empty diagonals set to 1 (their right-hand side is zero), border transpose.
__global__ void k_adj_finalize(Shape S, DevPtrs D, RedOut<double> R) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nd = 6 * S.ncb;
    if (t < nd) {
        const int b = t / 6, a = t - b * 6;
        double* d = R.vals + static_cast<size_t>(D.diag_pos[b]) * 36 + a * 7;
        if (*d == 0.0) *d = 1.0;
        for (int k = 0; k < S.nb; ++k)
            R.border_t[static_cast<size_t>(k) * nd + t] = R.border[static_cast<size_t>(t) * S.nb + k];
    } else if (t < nd + S.nb) {
        const int q = t - nd, g = q / S.ni, k = q - g * S.ni;
        const double w = D.groups[static_cast<size_t>(g) * kGroupRec + 2 * kP + S.int_cols[k]];
        double* d = R.Cm + static_cast<size_t>(q) * S.nb + q;
        const double v = *d + w * w;
        *d = v != 0.0 ? v : 1.0;
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
        for (int i = 0; i < 3; ++i) acc[i] = D.pscale[t] * B.gpt[static_cast<size_t>(t) * 3 + i];
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

void launch_adjoint_schur(const Shape& S, const DevPtrs& D, const AdjBuffers& B, const RedOut<double>& R,
                          cudaStream_t st) {
    if (S.ntp <= 0) return;
    const size_t smem = static_cast<size_t>(S.nb * S.nb + S.nb) * sizeof(double);
    k_adj_schur<<<(S.ntp + kSchurThreads - 1) / kSchurThreads, kSchurThreads, smem, st>>>(S, D, B, R);
    const int n = 6 * S.ncb + S.nb;
    k_adj_finalize<<<(n + 127) / 128, 128, 0, st>>>(S, D, R);
}

void launch_adjoint_gradient(const Shape& S, const DevPtrs& D, const AdjBuffers& B, const double* mu, cudaStream_t st) {
    if (S.ntp <= 0) return;
    k_adj_gradient<<<(S.ntp + 127) / 128, 128, 0, st>>>(S, D, B, mu);
}

}  // namespace pb
