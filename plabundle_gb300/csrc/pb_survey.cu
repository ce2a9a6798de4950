// pb_survey.cu -- scale bars on the general path: the tracks of the bars as primary point blocks.
//
// The reference promotes the active, non-fixed tracks of scale bars to primary 3-column blocks
// (prepareActiveProblem, BundleAdjustPlaMatrixProblem.cpp:235-266) and leaves the online Schur
// path whenever a bar is present (canUseReferenceOnlineSchur, ...ReferenceSchur.cpp:667-673).
// Here the fused assembly treats a promoted track like a fixed one (its observations contribute
// their camera and intrinsic terms, its point is not eliminated), and the reduced system is then
// extended by three border columns per promoted point:
//   border  [6 ncb x nbx]: the camera rows of the intrinsic columns (copied), then w J_pose^T J_p
//                          of every observation of a promoted point in that point's columns;
//   Cm      [nbx x nbx]:   the intrinsic block (copied), w J_intr^T J_p and its transpose, the
//                          point blocks w J_p^T J_p + control-point terms, and the scale bars'
//                          w_h J^T J on and between the blocks of their two points;
//   rhs     [n + 3 npr]:   the reduced right-hand side (copied), then -(w J_p^T r + ...) of each
//                          promoted point.
// The extended system is solved like the reduced one (dense factor + CG).  Observation terms are
// FP64 (linearize_obs<double>, the function of the FP64 assembly), one thread per promoted point
// over its observations in processing order; the bars are applied by one thread in bar order,
// so every sum has a fixed order.  The promoted blocks are damped like every primary diagonal,
// finalizePrimaryDiagonal(1 + damping, 1): a promoted point is not coupled to any eliminated
// point, so its block is the same before and after the point elimination.
#include <cuda_runtime.h>

#include "pb_device.cuh"
#include "pb_kernels.h"

namespace pb {

namespace {

// linearizeScaleBar (BundleAdjustPlaMatrixConstraints.cpp:118-153) with finishRobust's Huber
// loss on the squared residual: r = s (|Xa - Xb| - L), dr/dXa = s (Xa - Xb) / |Xa - Xb| = -dr/dXb.
// False when the points coincide (the bar is skipped, as the reference skips it).
__device__ __forceinline__ bool bar_eval(const double* Xa, const double* Xb, double length, double scale, double delta,
                                         double& r, double* J, double& cost, double& weight) {
    const double d0 = Xa[0] - Xb[0], d1 = Xa[1] - Xb[1], d2 = Xa[2] - Xb[2];
    const double dist = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    if (!(dist > 1e-12)) return false;
    r = scale * (dist - length);
    J[0] = scale * d0 / dist;
    J[1] = scale * d1 / dist;
    J[2] = scale * d2 / dist;
    const double sq = r * r;
    if (!isfinite(sq)) return false;
    if (sq <= delta * delta) {
        cost = 0.5 * sq;
        weight = 1.0;
    } else {
        const double n = sqrt(sq);
        cost = delta * n - 0.5 * delta * delta;
        weight = delta / n;
    }
    return isfinite(cost) && isfinite(weight);
}

}  // namespace

// Copies of the reduced system into the extended one; the new columns and rows start at zero.
__global__ void k_ext_copy(Shape S, RedOut<double> R, ExtSys X) {
    const int n6 = 6 * S.ncb, nb = S.nb, nbx = X.nbx;
    const long long nB = static_cast<long long>(n6) * nbx, nC = static_cast<long long>(nbx) * nbx;
    const long long tot = nB + nC + X.nx;
    for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < tot;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (e < nB) {
            const int row = static_cast<int>(e / nbx), col = static_cast<int>(e - static_cast<long long>(row) * nbx);
            X.border[e] = col < nb ? R.border[static_cast<size_t>(row) * nb + col] : 0.0;
        } else if (e < nB + nC) {
            const long long f = e - nB;
            const int i = static_cast<int>(f / nbx), j = static_cast<int>(f - static_cast<long long>(i) * nbx);
            X.Cm[f] = (i < nb && j < nb) ? R.Cm[static_cast<size_t>(i) * nb + j] : 0.0;
        } else {
            const int i = static_cast<int>(e - nB - nC);
            X.rhs[i] = i < S.n ? R.rhs[i] : 0.0;
        }
    }
}

// One thread per promoted point: its observations' point terms and couplings, its control points.
__global__ void k_ext_points(Shape S, DevPtrs D, ExtSys X, int* __restrict__ flags) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= S.npr) return;
    const int t = D.prom_proc[k];
    const int nb = S.nb, nbx = X.nbx, ni = S.ni, col = nb + 3 * k;
    const double* Xp = D.points + static_cast<size_t>(t) * 3;
    double P[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, g[3] = {0, 0, 0};
    for (int o = D.trk_obs_begin[t]; o < D.trk_obs_begin[t + 1]; ++o) {
        const int cam = D.obs_cam[o];
        DCam c;
        load_cam(D.cams_eff + static_cast<size_t>(cam) * kCamStride, c);
        const bool tangent = cam == S.gauge_scale && S.gauge_anchor >= 0 && S.gauge_baseline > 0.0;
        Lin<double> L;
        double grad[9 + kMaxNI];
        if (!linearize_obs<double>(c, Xp[0], Xp[1], Xp[2], D.pscale[t], D.obs_u[o], D.obs_v[o], D.obs_w[o], S.loss,
                                   S.loss_scale, tangent, !S.ref_param, D.gauge_basis, ni, S.int_cols, true, L, grad)) {
            atomicOr(flags, 2);
            continue;
        }
        const double w = L.wd, r0 = L.rd0, r1 = L.rd1;
        const double* Jp = L.Jp;
        for (int i = 0; i < 3; ++i) {
            g[i] += w * (Jp[i] * r0 + Jp[3 + i] * r1);
            for (int j = 0; j < 3; ++j) P[i * 3 + j] += w * (Jp[i] * Jp[j] + Jp[3 + i] * Jp[3 + j]);
        }
        const int b = D.cam_block[cam];
        if (b >= 0)
            for (int a = 0; a < 6; ++a)
                for (int j = 0; j < 3; ++j)
                    X.border[static_cast<size_t>(6 * b + a) * nbx + col + j] +=
                        w * (L.Jc[a] * Jp[j] + L.Jc[6 + a] * Jp[3 + j]);
        const int grp = S.ng > 0 ? D.cam_group[cam] : -1;
        if (grp >= 0)
            for (int i = 0; i < ni; ++i)
                for (int j = 0; j < 3; ++j) {
                    const double v = w * (L.Ji[i] * Jp[j] + L.Ji[kMaxNI + i] * Jp[3 + j]);
                    X.Cm[static_cast<size_t>(grp * ni + i) * nbx + col + j] += v;
                    X.Cm[static_cast<size_t>(col + j) * nbx + grp * ni + i] += v;
                }
    }
    // control points of the track: point-only primary residuals (addPointResidual,
    // BundleAdjustPlaMatrixAssembly.cpp:356-380), J = sqrt(weight) W, Huber weight
    if (S.ncp > 0)
        for (int q = D.trk_cp_begin[t]; q < D.trk_cp_begin[t + 1]; ++q) {
            const double* rec = D.cp_rec + static_cast<size_t>(q) * 12;
            double r[3], cc, cw;
            if (!cp_eval(rec, Xp[0], Xp[1], Xp[2], S.cp_huber, r, cc, cw)) continue;
            for (int i = 0; i < 3; ++i) {
                g[i] += cw * (rec[i] * r[0] + rec[3 + i] * r[1] + rec[6 + i] * r[2]);
                for (int j = 0; j < 3; ++j)
                    P[i * 3 + j] += cw * (rec[i] * rec[j] + rec[3 + i] * rec[3 + j] + rec[6 + i] * rec[6 + j]);
            }
        }
    for (int i = 0; i < 3; ++i) {
        X.rhs[S.n + 3 * k + i] = -g[i];
        for (int j = 0; j < 3; ++j) X.Cm[static_cast<size_t>(col + i) * nbx + col + j] = P[i * 3 + j];
    }
}

// The scale bars, in bar order (one thread): their terms on the promoted blocks and their cost at
// the current state; then the damping of the promoted diagonals.
__global__ void k_ext_bars(Shape S, DevPtrs D, ExtSys X, double damping, double* __restrict__ bar_cost) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int nb = S.nb, nbx = X.nbx;
    double cost = 0.0;
    for (int i = 0; i < S.nbar; ++i) {
        const int ta = D.bar_pidx[2 * i], tb = D.bar_pidx[2 * i + 1];
        if (ta < 0 || tb < 0) continue;  // a track that is not active
        double r, J[3], cc, w;
        if (!bar_eval(D.points + static_cast<size_t>(ta) * 3, D.points + static_cast<size_t>(tb) * 3, D.bar_par[2 * i],
                      D.bar_par[2 * i + 1], S.bar_huber, r, J, cc, w))
            continue;
        cost += cc;
        const int ka = D.trk_prom[ta], kb = D.trk_prom[tb];
        const int ca = nb + 3 * ka, cb = nb + 3 * kb;
        // dr/dXa = J, dr/dXb = -J
        if (ka >= 0)
            for (int p = 0; p < 3; ++p) {
                X.rhs[S.n + 3 * ka + p] -= w * J[p] * r;
                for (int q = 0; q < 3; ++q) X.Cm[static_cast<size_t>(ca + p) * nbx + ca + q] += w * J[p] * J[q];
            }
        if (kb >= 0)
            for (int p = 0; p < 3; ++p) {
                X.rhs[S.n + 3 * kb + p] += w * J[p] * r;
                for (int q = 0; q < 3; ++q) X.Cm[static_cast<size_t>(cb + p) * nbx + cb + q] += w * J[p] * J[q];
            }
        if (ka >= 0 && kb >= 0)
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q) {
                    X.Cm[static_cast<size_t>(ca + p) * nbx + cb + q] -= w * J[p] * J[q];
                    X.Cm[static_cast<size_t>(cb + q) * nbx + ca + p] -= w * J[p] * J[q];
                }
    }
    *bar_cost = cost;
    for (int k = 0; k < S.npr; ++k)
        for (int p = 0; p < 3; ++p) {
            double* d = X.Cm + static_cast<size_t>(nb + 3 * k + p) * nbx + nb + 3 * k + p;
            *d = *d != 0.0 ? *d * (1.0 + damping) : 1.0;
        }
}

// border_t = border^T for the solvers' border rows.
__global__ void k_ext_transpose(Shape S, ExtSys X) {
    const int n6 = 6 * S.ncb, nbx = X.nbx;
    const long long tot = static_cast<long long>(n6) * nbx;
    for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < tot;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int c = static_cast<int>(e / n6), row = static_cast<int>(e - static_cast<long long>(c) * n6);
        X.border_t[e] = X.border[static_cast<size_t>(row) * nbx + c];
    }
}

// After the solve of the extended system: the camera / intrinsic step (first n entries) and the
// promoted points' steps into the point-step array, with the squared sum of the latter (fixed
// order, one thread).
__global__ void k_ext_step(Shape S, DevPtrs D, const double* __restrict__ xsol, double* __restrict__ step_c,
                           double* __restrict__ step_p, double* __restrict__ out) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    for (int i = tid; i < S.n; i += gridDim.x * blockDim.x) step_c[i] = xsol[i];
    if (tid == 0) {
        double sq = 0.0;
        for (int k = 0; k < S.npr; ++k) {
            const int t = D.prom_proc[k];
            for (int p = 0; p < 3; ++p) {
                const double v = xsol[S.n + 3 * k + p];
                step_p[static_cast<size_t>(t) * 3 + p] = v;
                sq += v * v;
            }
        }
        *out = sq;
    }
}

// Scale-bar cost of each trial state (points + alpha step for the points that move) or of the
// current state, one thread per step length, bars in order.
__global__ void k_bar_cost(Shape S, DevPtrs D, const double* __restrict__ step_p, const double* __restrict__ alphas,
                           int n_alpha, int use_trial, double* __restrict__ out) {
    const int a = threadIdx.x;
    if (a >= n_alpha) return;
    const double alpha = use_trial ? alphas[a] : 0.0;
    double cost = 0.0;
    for (int i = 0; i < S.nbar; ++i) {
        const int ta = D.bar_pidx[2 * i], tb = D.bar_pidx[2 * i + 1];
        if (ta < 0 || tb < 0) continue;
        double Xa[3], Xb[3];
        for (int p = 0; p < 3; ++p) {
            Xa[p] = D.points[static_cast<size_t>(ta) * 3 + p];
            Xb[p] = D.points[static_cast<size_t>(tb) * 3 + p];
        }
        if (use_trial) {
            if (D.trk_free[ta]) {
                const double f = D.pscale[ta] * alpha;
                for (int p = 0; p < 3; ++p) Xa[p] += f * step_p[static_cast<size_t>(ta) * 3 + p];
            }
            if (D.trk_free[tb]) {
                const double f = D.pscale[tb] * alpha;
                for (int p = 0; p < 3; ++p) Xb[p] += f * step_p[static_cast<size_t>(tb) * 3 + p];
            }
        }
        double r, J[3], cc, w;
        if (!bar_eval(Xa, Xb, D.bar_par[2 * i], D.bar_par[2 * i + 1], S.bar_huber, r, J, cc, w)) continue;
        cost += cc;
    }
    out[a] = cost;
}

void launch_extend_system(const Shape& S, const DevPtrs& D, const RedOut<double>& R, const ExtSys& X, double damping,
                          int* flags, double* bar_cost, cudaStream_t st) {
    k_ext_copy<<<std::max(1, 2 * 152), 256, 0, st>>>(S, R, X);
    if (S.npr > 0) k_ext_points<<<(S.npr + 63) / 64, 64, 0, st>>>(S, D, X, flags);
    k_ext_bars<<<1, 32, 0, st>>>(S, D, X, damping, bar_cost);
    k_ext_transpose<<<std::max(1, 2 * 152), 256, 0, st>>>(S, X);
}

void launch_ext_step(const Shape& S, const DevPtrs& D, const double* xsol, double* step_c, double* step_p, double* out,
                     cudaStream_t st) {
    k_ext_step<<<std::max(1, (S.n + 255) / 256), 256, 0, st>>>(S, D, xsol, step_c, step_p, out);
}

void launch_bar_cost(const Shape& S, const DevPtrs& D, const double* step_p, const double* alphas, int n_alpha,
                     int use_trial, double* out, cudaStream_t st) {
    k_bar_cost<<<1, 32, 0, st>>>(S, D, step_p, alphas, n_alpha, use_trial, out);
}

}  // namespace pb
