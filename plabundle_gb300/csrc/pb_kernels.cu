// pb_kernels.cu -- reduction of the assembly partials, back-substitution, objective and
// state-update kernels (the assembly kernel itself is in pb_assemble.cu).
//
// `k_reduce_*` sum the chunk partials of every reduced block in a fixed order, with the
// accumulator of the arithmetic path (two-sum compensated float-float on the FP32 path), so the
// reduced matrix is assembled without atomics and reproducibly.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "pb_device.cuh"
#include "pb_kernels.h"

namespace pb {

// The three fixed-order sums below are independent of one another and each is latency-bound on
// a small grid (the chunk-record sum has one CTA per 32 record entries), so one launch runs them
// side by side over block ranges [pose pairs | cameras | chunk records + cost].  Each keeps the
// summation order of its own loop; the loads of a loop are issued ahead of its merge chain.
template <typename T>
struct ReduceArgs {
    using part_t = typename Acc<T>::part_type;
    const part_t* part_pair;
    const part_t* part_cam;
    const part_t* part_chunk;
    const double* part_cost;
    const int* part_flags;
    double *vals, *rhs, *direct, *border, *border_t, *Cm, *result;
    unsigned pair_blocks, cam_blocks;
};

// Sum of the chunk partials of every upper pose block, written to both CSR orientations.
template <typename T>
__device__ __forceinline__ void reduce_pairs(const Shape& S, const DevPtrs& D, const ReduceArgs<T>& R, unsigned blk) {
    const long long idx = static_cast<long long>(blk) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<long long>(S.nupper) * 36) return;
    const int u = static_cast<int>(idx / 36), e = static_cast<int>(idx - static_cast<long long>(u) * 36);
    Acc<T> acc;
    const int c1 = D.up_contrib_begin[u + 1];
#pragma unroll 4
    for (int c = D.up_contrib_begin[u]; c < c1; ++c)
        acc.merge_part(R.part_pair[static_cast<size_t>(D.up_contrib[c]) * 36 + e]);
    const double v = acc.value64();
    R.vals[static_cast<size_t>(D.up_csr[u]) * 36 + e] = v;
    const int t = D.up_csr_t[u];
    if (t >= 0) R.vals[static_cast<size_t>(t) * 36 + (e % 6) * 6 + e / 6] = v;
}

// Sum of the per-camera partials: rhs, direct rhs and the intrinsic border rows.
template <typename T>
__device__ __forceinline__ void reduce_cams(const Shape& S, const DevPtrs& D, const ReduceArgs<T>& R, unsigned blk) {
    const int camrec = 12 + S.ng * 6 * S.ni;
    const long long idx = static_cast<long long>(blk) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<long long>(S.ncb) * camrec) return;
    const int i = static_cast<int>(idx / camrec), e = static_cast<int>(idx - static_cast<long long>(i) * camrec);
    Acc<T> acc;
    const int c1 = D.cam_contrib_begin[i + 1];
#pragma unroll 4
    for (int c = D.cam_contrib_begin[i]; c < c1; ++c)
        acc.merge_part(R.part_cam[static_cast<size_t>(D.cam_contrib[c]) * camrec + e]);
    const double v = acc.value64();
    if (e < 6) R.rhs[i * 6 + e] = v;
    else if (e < 12) R.direct[i * 6 + e - 6] = v;
    else {
        const int f = e - 12;  // (g * 6 + a) * ni + c
        const int g = f / (6 * S.ni), rem = f - g * 6 * S.ni, a = rem / S.ni, c = rem - a * S.ni;
        R.border[(static_cast<size_t>(i) * 6 + a) * S.nb + g * S.ni + c] = v;
        R.border_t[static_cast<size_t>(g * S.ni + c) * 6 * S.ncb + i * 6 + a] = v;
    }
}

// Chunk-level sums (intrinsic block, intrinsic rhs): one CTA per 32 record entries, its warps
// striding over the chunks, merged in warp order.  The block after the last tile sums the costs
// and flags.
template <typename T>
__device__ __forceinline__ void reduce_chunks(const Shape& S, const ReduceArgs<T>& R, unsigned blk) {
    const int nb = S.nb, chrec = nb * nb + 2 * nb;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int tiles = (chrec + 31) / 32;
    double* Cm = R.Cm;
    double* rhs_b = R.rhs + 6 * S.ncb;
    double* direct_b = R.direct + 6 * S.ncb;
    if (static_cast<int>(blk) < tiles) {
        __shared__ typename Acc<T>::part_type s_acc[8][32];
        const int e = blk * 32 + lane;
        Acc<T> acc;
        if (e < chrec) {
#pragma unroll 4
            for (int c = wid; c < S.nchunks; c += nw) acc.merge_part(R.part_chunk[static_cast<size_t>(c) * chrec + e]);
        }
        s_acc[wid][lane] = acc.part();
        __syncthreads();
        if (wid == 0 && e < chrec) {
            Acc<T> tot;
            for (int w = 0; w < nw; ++w) tot.merge_part(s_acc[w][lane]);
            const double v = tot.value64();
            if (e < nb * nb) Cm[e] = v;
            else if (e < nb * nb + nb) rhs_b[e - nb * nb] = v;
            else direct_b[e - nb * nb - nb] = v;
        }
        return;
    }
    __shared__ double s_cost[256];
    __shared__ int s_flag[256];
    double c = 0.0;
    int f = 0;
    for (int i = threadIdx.x; i < S.nchunks; i += blockDim.x) {
        c += R.part_cost[i];
        f |= R.part_flags[i];
    }
    s_cost[threadIdx.x] = c;
    s_flag[threadIdx.x] = f;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
            s_cost[threadIdx.x] += s_cost[threadIdx.x + st];
            s_flag[threadIdx.x] |= s_flag[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        R.result[0] = s_cost[0];
        R.result[1] = static_cast<double>(s_flag[0]);
    }
}

// 256 threads per block (the chunk-record sum's warp count and cost buffers assume it); the block
// range decides the sum, uniformly per block.
template <typename T>
__global__ void __launch_bounds__(256) k_reduce_sums(Shape S, DevPtrs D, ReduceArgs<T> R) {
    const unsigned b = blockIdx.x;
    if (b < R.pair_blocks) reduce_pairs<T>(S, D, R, b);
    else if (b < R.pair_blocks + R.cam_blocks) reduce_cams<T>(S, D, R, b - R.pair_blocks);
    else reduce_chunks<T>(S, R, b - R.pair_blocks - R.cam_blocks);
}

// Intrinsic priors (assembleReferencePriors, ...ReferenceSchur.cpp:492-536) and
// finalizePrimaryDiagonal(1 + lambda, 1): positive diagonal entries scaled, empty ones set to 1.
__global__ void k_finalize(Shape S, DevPtrs D, double* __restrict__ vals, double* __restrict__ Cm,
                           double* __restrict__ rhs_b, double* __restrict__ direct_b, double* __restrict__ result,
                           double damping) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    // rig problems damp the diagonal of the rig pose blocks after the map (pb_rig.cu) instead
    if (tid < S.ncb * 6 && !S.rig) {
        const int i = tid / 6, a = tid - i * 6;
        double* d = vals + static_cast<size_t>(D.diag_pos[i]) * 36 + a * 7;
        const double v = *d;
        *d = v != 0.0 ? v * (1.0 + damping) : 1.0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && S.ng > 0) {
        double cost = 0.0;
        for (int g = 0; g < S.ng; ++g) {
            const double* G = D.groups + static_cast<size_t>(g) * kGroupRec;
            for (int c = 0; c < S.ni; ++c) {
                const int p = S.int_cols[c];
                const double w = G[2 * kP + p];
                const double r = w * (G[p] - G[kP + p]);
                cost += 0.5 * r * r;
                const int col = g * S.ni + c;
                double* cd = Cm + col * S.nb + col;
                const double v = *cd + w * w;
                *cd = v != 0.0 ? v * (1.0 + damping) : 1.0;
                rhs_b[col] -= w * r;
                direct_b[col] -= w * r;
            }
        }
        result[0] += cost;
    }
}

// Effective cameras of the current state (group intrinsics applied, makeCameraWithSharedIntrinsics,
// BundleAdjustPlaMatrixProjection.cpp:134-171) and the gauge tangent basis
// (referenceGaugeTargetTangentBasis, BundleAdjustPlaMatrixAssembly.cpp:69-99).
__device__ void group_camera(const double* __restrict__ state, const double* __restrict__ ref,
                             const double* __restrict__ G, double* __restrict__ out) {
    for (int i = 0; i < kCamStride; ++i) out[i] = state[i];
    if (!G) return;
    const double* en = G + 5 * kP;
    const double fx = en[0] != 0.0 ? G[0] : state[12];
    const double src_aspect = state[12] > 1e-12 ? state[13] / state[12] : 1.0;
    const double aspect = en[1] != 0.0 ? exp(G[1]) : src_aspect;
    out[12] = fx;
    out[13] = fx * aspect;
    out[14] = en[2] != 0.0 ? ref[14] + G[2] : state[14];
    out[15] = en[3] != 0.0 ? ref[15] + G[3] : state[15];
    for (int p = 4; p < 9; ++p)
        if (en[p] != 0.0) out[12 + p] = G[p];
}

__device__ void gauge_basis(const double* anchor_c, const double* scale_c, double* target_basis, double* world_basis) {
    const double o[3] = {anchor_c[0], -anchor_c[1], -anchor_c[2]};
    const double c[3] = {scale_c[0], -scale_c[1], -scale_c[2]};
    double u[3] = {c[0] - o[0], c[1] - o[1], c[2] - o[2]};
    const double len = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    const double il = len >= 1e-20 ? 1.0 / len : 0.0;
    for (int i = 0; i < 3; ++i) u[i] *= il;
    int axis = fabs(u[0]) > fabs(u[1]) ? 1 : 0;
    if (fabs(u[axis]) > fabs(u[2])) axis = 2;
    double ax[3] = {0, 0, 0};
    ax[axis] = 1.0;
    double s[3] = {ax[1] * u[2] - ax[2] * u[1], ax[2] * u[0] - ax[0] * u[2], ax[0] * u[1] - ax[1] * u[0]};
    const double sl = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    const double isl = sl >= 1e-20 ? 1.0 / sl : 0.0;
    for (int i = 0; i < 3; ++i) s[i] *= isl;
    const double f[3] = {u[1] * s[2] - u[2] * s[1], u[2] * s[0] - u[0] * s[2], u[0] * s[1] - u[1] * s[0]};
    for (int i = 0; i < 3; ++i) {
        target_basis[i] = f[i];
        target_basis[3 + i] = s[i];
    }
    world_basis[0] = f[0]; world_basis[1] = -f[1]; world_basis[2] = -f[2];
    world_basis[3] = s[0]; world_basis[4] = -s[1]; world_basis[5] = -s[2];
}

__global__ void k_effective(Shape S, DevPtrs D) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < S.ntp) {
        const double* X = D.points + static_cast<size_t>(c) * 3;
        const double sc = S.ref_param ? point_scale(X[0], X[1], X[2]) : 1.0;
        D.pscale[c] = sc;
        D.pscale_ff[c] = ff_pack(sc);
    }
    if (c < S.nc) {
        const double* G = S.ng > 0 ? D.groups + static_cast<size_t>(D.cam_group[c]) * kGroupRec : nullptr;
        double* ef = D.cams_eff + static_cast<size_t>(c) * kCamStride;
        group_camera(D.cams_state + static_cast<size_t>(c) * kCamStride, D.cams_ref + static_cast<size_t>(c) * kCamStride,
                     G, ef);
        camera_ff(ef, D.cams_ff + static_cast<size_t>(c) * kCamFF);
    }
    if (c == 0 && S.gauge_anchor >= 0 && S.gauge_scale >= 0 && S.gauge_baseline > 0.0)
        gauge_basis(D.cams_state + static_cast<size_t>(S.gauge_anchor) * kCamStride + 9,
                    D.cams_state + static_cast<size_t>(S.gauge_scale) * kCamStride + 9, D.gauge_basis + 6,
                    D.gauge_basis);
}

// Trial states for a batch of step lengths: pose retraction (applyReferenceCameraPoseStep,
// BundleAdjustPlaMatrixAssembly.cpp:130-179; gauge tangent step :101-128; the plain
// parameterisation's pose delta :1134-1136) and clamped intrinsic update (applyIntrinsicStep,
// BundleAdjustPlaMatrixModel.cpp:248-269).
__global__ void k_trial_cameras(Shape S, DevPtrs D, const double* __restrict__ step_c, const double* __restrict__ alphas,
                                int n_alpha) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n_alpha * S.nc) return;
    const int a = idx / S.nc, c = idx - a * S.nc;
    const double alpha = alphas[a];
    // trial groups (each camera thread of the first ng cameras writes one group)
    double Gt[kGroupRec];
    const double* Gs = nullptr;
    if (S.ng > 0) {
        const int g = D.cam_group[c];
        const double* G = D.groups + static_cast<size_t>(g) * kGroupRec;
        for (int i = 0; i < kGroupRec; ++i) Gt[i] = G[i];
        for (int k = 0; k < S.ni; ++k) {
            const int p = S.int_cols[k];
            const double v = G[p] + alpha * step_c[6 * S.ncb + g * S.ni + k];
            Gt[p] = fmin(fmax(v, G[3 * kP + p]), G[4 * kP + p]);
        }
        Gs = Gt;
        if (c < S.ng) {
            const double* G2 = D.groups + static_cast<size_t>(c) * kGroupRec;
            double* out = D.groups_trial + (static_cast<size_t>(a) * S.ng + c) * kGroupRec;
            for (int i = 0; i < kGroupRec; ++i) out[i] = G2[i];
            for (int k = 0; k < S.ni; ++k) {
                const int p = S.int_cols[k];
                const double v = G2[p] + alpha * step_c[6 * S.ncb + c * S.ni + k];
                out[p] = fmin(fmax(v, G2[3 * kP + p]), G2[4 * kP + p]);
            }
        }
    }
    double pose[kCamStride];
    const double* st = D.cams_state + static_cast<size_t>(c) * kCamStride;
    for (int i = 0; i < kCamStride; ++i) pose[i] = st[i];
    const int b = D.cam_block[c];
    if (b >= 0 && !S.ref_param) {
        // plain parameterisation: the camera's own pose delta (CameraState::applyDeltaPose,
        // BundleAdjustPlaMatrixAssembly.cpp:1134-1136), C2W' = Exp(alpha w) C2W by Rodrigues'
        // formula and C' = C + alpha dC for every refined camera, the gauge scale camera's
        // tangent coordinates included
        const double* d = step_c + 6 * b;
        const double w0 = alpha * d[0], w1 = alpha * d[1], w2 = alpha * d[2];
        const double th2 = w0 * w0 + w1 * w1 + w2 * w2;
        double A, B;
        if (th2 < 1e-16) {
            A = 1.0 - th2 / 6.0;
            B = 0.5 - th2 / 24.0;
        } else {
            const double th = sqrt(th2), sh = sin(0.5 * th);
            A = sin(th) / th;
            B = 2.0 * sh * sh / th2;  // (1 - cos th) / th^2 without the cancellation
        }
        const double K[9] = {0.0, -w2, w1, w2, 0.0, -w0, -w1, w0, 0.0};
        double E[9];
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) {
                const double kk = K[r * 3] * K[q] + K[r * 3 + 1] * K[3 + q] + K[r * 3 + 2] * K[6 + q];
                E[r * 3 + q] = (r == q ? 1.0 : 0.0) + A * K[r * 3 + q] + B * kk;
            }
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q)
                pose[r * 3 + q] = E[r * 3] * st[q] + E[r * 3 + 1] * st[3 + q] + E[r * 3 + 2] * st[6 + q];
        for (int i = 0; i < 3; ++i) pose[9 + i] = st[9 + i] + alpha * d[3 + i];
    } else if (b >= 0) {
        const double* d = step_c + 6 * b;
        const double dx = alpha * d[0], dy = alpha * d[1], dz = alpha * d[2];
        double sx, cx, sy, cy, sz, cz;
        sincos(dx, &sx, &cx);
        sincos(dy, &sy, &cy);
        sincos(dz, &sz, &cz);
        // E = Rx Ry Rz
        const double E[9] = {cy * cz, -cy * sz, sy,
                             sx * sy * cz + cx * sz, -sx * sy * sz + cx * cz, -sx * cy,
                             -cx * sy * cz + sx * sz, cx * sy * sz + sx * cz, cx * cy};
        const double sg[3] = {1.0, -1.0, -1.0};
        double Tl[9];
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) Tl[r * 3 + q] = sg[r] * E[q * 3 + r] * sg[q];
        double Rn[9];
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q)
                Rn[r * 3 + q] = Tl[r * 3 + 0] * st[0 * 3 + q] + Tl[r * 3 + 1] * st[1 * 3 + q] + Tl[r * 3 + 2] * st[2 * 3 + q];
        for (int i = 0; i < 9; ++i) pose[i] = Rn[i];
        const bool tangent = c == S.gauge_scale && S.gauge_anchor >= 0 && S.gauge_baseline > 0.0;
        if (tangent) {
            const double* tb = D.gauge_basis + 6;
            const double* ac = D.cams_state + static_cast<size_t>(S.gauge_anchor) * kCamStride + 9;
            const double o[3] = {ac[0], -ac[1], -ac[2]};
            const double ce[3] = {st[9], -st[10], -st[11]};
            const double ta = alpha * d[3], tb2 = alpha * d[4];
            double dir[3];
            for (int i = 0; i < 3; ++i) dir[i] = ce[i] + tb[i] * ta + tb[3 + i] * tb2 - o[i];
            const double len = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
            double nc[3];
            if (len < 1e-20) {
                for (int i = 0; i < 3; ++i) nc[i] = o[i];
            } else {
                const double il = 1.0 / len;
                for (int i = 0; i < 3; ++i) nc[i] = o[i] + dir[i] * il * S.gauge_baseline;
            }
            pose[9] = nc[0];
            pose[10] = -nc[1];
            pose[11] = -nc[2];
        } else {
            pose[9] = st[9] + alpha * d[3];
            pose[10] = st[10] + alpha * d[4];
            pose[11] = st[11] + alpha * d[5];
        }
    }
    group_camera(pose, D.cams_ref + static_cast<size_t>(c) * kCamStride, Gs,
                 D.cams_trial + (static_cast<size_t>(a) * S.nc + c) * kCamStride);
}

// Objective of the trial states: image costs (FP64) per step length, block partials.
__global__ void __launch_bounds__(256) k_cost_batch(Shape S, DevPtrs D, const double* __restrict__ step_p,
                                                    const double* __restrict__ alphas, int n_alpha, int use_trial,
                                                    double* __restrict__ part) {
    __shared__ double s_c[kMaxAlpha][8];
    __shared__ int s_bad[kMaxAlpha];
    const long long o = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (threadIdx.x < kMaxAlpha) s_bad[threadIdx.x] = 0;
    __syncthreads();
    double c[kMaxAlpha];
    for (int a = 0; a < kMaxAlpha; ++a) c[a] = 0.0;
    if (o < S.nop) {
        const int cam = D.obs_cam[o], trk = D.obs_trk[o];
        const double* X = D.points + static_cast<size_t>(trk) * 3;
        const double u = D.obs_u[o], v = D.obs_v[o], w = D.obs_w[o];
        const bool moves = use_trial && D.trk_free[trk];
        const double s = moves ? D.pscale[trk] : 0.0;
        const double* dp = moves ? step_p + static_cast<size_t>(trk) * 3 : nullptr;
        for (int a = 0; a < n_alpha; ++a) {
            DCam k;
            load_cam((use_trial ? D.cams_trial + (static_cast<size_t>(a) * S.nc) * kCamStride : D.cams_eff) +
                         static_cast<size_t>(cam) * kCamStride,
                     k);
            double X0 = X[0], X1 = X[1], X2 = X[2];
            if (moves) {
                const double f = s * alphas[a];
                X0 += f * dp[0];
                X1 += f * dp[1];
                X2 += f * dp[2];
            }
            Proj p;
            double cost = 0.0, rw;
            bool good = project64(k, X0, X1, X2, p);
            if (good) {
                const double r0 = p.px - u, r1 = p.py - v;
                good = robust_loss(w * (r0 * r0 + r1 * r1), S.loss, S.loss_scale, cost, rw) && isfinite(cost);
            }
            if (good && S.ncp > 0 && o == D.trk_obs_begin[trk]) {
                // the track's control points, once per track (its first observation's thread); a
                // term that is not finite is skipped (BundleAdjustPlaMatrixAssembly.cpp:674-690)
                for (int q = D.trk_cp_begin[trk]; q < D.trk_cp_begin[trk + 1]; ++q) {
                    double r[3], cc, cw;
                    if (cp_eval(D.cp_rec + static_cast<size_t>(q) * 12, X0, X1, X2, S.cp_huber, r, cc, cw)) cost += cc;
                }
            }
            if (!good) atomicOr(&s_bad[a], 1);
            else c[a] = cost;
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int a = 0; a < n_alpha; ++a) {
        const double v = warp_sum(c[a]);
        if (lane == 0) s_c[a][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < n_alpha) {
        double t = 0.0;
        for (int w2 = 0; w2 < static_cast<int>(blockDim.x >> 5); ++w2) t += s_c[threadIdx.x][w2];
        part[static_cast<size_t>(blockIdx.x) * kMaxAlpha * 2 + threadIdx.x] = t;
        part[static_cast<size_t>(blockIdx.x) * kMaxAlpha * 2 + kMaxAlpha + threadIdx.x] = s_bad[threadIdx.x];
    }
}

// Final objective per step length: block partials in fixed order plus the intrinsic priors of the
// trial groups (assemblePrimaryPriors cost, BundleAdjustPlaMatrixAssemblySurvey.cpp:43-91).
__global__ void k_cost_final(Shape S, DevPtrs D, const double* __restrict__ part, int nblocks, int n_alpha,
                             int use_trial, double* __restrict__ out) {
    __shared__ double s_v[256];
    __shared__ int s_b[256];
    for (int a = 0; a < n_alpha; ++a) {
        double v = 0.0;
        int bad = 0;
        for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
            v += part[static_cast<size_t>(i) * kMaxAlpha * 2 + a];
            bad |= part[static_cast<size_t>(i) * kMaxAlpha * 2 + kMaxAlpha + a] != 0.0;
        }
        s_v[threadIdx.x] = v;
        s_b[threadIdx.x] = bad;
        __syncthreads();
        for (int st = blockDim.x / 2; st > 0; st >>= 1) {
            if (threadIdx.x < st) {
                s_v[threadIdx.x] += s_v[threadIdx.x + st];
                s_b[threadIdx.x] |= s_b[threadIdx.x + st];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            double cost = s_v[0];
            for (int g = 0; g < S.ng; ++g) {
                const double* G = (use_trial ? D.groups_trial + static_cast<size_t>(a) * S.ng * kGroupRec : D.groups) +
                                  static_cast<size_t>(g) * kGroupRec;
                for (int c = 0; c < S.ni; ++c) {
                    const int p = S.int_cols[c];
                    const double r = G[2 * kP + p] * (G[p] - G[kP + p]);
                    cost += 0.5 * r * r;
                }
            }
            out[a] = s_b[0] ? __longlong_as_double(0x7ff0000000000000ll) : cost;
        }
        __syncthreads();
    }
}

// Back-substitution (recoverReferencePointSteps, ...ReferenceSchur.cpp:982-1082), one thread per
// track:  dp = R^-T (q - R^-1 u),  u = sum_o w J_p^T (J_o dc).
// Per observation o of an eliminated track: the term Y_o^T A_o dc (3 values) of its track's sum,
// one thread per observation (records read by consecutive lanes, FP64 accumulation).
template <typename T>
__global__ void __launch_bounds__(256) k_backsub_terms(Shape S, DevPtrs D, const T* __restrict__ obs_rec,
                                                       const double* __restrict__ step_c, double* __restrict__ terms) {
    const long long o = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (o >= S.nop) return;
    const int nA = 6 + S.ni, stride = 2 * nA + 6;
    const int cam = D.obs_cam[o];
    const T* rec = obs_rec + static_cast<size_t>(o) * stride;
    double e0 = 0.0, e1 = 0.0;
    const int b = D.cam_block[cam];
    if (b >= 0)
        for (int a = 0; a < 6; ++a) {
            const double dcv = step_c[6 * b + a];
            e0 = fma(static_cast<double>(rec[a]), dcv, e0);
            e1 = fma(static_cast<double>(rec[nA + a]), dcv, e1);
        }
    const int g = S.ng > 0 ? D.cam_group[cam] : -1;
    if (g >= 0)
        for (int a = 0; a < S.ni; ++a) {
            const double dcv = step_c[6 * S.ncb + g * S.ni + a];
            e0 = fma(static_cast<double>(rec[6 + a]), dcv, e0);
            e1 = fma(static_cast<double>(rec[nA + 6 + a]), dcv, e1);
        }
    const T* Y = rec + 2 * nA;
    double* u = terms + static_cast<size_t>(o) * 3;
    u[0] = static_cast<double>(Y[0]) * e0 + static_cast<double>(Y[3]) * e1;
    u[1] = static_cast<double>(Y[1]) * e0 + static_cast<double>(Y[4]) * e1;
    u[2] = static_cast<double>(Y[2]) * e0 + static_cast<double>(Y[5]) * e1;
}

// track:  dp = R^-T (q - R^-1 u),  u = sum_o w J_p^T (J_o dc).
__global__ void __launch_bounds__(256) k_back_substitute(Shape S, DevPtrs D, const double* __restrict__ trk_data,
                                                         const double* __restrict__ terms,
                                                         double* __restrict__ step_p, double* __restrict__ part) {
    // Point steps dp = V^-1 (g_p - W^T dc) = R^-T (q - sum_o Y_o^T A_o dc) from the records the
    // assembly kept (A = [J_pose | J_intr] rows and Y = w Jp R^-T of every observation), with
    // FP64 accumulation (recoverReferencePointSteps, BundleAdjustPlaMatrixReferenceSchur.cpp:982-1082).
    // The per-observation terms come from k_backsub_terms and are summed here in observation order,
    // the order of a single-thread loop over the track.
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double dd = 0.0, ss = 0.0;
    if (t < S.ntp && D.trk_block[t] >= 0) {
        double u0 = 0.0, u1 = 0.0, u2 = 0.0;
        for (int o = D.trk_obs_begin[t]; o < D.trk_obs_begin[t + 1]; ++o) {
            const double* u = terms + static_cast<size_t>(o) * 3;
            u0 += u[0];
            u1 += u[1];
            u2 += u[2];
        }
        const double* td = trk_data + static_cast<size_t>(t) * kTrackRec;
        const double i00 = td[0], i10 = td[1], i11 = td[2], i20 = td[3], i21 = td[4], i22 = td[5];
        const double v0 = td[6] - u0;
        const double v1 = td[7] - u1;
        const double v2 = td[8] - u2;
        const double p0 = i00 * v0 + i10 * v1 + i20 * v2;
        const double p1 = i11 * v1 + i21 * v2;
        const double p2 = i22 * v2;
        step_p[static_cast<size_t>(t) * 3 + 0] = p0;
        step_p[static_cast<size_t>(t) * 3 + 1] = p1;
        step_p[static_cast<size_t>(t) * 3 + 2] = p2;
        dd = td[9] * p0 + td[10] * p1 + td[11] * p2;
        ss = p0 * p0 + p1 * p1 + p2 * p2;
    } else if (t < S.ntp) {
        step_p[static_cast<size_t>(t) * 3 + 0] = 0.0;
        step_p[static_cast<size_t>(t) * 3 + 1] = 0.0;
        step_p[static_cast<size_t>(t) * 3 + 2] = 0.0;
    }
    __shared__ double s_d[8], s_s[8];
    dd = warp_sum(dd);
    ss = warp_sum(ss);
    if ((threadIdx.x & 31) == 0) {
        s_d[threadIdx.x >> 5] = dd;
        s_s[threadIdx.x >> 5] = ss;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
            a += s_d[w];
            b += s_s[w];
        }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

// Fixed-order sum of block partials (pairs of values) plus the camera-side terms of the
// directional decrease (dc . direct rhs) and of the step RMS.
__global__ void k_backsub_final(Shape S, DevPtrs D, const double* __restrict__ part, int nblocks,
                                const double* __restrict__ step_c, const double* __restrict__ direct64,
                                double* __restrict__ out) {
    __shared__ double s_a[256], s_b[256], s_c[256];
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        a += part[2 * i];
        b += part[2 * i + 1];
    }
    for (int i = threadIdx.x; i < S.n; i += blockDim.x) {
        a += step_c[i] * direct64[i];
        c += step_c[i] * step_c[i];
    }
    s_a[threadIdx.x] = a;
    s_b[threadIdx.x] = b;
    s_c[threadIdx.x] = c;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
            s_a[threadIdx.x] += s_a[threadIdx.x + st];
            s_b[threadIdx.x] += s_b[threadIdx.x + st];
            s_c[threadIdx.x] += s_c[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = s_a[0];  // directional decrease
        out[1] = s_b[0];  // sum of squared point steps
        out[2] = s_c[0];  // sum of squared camera/intrinsic steps
    }
}

// Accept trial `a`: poses and effective cameras from the trial, groups, points += s(X) alpha dp.
__global__ void k_accept(Shape S, DevPtrs D, const double* __restrict__ step_p, double alpha, int a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < S.nc) {
        const double* tr = D.cams_trial + (static_cast<size_t>(a) * S.nc + i) * kCamStride;
        double* st = D.cams_state + static_cast<size_t>(i) * kCamStride;
        double* ef = D.cams_eff + static_cast<size_t>(i) * kCamStride;
        for (int q = 0; q < 12; ++q) st[q] = tr[q];
        for (int q = 0; q < kCamStride; ++q) ef[q] = tr[q];
        camera_ff(tr, D.cams_ff + static_cast<size_t>(i) * kCamFF);
        // the gauge tangent basis follows the accepted state (referenceGaugeTargetTangentBasis is
        // evaluated on the current cameras, BundleAdjustPlaMatrixAssembly.cpp:69-99, :110, :205);
        // read from the trial records, which this kernel does not write
        if (i == S.gauge_scale && S.gauge_anchor >= 0 && S.gauge_baseline > 0.0)
            gauge_basis(D.cams_trial + (static_cast<size_t>(a) * S.nc + S.gauge_anchor) * kCamStride + 9, tr + 9,
                        D.gauge_basis + 6, D.gauge_basis);
    }
    if (i < S.ng * kGroupRec) D.groups[i] = D.groups_trial[static_cast<size_t>(a) * S.ng * kGroupRec + i];
    if (i < S.ntp && D.trk_free[i]) {
        double* X = D.points + static_cast<size_t>(i) * 3;
        const double f = D.pscale[i] * alpha;
        X[0] += f * step_p[static_cast<size_t>(i) * 3 + 0];
        X[1] += f * step_p[static_cast<size_t>(i) * 3 + 1];
        X[2] += f * step_p[static_cast<size_t>(i) * 3 + 2];
        const double sc = S.ref_param ? point_scale(X[0], X[1], X[2]) : 1.0;
        D.pscale[i] = sc;
        D.pscale_ff[i] = ff_pack(sc);
    }
}

// Strict per-track RMS (strictTrackRms, BundleAdjustQuality.cpp:302-364) over the raw observations.
// `proc_of_track` maps an original track to its processing index (-1: use the initial point).
__global__ void k_strict_rms(Shape S, DevPtrs D, const double* __restrict__ cams, const double* __restrict__ init_points,
                             const int* __restrict__ proc_of_track, int use_state, int nt, double* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    double X0, X1, X2;
    const int pidx = use_state ? proc_of_track[t] : -1;
    if (use_state && pidx < 0) { out[t] = __longlong_as_double(0x7ff0000000000000ll); return; }
    if (pidx >= 0) {
        X0 = D.points[3 * pidx]; X1 = D.points[3 * pidx + 1]; X2 = D.points[3 * pidx + 2];
    } else {
        X0 = init_points[3 * t]; X1 = init_points[3 * t + 1]; X2 = init_points[3 * t + 2];
    }
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    if (!isfinite(X0) || !isfinite(X1) || !isfinite(X2)) { out[t] = inf; return; }
    double sum = 0.0;
    int count = 0, first = -1;
    bool second = false;
    for (long long k = D.raw_offsets[t]; k < D.raw_offsets[t + 1]; ++k) {
        const double w = D.raw_w[k];
        if (!(w > 0.0)) continue;
        if (D.raw_bad[k]) { out[t] = inf; return; }
        const int cam = D.raw_cam[k];
        DCam c;
        load_cam(cams + static_cast<size_t>(cam) * kCamStride, c);
        Proj p;
        if (!project64(c, X0, X1, X2, p)) { out[t] = inf; return; }
        const double du = p.px - D.raw_u[k], dv = p.py - D.raw_v[k];
        sum += w * (du * du + dv * dv);
        count += 2;
        if (first < 0) first = cam;
        else if (cam != first) second = true;
    }
    out[t] = (count < 4 || !second) ? inf : sqrt(sum / count);
}

// Per-observation linearisation in the original observation order (parity export of kernel (a)).
template <typename T>
__global__ void k_linearize_export(Shape S, DevPtrs D, double* __restrict__ res, double* __restrict__ jp,
                                   double* __restrict__ jpose, double* __restrict__ ji, double* __restrict__ nw,
                                   double* __restrict__ cost, signed char* __restrict__ valid) {
    const long long o = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (o >= S.nop) return;
    const int cam = D.obs_cam[o], trk = D.obs_trk[o];
    const long long k = D.obs_orig[o];
    DCam c;
    load_cam(D.cams_eff + static_cast<size_t>(cam) * kCamStride, c);
    const double* X = D.points + static_cast<size_t>(trk) * 3;
    const bool tangent = cam == S.gauge_scale && S.gauge_anchor >= 0 && S.gauge_baseline > 0.0;
    Lin<T> L;
    const bool ok = linearize_obs<T>(c, X[0], X[1], X[2], D.pscale[trk], D.obs_u[o], D.obs_v[o], D.obs_w[o], S.loss,
                                     S.loss_scale, tangent, !S.ref_param, D.gauge_basis, S.ni, S.int_cols, true, L);
    valid[k] = ok ? 1 : 0;
    if (!ok) return;
    res[2 * k] = static_cast<double>(L.r0);
    res[2 * k + 1] = static_cast<double>(L.r1);
    for (int i = 0; i < 6; ++i) jp[6 * k + i] = static_cast<double>(L.Jp[i]);
    for (int i = 0; i < 2 * kP; ++i) jpose[2 * kP * k + i] = 0.0;
    if (D.cam_block[cam] >= 0)
        for (int r = 0; r < 2; ++r)
            for (int i = 0; i < 6; ++i) jpose[2 * kP * k + r * kP + i] = static_cast<double>(L.Jc[r * 6 + i]);
    for (int i = 0; i < 2 * kP; ++i) ji[2 * kP * k + i] = 0.0;
    for (int r = 0; r < 2; ++r)
        for (int i = 0; i < S.ni; ++i) ji[2 * kP * k + r * kP + S.int_cols[i]] = static_cast<double>(L.Ji[r * kMaxNI + i]);
    nw[k] = static_cast<double>(L.w);
    cost[k] = L.cost;
    if constexpr (std::is_same<T, float>::value) {
        // the mixed path's weight and gradient chain are float-float (the assembly's phase A);
        // its residual, Jacobians and weight replace the FP64 ones, the cost stays the FP64 one
        Proj pr;
        LinFF F;
        const bool okf = project64(c, X[0], X[1], X[2], pr) &&
                         linearize_obs_ff(pr, D.obs_u[o], D.obs_v[o], D.cams_ff + static_cast<size_t>(cam) * kCamFF,
                                          ffl(D.pscale_ff[trk]), ffl(D.obs_w_ff[o]), S.loss,
                                          ff{S.loss_scale_hi, S.loss_scale_lo}, tangent, !S.ref_param, D.gauge_basis,
                                          S.ni, S.int_cols, F);
        valid[k] = okf ? 1 : 0;
        if (!okf) return;
        res[2 * k] = static_cast<double>(F.r0.hi) + static_cast<double>(F.r0.lo);
        res[2 * k + 1] = static_cast<double>(F.r1.hi) + static_cast<double>(F.r1.lo);
        for (int i = 0; i < 6; ++i) jp[6 * k + i] = static_cast<double>(F.Jp[i]);
        if (D.cam_block[cam] >= 0)
            for (int r = 0; r < 2; ++r)
                for (int i = 0; i < 6; ++i) jpose[2 * kP * k + r * kP + i] = static_cast<double>(F.Jc[r * 6 + i]);
        for (int r = 0; r < 2; ++r)
            for (int i = 0; i < S.ni; ++i)
                ji[2 * kP * k + r * kP + S.int_cols[i]] = static_cast<double>(F.Ji[r * kMaxNI + i]);
        nw[k] = static_cast<double>(F.w.hi) + static_cast<double>(F.w.lo);
    }
}

// ---------------------------------------------------------------- launchers
template <typename T>
static AsmOutT<T> typed(const AsmOut& o) {
    using P = typename Acc<T>::part_type;
    return {static_cast<P*>(o.part_pair_v), static_cast<P*>(o.part_cam_v), static_cast<P*>(o.part_chunk_v),
            o.part_cost, o.part_flags, static_cast<double*>(o.trk_data_v), static_cast<T*>(o.obs_rec_v)};
}

template <typename T>
void launch_reduce_sums(const Shape& S, const DevPtrs& D, const AsmOut& O, const RedOut<double>& R, cudaStream_t st) {
    const AsmOutT<T> P = typed<T>(O);
    ReduceArgs<T> A;
    A.part_pair = P.part_pair;
    A.part_cam = P.part_cam;
    A.part_chunk = P.part_chunk;
    A.part_cost = O.part_cost;
    A.part_flags = O.part_flags;
    A.vals = R.vals;
    A.rhs = R.rhs;
    A.direct = R.direct;
    A.border = R.border;
    A.border_t = R.border_t;
    A.Cm = R.Cm;
    A.result = R.result;
    const long long np = static_cast<long long>(S.nupper) * 36;
    const long long nc = static_cast<long long>(S.ncb) * (12 + S.ng * 6 * S.ni);
    A.pair_blocks = static_cast<unsigned>((np + 255) / 256);
    A.cam_blocks = static_cast<unsigned>((nc + 255) / 256);
    const int chrec = S.nb * S.nb + 2 * S.nb;
    const unsigned chunk_blocks = static_cast<unsigned>((chrec + 31) / 32) + 1;
    k_reduce_sums<T><<<A.pair_blocks + A.cam_blocks + chunk_blocks, 256, 0, st>>>(S, D, A);
}

template <typename T>
void launch_reduce(const Shape& S, const DevPtrs& D, const AsmOut& O, const RedOut<double>& R, double damping,
                   cudaStream_t st) {
    launch_reduce_sums<T>(S, D, O, R, st);
    const int nf = std::max(S.ncb * 6, 1);
    k_finalize<<<(nf + 255) / 256, 256, 0, st>>>(S, D, R.vals, R.Cm, R.rhs + 6 * S.ncb, R.direct + 6 * S.ncb, R.result,
                                                  damping);
}

// The fixed-order sums of FP64 chunk partials of launch_reduce, without the damping and prior
// finalisation (the backward pass finalises its exact Hessian itself).
void launch_reduce_sums64(const Shape& S, const DevPtrs& D, const AsmOut& O, const RedOut<double>& R, cudaStream_t st) {
    launch_reduce_sums<double>(S, D, O, R, st);
}

template <typename T>
void launch_back_substitute(const Shape& S, const DevPtrs& D, const double* trk_data, const T* obs_rec, const double* step_c,
                            double* step_p, double* terms, double* part, const double* direct64, double* out,
                            cudaStream_t st) {
    const int nblk = std::max(1, (S.ntp + 255) / 256);
    if (S.nop > 0)
        k_backsub_terms<T><<<static_cast<unsigned>((S.nop + 255) / 256), 256, 0, st>>>(S, D, obs_rec, step_c, terms);
    k_back_substitute<<<nblk, 256, 0, st>>>(S, D, trk_data, terms, step_p, part);
    k_backsub_final<<<1, 256, 0, st>>>(S, D, part, nblk, step_c, direct64, out);
}

template <typename T>
void launch_linearize_export(const Shape& S, const DevPtrs& D, double* res, double* jp, double* jpose, double* ji,
                             double* nw, double* cost, signed char* valid, cudaStream_t st) {
    if (S.nop == 0) return;
    k_linearize_export<T><<<static_cast<unsigned>((S.nop + 255) / 256), 256, 0, st>>>(S, D, res, jp, jpose, ji, nw, cost,
                                                                                       valid);
}

__global__ void k_gather_obs(long long nop, int ntp, DevPtrs D) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < nop) {
        const int k = D.obs_orig[i];
        D.obs_cam[i] = D.raw_cam[k];
        D.obs_u[i] = D.raw_u[k];
        D.obs_v[i] = D.raw_v[k];
        D.obs_w[i] = D.raw_w[k];
        D.obs_w_ff[i] = ff_pack(D.raw_w[k]);
    }
    if (i < ntp)
        for (int o = D.trk_obs_begin[i]; o < D.trk_obs_begin[i + 1]; ++o) D.obs_trk[o] = static_cast<int>(i);
}

void launch_gather_obs(long long nop, int ntp, const DevPtrs& D, cudaStream_t st) {
    const long long n = std::max<long long>(std::max<long long>(nop, ntp), 1);
    k_gather_obs<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(nop, ntp, D);
}

void launch_effective(const Shape& S, const DevPtrs& D, cudaStream_t st) {
    const int n = std::max(std::max(S.nc, S.ntp), 1);
    k_effective<<<(n + 127) / 128, 128, 0, st>>>(S, D);
}

void launch_cost(const Shape& S, const DevPtrs& D, const double* step_c, const double* step_p, const double* alphas,
                 int n_alpha, int use_trial, double* part, double* out, cudaStream_t st, const RigDev* rig) {
    if (use_trial) {
        const int n = n_alpha * S.nc;
        k_trial_cameras<<<(n + 127) / 128, 128, 0, st>>>(S, D, step_c, alphas, n_alpha);
        // rig cameras: poses composed from the trial captures and sensors
        if (rig) launch_rig_trial(*rig, S.nc, alphas, n_alpha, D.cams_trial, st);
    }
    const int nblk = static_cast<int>(std::max<long long>(1, (S.nop + 255) / 256));
    k_cost_batch<<<nblk, 256, 0, st>>>(S, D, step_p, alphas, n_alpha, use_trial, part);
    k_cost_final<<<1, 256, 0, st>>>(S, D, part, nblk, n_alpha, use_trial, out);
}

void launch_accept(const Shape& S, const DevPtrs& D, const double* step_p, double alpha, int a, cudaStream_t st) {
    const int n = std::max(std::max(S.nc, S.ntp), S.ng * kGroupRec);
    k_accept<<<(n + 255) / 256, 256, 0, st>>>(S, D, step_p, alpha, a);
}

void launch_strict_rms(const Shape& S, const DevPtrs& D, const double* cams, const double* init_points,
                       const int* proc_of_track, int use_state, int nt, double* out, cudaStream_t st) {
    k_strict_rms<<<(nt + 255) / 256, 256, 0, st>>>(S, D, cams, init_points, proc_of_track, use_state, nt, out);
}

// ---------------------------------------------------------------- quality finalisation
// finalizeBundleAdjustResult (BundleAdjustQuality.cpp:403-502) on the device: the strict RMS
// after the solve of every active track, the filter threshold max(filterMaxReprojError,
// filterSigmaFactor * median of the finite RMS values), the valid mask and the mean RMS of the
// kept tracks.  The median is an exact order statistic (radix select over the bit patterns of
// the non-negative doubles, which order like their values), the mean of the two middle values
// for an even count, as the host's finite median.

constexpr int kQualityThreads = 1024;

__device__ __forceinline__ bool quality_candidate(const signed char* active, const double* rms, int t) {
    return active[t] && isfinite(rms[t]);
}

// k-th smallest (0-based) candidate value, by eight 8-bit radix passes; all threads take part
__device__ double quality_select(int nt, const signed char* active, const double* rms, unsigned long long k,
                                 unsigned int* hist, unsigned long long* s_prefix, unsigned long long* s_rank) {
    unsigned long long prefix = 0ull, mask = 0ull;
    if (threadIdx.x == 0) *s_rank = k;
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = 56 - 8 * pass;
        for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0u;
        __syncthreads();
        for (int t = threadIdx.x; t < nt; t += blockDim.x) {
            if (!quality_candidate(active, rms, t)) continue;
            const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(rms[t]));
            if ((bits & mask) == prefix) atomicAdd(&hist[(bits >> shift) & 255ull], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long r = *s_rank, before = 0ull;
            int b = 0;
            for (; b < 255; ++b) {
                if (before + hist[b] > r) break;
                before += hist[b];
            }
            *s_rank = r - before;
            *s_prefix = prefix | (static_cast<unsigned long long>(b) << shift);
        }
        __syncthreads();
        prefix = *s_prefix;
        mask |= 255ull << shift;
        __syncthreads();
    }
    return __longlong_as_double(static_cast<long long>(prefix));
}

// one CTA: out[0] = threshold, out[1] = candidate count
__global__ void __launch_bounds__(kQualityThreads) k_quality_threshold(int nt, const signed char* __restrict__ active,
                                                                       const double* __restrict__ rms, int enable,
                                                                       double max_err, double sigma,
                                                                       double* __restrict__ out) {
    __shared__ unsigned int hist[256];
    __shared__ unsigned long long s_prefix, s_rank;
    __shared__ int s_count[kQualityThreads / 32];
    int cnt = 0;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) cnt += quality_candidate(active, rms, t) ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) s_count[threadIdx.x >> 5] = cnt;
    __syncthreads();
    long long n = 0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) n += s_count[w];
    double thr = __longlong_as_double(0x7ff0000000000000ll);
    if (enable) {
        thr = isfinite(max_err) && max_err >= 0.0 ? max_err : 0.0;
        if (n > 0 && isfinite(sigma) && sigma > 0.0) {
            const unsigned long long h = static_cast<unsigned long long>(n / 2);
            const double upper = quality_select(nt, active, rms, h, hist, &s_prefix, &s_rank);
            double med = upper;
            if ((n & 1) == 0) med = 0.5 * (quality_select(nt, active, rms, h - 1, hist, &s_prefix, &s_rank) + upper);
            thr = fmax(thr, sigma * med);
        }
    }
    if (threadIdx.x == 0) {
        out[0] = thr;
        out[1] = static_cast<double>(n);
    }
}

// valid mask and per-block partials (kept, sum RMS before, sum RMS after)
__global__ void __launch_bounds__(256) k_quality_filter(int nt, const signed char* __restrict__ active,
                                                        const double* __restrict__ rms_before,
                                                        const double* __restrict__ rms_after,
                                                        const double* __restrict__ thr_in, signed char* __restrict__ valid,
                                                        double* __restrict__ part) {
    __shared__ double s[3][8];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double k = 0.0, b = 0.0, a = 0.0;
    if (t < nt) {
        const double thr = thr_in[0];
        const bool v = quality_candidate(active, rms_after, t) && !(rms_after[t] > thr);
        valid[t] = v ? 1 : 0;
        if (v) {
            k = 1.0;
            b = rms_before[t];
            a = rms_after[t];
        }
    }
    const double w[3] = {warp_sum(k), warp_sum(b), warp_sum(a)};
    if ((threadIdx.x & 31) == 0)
        for (int i = 0; i < 3; ++i) s[i][threadIdx.x >> 5] = w[i];
    __syncthreads();
    if (threadIdx.x < 3) {
        double acc = 0.0;
        for (int i = 0; i < 8; ++i) acc += s[threadIdx.x][i];
        part[static_cast<size_t>(blockIdx.x) * 3 + threadIdx.x] = acc;
    }
}

// fixed-order sums of the block partials into out[2..4]
__global__ void k_quality_sums(int nblocks, const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double s[3][256];
    for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc += part[static_cast<size_t>(b) * 3 + i];
        s[i][threadIdx.x] = acc;
    }
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st)
            for (int i = 0; i < 3; ++i) s[i][threadIdx.x] += s[i][threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x < 3) out[2 + threadIdx.x] = s[threadIdx.x][0];
}

size_t quality_part_size(int nt) { return static_cast<size_t>(std::max(1, (nt + 255) / 256)) * 3; }

void launch_quality(int nt, const signed char* active, const double* rms_before, const double* rms_after, int enable,
                    double max_err, double sigma, signed char* valid, double* part, double* out, cudaStream_t st) {
    k_quality_threshold<<<1, kQualityThreads, 0, st>>>(nt, active, rms_after, enable, max_err, sigma, out);
    const int nblk = std::max(1, (nt + 255) / 256);
    k_quality_filter<<<nblk, 256, 0, st>>>(nt, active, rms_before, rms_after, out, valid, part);
    k_quality_sums<<<1, 256, 0, st>>>(nblk, part, out);
}


template void launch_reduce<float>(const Shape&, const DevPtrs&, const AsmOut&, const RedOut<double>&, double,
                                   cudaStream_t);
template void launch_reduce<double>(const Shape&, const DevPtrs&, const AsmOut&, const RedOut<double>&, double,
                                    cudaStream_t);
template void launch_back_substitute<float>(const Shape&, const DevPtrs&, const double*, const float*, const double*,
                                            double*, double*, double*, const double*, double*, cudaStream_t);
template void launch_back_substitute<double>(const Shape&, const DevPtrs&, const double*, const double*, const double*,
                                             double*, double*, double*, const double*, double*, cudaStream_t);
template void launch_linearize_export<float>(const Shape&, const DevPtrs&, double*, double*, double*, double*, double*,
                                             double*, signed char*, cudaStream_t);
template void launch_linearize_export<double>(const Shape&, const DevPtrs&, double*, double*, double*, double*,
                                              double*, double*, signed char*, cudaStream_t);

}  // namespace pb
