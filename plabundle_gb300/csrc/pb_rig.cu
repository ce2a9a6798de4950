// pb_rig.cu -- rig problems: capture / sensor chaining of the camera poses.
//
// The reference chains the Jacobian of a rig camera to its capture and sensor blocks
// (cameraPosePrimaryTerms, BundleAdjustPlaMatrixAssembly.cpp:207-284) with the lever
// L = R_rig c_sensor:
//   capture block: rotation column a = J_rot[a] + J_ctr (e_a x L), centre column a = J_ctr[a];
//   sensor block:  rotation / centre column a = J_rot R_rig[:, a] / J_ctr R_rig[:, a].
// Both are linear maps of the camera's own pose Jacobian: J_capture = J_camera Mc, J_sensor =
// J_camera Ms with
//   Mc = [[I, 0], [-[L]x, I]],   Ms = [[R_rig, 0], [0, R_rig]]   (camera delta = M rig delta).
// The point elimination commutes with a linear change of the primary parameters, so the fused
// assembly runs unchanged on one 6-column block per camera (the kernels' camera blocks) and the
// reduced system over the rig's blocks is S_rig[I][J] = sum M_aI^T S[a][b] M_bJ over the camera
// blocks a, b chained to I and J, B_rig[I] = sum M_aI^T B[a], g_rig[I] = sum M_aI^T g[a].  The
// sums follow host-built term lists in a fixed order: the pose terms of one rig block in
// segments of kRigSegTerms consecutive terms (one warp each), then the segments in order; the
// border and right-hand side over segments of kRigItemSeg camera blocks likewise.  The rig pose
// diagonal is then damped as finalizePrimaryDiagonal(1 + damping, 1) damps every primary
// diagonal, the solution is mapped
// back to the camera blocks (camera delta = Mc capture delta + Ms sensor delta) for the point
// back-substitution, and the trial states update captures and sensors with the plain pose delta
// (placamera::applyPoseDelta, BundleAdjustPlaMatrixAssembly.cpp:1152-1209: R' = Exp(w) R,
// C' = C + dC) and compose the cameras again (R = R_rig R_sensor, C = C_rig + R_rig c_sensor).
#include <cuda_runtime.h>

#include "pb_kernels.h"

namespace pb {

namespace {

// R' = Exp(alpha w) R (Rodrigues), C' = C + alpha dC; d = (w, dC).
__device__ void pose_delta(const double* __restrict__ in, const double* __restrict__ d, double alpha,
                           double* __restrict__ out) {
    const double w0 = alpha * d[0], w1 = alpha * d[1], w2 = alpha * d[2];
    const double th2 = w0 * w0 + w1 * w1 + w2 * w2;
    double A, B;
    if (th2 < 1e-16) {
        A = 1.0 - th2 / 6.0;
        B = 0.5 - th2 / 24.0;
    } else {
        const double th = sqrt(th2), sh = sin(0.5 * th);
        A = sin(th) / th;
        B = 2.0 * sh * sh / th2;
    }
    const double K[9] = {0.0, -w2, w1, w2, 0.0, -w0, -w1, w0, 0.0};
    double E[9];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) {
            const double kk = K[r * 3] * K[q] + K[r * 3 + 1] * K[3 + q] + K[r * 3 + 2] * K[6 + q];
            E[r * 3 + q] = (r == q ? 1.0 : 0.0) + A * K[r * 3 + q] + B * kk;
        }
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) out[r * 3 + q] = E[r * 3] * in[q] + E[r * 3 + 1] * in[3 + q] + E[r * 3 + 2] * in[6 + q];
    for (int i = 0; i < 3; ++i) out[9 + i] = in[9 + i] + alpha * d[3 + i];
}

// Trial record of capture k (or sensor s): the state moved by its block's step, or the state.
__device__ void rig_trial_record(const double* __restrict__ state, int block, const double* __restrict__ step_r,
                                 double alpha, double* __restrict__ out) {
    if (block >= 0) {
        pose_delta(state, step_r + 6 * block, alpha, out);
    } else {
        for (int i = 0; i < 12; ++i) out[i] = state[i];
    }
}

__global__ void k_rig_maps(RigDev R) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= R.ncb) return;
    const int c = R.cb_camera[a];
    const double* cp = R.cap_state + static_cast<size_t>(R.cam_capture[c]) * 12;
    const double* sp = R.sen_state + static_cast<size_t>(R.cam_sensor[c]) * 12;
    double L[3];
    for (int r = 0; r < 3; ++r) L[r] = cp[r * 3] * sp[9] + cp[r * 3 + 1] * sp[10] + cp[r * 3 + 2] * sp[11];
    double* Mc = R.maps + static_cast<size_t>(a) * 72;
    double* Ms = Mc + 36;
    for (int i = 0; i < 36; ++i) Mc[i] = Ms[i] = 0.0;
    for (int i = 0; i < 6; ++i) Mc[i * 7] = 1.0;
    // rows 3-5, columns 0-2: -[L]x (column a is e_a x L)
    Mc[3 * 6 + 1] = L[2];
    Mc[3 * 6 + 2] = -L[1];
    Mc[4 * 6 + 0] = -L[2];
    Mc[4 * 6 + 2] = L[0];
    Mc[5 * 6 + 0] = L[1];
    Mc[5 * 6 + 1] = -L[0];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) {
            Ms[r * 6 + q] = cp[r * 3 + q];
            Ms[(3 + r) * 6 + 3 + q] = cp[r * 3 + q];
        }
}

// Pose blocks, first pass: one warp per segment of at most kRigSeg terms of one upper rig block.
// Per term (camera-block CSR entry p = (a, b) and the sides of its chains) the warp forms
// Y = S_ab M_b in shared memory and Z = M_a^T Y, and keeps the running sum of Z over the segment's
// terms in order (lane e holds entries e and e + 32 of the 6x6 block); the partial goes to
// seg_part[segment].
__global__ void __launch_bounds__(256) k_rig_segments(RigDev R, const double* __restrict__ vals) {
    __shared__ double sY[8][36];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int seg = blockIdx.x * 8 + warp;
    if (seg >= R.nseg) return;
    double* Y = sY[warp];
    const int t0 = R.seg_begin[seg], t1 = R.seg_begin[seg + 1];
    const int e0 = lane, e1 = lane + 32;  // entries (row-major 6x6); e1 valid for lanes 0-3
    double acc0 = 0.0, acc1 = 0.0;
    for (int t = t0; t < t1; ++t) {
        const int p = R.terms[2 * t], code = R.terms[2 * t + 1];
        const int a = code >> 2, b = R.cb_col_idx[p];
        const double* Ma = R.maps + static_cast<size_t>(a) * 72 + ((code >> 1) & 1) * 36;
        const double* Mb = R.maps + static_cast<size_t>(b) * 72 + (code & 1) * 36;
        const double* Sb = vals + static_cast<size_t>(p) * 36;
        // Y[k][q] = sum_l S[k][l] Mb[l][q] over the non-zero entries of the map: Mc has the unit
        // diagonal and -[L]x in rows 3-5 / columns 0-2, Ms the rotation twice on its diagonal
        const bool b_sensor = code & 1, a_sensor = (code >> 1) & 1;
        for (int e = lane; e < 36; e += 32) {
            const int k = e / 6, q = e - 6 * (e / 6);
            double v;
            if (!b_sensor) {
                v = Sb[k * 6 + q];
                if (q < 3)
                    for (int j = 0; j < 3; ++j) v += Sb[k * 6 + 3 + j] * Mb[(3 + j) * 6 + q];
            } else {
                const int o = q < 3 ? 0 : 3;
                v = 0.0;
                for (int j = 0; j < 3; ++j) v += Sb[k * 6 + o + j] * Mb[(o + j) * 6 + q];
            }
            Y[e] = v;
        }
        __syncwarp();
        // Z[r][q] = sum_k Ma[k][r] Y[k][q], likewise
        for (int h = 0; h < 2; ++h) {
            const int e = h == 0 ? e0 : e1;
            if (e >= 36) break;
            const int r = e / 6, q = e - 6 * (e / 6);
            double v;
            if (!a_sensor) {
                v = Y[r * 6 + q];
                if (r < 3)
                    for (int j = 0; j < 3; ++j) v += Ma[(3 + j) * 6 + r] * Y[(3 + j) * 6 + q];
            } else {
                const int o = r < 3 ? 0 : 3;
                v = 0.0;
                for (int j = 0; j < 3; ++j) v += Ma[(o + j) * 6 + r] * Y[(o + j) * 6 + q];
            }
            if (h == 0) acc0 += v;
            else acc1 += v;
        }
        __syncwarp();
    }
    double* out = R.seg_part + static_cast<size_t>(seg) * 36;
    out[e0] = acc0;
    if (e1 < 36) out[e1] = acc1;
}

// Pose blocks, second pass: one thread per entry of an upper rig block sums its segments in order,
// damps the diagonal (finalizePrimaryDiagonal(1 + damping, 1)) and writes both orientations.
__global__ void k_rig_pose_sum(RigDev R, double damping) {
    const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= static_cast<long long>(R.nup) * 36) return;
    const int u = static_cast<int>(e / 36), rq = static_cast<int>(e - 36LL * u);
    const int r = rq / 6, q = rq - 6 * (rq / 6);
    double v = 0.0;
    for (int g = R.up_seg_begin[u]; g < R.up_seg_begin[u + 1]; ++g) v += R.seg_part[static_cast<size_t>(g) * 36 + rq];
    const int tp = R.up_tpos[u];
    if (tp < 0 && r == q) v = v != 0.0 ? v * (1.0 + damping) : 1.0;
    R.vals[static_cast<size_t>(R.up_pos[u]) * 36 + rq] = v;
    if (tp >= 0) R.vals[static_cast<size_t>(tp) * 36 + q * 6 + r] = v;
}

// Border rows and right-hand side, first pass: one warp per (segment of at most kRigItemSeg
// camera blocks chained to one rig block, row r of that block); the lanes take the border columns
// and, as column nbw, the right-hand side, and sum M_a[:, r]^T B[a] over the segment's camera
// blocks in order into bpart[segment][r][column].
__global__ void __launch_bounds__(256) k_rig_border_seg(RigDev R, const double* __restrict__ border,
                                                        const double* __restrict__ rhs, int nbw) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (gw >= R.nbseg * 6) return;
    const int g = gw / 6, r = gw - 6 * (gw / 6);
    const int w = nbw + 1;
    const int t0 = R.bseg_begin[g], t1 = R.bseg_begin[g + 1];
    for (int j = lane; j < w; j += 32) {
        double v = 0.0;
        for (int t = t0; t < t1; ++t) {
            const int code = R.blk_items[t], a = code >> 1;
            const double* M = R.maps + static_cast<size_t>(a) * 72 + (code & 1) * 36;
            if (j < nbw) {
                for (int k = 0; k < 6; ++k) v += M[k * 6 + r] * border[static_cast<size_t>(6 * a + k) * nbw + j];
            } else {
                for (int k = 0; k < 6; ++k) v += M[k * 6 + r] * rhs[6 * a + k];
            }
        }
        R.bpart[(static_cast<size_t>(g) * 6 + r) * w + j] = v;
    }
}

// Second pass: one thread per border entry and rhs entry of a rig block sums its segments in
// order; the right-hand side's group and promoted-point entries are copied.
__global__ void k_rig_border_sum(RigDev R, const double* __restrict__ rhs, int nbw) {
    const int w = nbw + 1;
    const long long nA = 6LL * R.nrb * w;
    const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e < nA) {
        const int row = static_cast<int>(e / w), j = static_cast<int>(e - static_cast<long long>(row) * w);
        const int I = row / 6, r = row - 6 * I;
        double v = 0.0;
        for (int g = R.blk_seg_begin[I]; g < R.blk_seg_begin[I + 1]; ++g)
            v += R.bpart[(static_cast<size_t>(g) * 6 + r) * w + j];
        if (j < nbw) {
            R.border[static_cast<size_t>(row) * nbw + j] = v;
            R.border_t[static_cast<size_t>(j) * (6 * R.nrb) + row] = v;
        } else {
            R.rhs[row] = v;
        }
    } else if (e < nA + nbw) {
        const int i = static_cast<int>(e - nA);
        R.rhs[6 * R.nrb + i] = rhs[6 * R.ncb + i];
    }
}

__global__ void k_rig_expand(RigDev R, const double* __restrict__ xr, int nbw) {
    const int n6 = 6 * R.ncb, nr6 = 6 * R.nrb;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nr6 + nbw) R.step_r[i] = xr[i];
    if (i >= n6 + nbw) return;
    if (i >= n6) {
        R.xv[i] = xr[nr6 + (i - n6)];
        return;
    }
    const int a = i / 6, k = i - 6 * a;
    const double* Mc = R.maps + static_cast<size_t>(a) * 72;
    const double* Ms = Mc + 36;
    double v = 0.0;
    const int cb = R.cb_cap[a], sb = R.cb_sen[a];
    if (cb >= 0)
        for (int r = 0; r < 6; ++r) v += Mc[k * 6 + r] * xr[6 * cb + r];
    if (sb >= 0)
        for (int r = 0; r < 6; ++r) v += Ms[k * 6 + r] * xr[6 * sb + r];
    R.xv[i] = v;
}

// Squared sum of the rig step in a fixed order (one block).
__global__ void k_rig_step_sq(RigDev R, const double* __restrict__ xr, int n) {
    __shared__ double s[256];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += xr[i] * xr[i];
    s[threadIdx.x] = v;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) R.sq[0] = s[0];
}

__global__ void k_rig_trial(RigDev R, int nc, const double* __restrict__ alphas, int n_alpha,
                            double* __restrict__ cams_trial) {
    const int per = R.ncap + R.nsen + nc;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= per * n_alpha) return;
    const int a = idx / per, i = idx - a * per;
    const double alpha = alphas[a];
    if (i < R.ncap) {
        rig_trial_record(R.cap_state + static_cast<size_t>(i) * 12, R.capture_block[i], R.step_r, alpha,
                         R.cap_trial + (static_cast<size_t>(a) * R.ncap + i) * 12);
    } else if (i < R.ncap + R.nsen) {
        const int s = i - R.ncap;
        rig_trial_record(R.sen_state + static_cast<size_t>(s) * 12, R.sensor_block[s], R.step_r, alpha,
                         R.sen_trial + (static_cast<size_t>(a) * R.nsen + s) * 12);
    } else {
        const int c = i - R.ncap - R.nsen;
        const int k = R.cam_capture[c], s = R.cam_sensor[c];
        double cp[12], sp[12];
        rig_trial_record(R.cap_state + static_cast<size_t>(k) * 12, R.capture_block[k], R.step_r, alpha, cp);
        rig_trial_record(R.sen_state + static_cast<size_t>(s) * 12, R.sensor_block[s], R.step_r, alpha, sp);
        double* out = cams_trial + (static_cast<size_t>(a) * nc + c) * kCamStride;
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q)
                out[r * 3 + q] = cp[r * 3] * sp[q] + cp[r * 3 + 1] * sp[3 + q] + cp[r * 3 + 2] * sp[6 + q];
        for (int r = 0; r < 3; ++r)
            out[9 + r] = cp[9 + r] + cp[r * 3] * sp[9] + cp[r * 3 + 1] * sp[10] + cp[r * 3 + 2] * sp[11];
    }
}

__global__ void k_rig_accept(RigDev R, int a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < R.ncap * 12) R.cap_state[i] = R.cap_trial[static_cast<size_t>(a) * R.ncap * 12 + i];
    if (i < R.nsen * 12) R.sen_state[i] = R.sen_trial[static_cast<size_t>(a) * R.nsen * 12 + i];
}

}  // namespace

void launch_rig_maps(const RigDev& R, cudaStream_t st) {
    if (R.ncb > 0) k_rig_maps<<<(R.ncb + 127) / 128, 128, 0, st>>>(R);
}

void launch_rig_transform(const RigDev& R, const double* vals, const double* border, const double* rhs, int nbw,
                          double damping, cudaStream_t st) {
    if (R.nseg > 0) k_rig_segments<<<(R.nseg + 7) / 8, 256, 0, st>>>(R, vals);
    const long long nu = static_cast<long long>(R.nup) * 36;
    if (nu > 0) k_rig_pose_sum<<<static_cast<unsigned>((nu + 255) / 256), 256, 0, st>>>(R, damping);
    if (R.nbseg > 0) k_rig_border_seg<<<(R.nbseg * 6 + 7) / 8, 256, 0, st>>>(R, border, rhs, nbw);
    const long long tot = 6LL * R.nrb * (nbw + 1) + nbw;
    if (tot > 0) k_rig_border_sum<<<static_cast<unsigned>((tot + 255) / 256), 256, 0, st>>>(R, rhs, nbw);
}

void launch_rig_expand(const RigDev& R, const double* xr, int nbw, int nglob, cudaStream_t st) {
    const int n = std::max(6 * R.ncb, 6 * R.nrb) + nbw;
    k_rig_expand<<<(n + 255) / 256, 256, 0, st>>>(R, xr, nbw);
    k_rig_step_sq<<<1, 256, 0, st>>>(R, xr, 6 * R.nrb + nglob);
}

void launch_rig_trial(const RigDev& R, int nc, const double* alphas, int n_alpha, double* cams_trial, cudaStream_t st) {
    const int n = (R.ncap + R.nsen + nc) * n_alpha;
    k_rig_trial<<<(n + 127) / 128, 128, 0, st>>>(R, nc, alphas, n_alpha, cams_trial);
}

void launch_rig_accept(const RigDev& R, int a, cudaStream_t st) {
    const int n = 12 * std::max(R.ncap, R.nsen);
    k_rig_accept<<<(n + 255) / 256, 256, 0, st>>>(R, a);
}

}  // namespace pb
