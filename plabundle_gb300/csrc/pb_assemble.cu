// pb_assemble.cu -- kernels (a)+(b): per-observation linearisation and online point Schur
// elimination into the block-sparse reduced camera system.
//
// One CTA of 256 threads per chunk of consecutive tracks (host-built: at most max_obs <= 256
// observations and max_tracks tracks), one thread per observation in phases A-C:
//   A. linearise the observation: residual, robust weight and gradient in FP64 with the cost on
//      the FP64 path, in float-float without the cost on the mixed path (FP64 runs at a small
//      fraction of the FP32 rate on this part; the LM takes the mixed path's FP64 cost from the
//      line search); Jacobians A = [J_pose | J_intr] and Jp in T (FP32 on the mixed path);
//   B. per track, V = sum w Jp^T Jp and the point gradient in FP64 and the factor V = R R^T
//      (the 3x3 point block inverse of BundleAdjustPlaMatrixReferenceSchur.cpp:350-490);
//   C. per observation, in FP64: Y = w Jp R^-T (2x3), the reduced weight M = w I - Y Y^T and Y q
//      (q = R^-1 g_p); then G = J_pose^T Y.  The matrix derives from the rounded Jacobians only,
//      so it is the exact Schur complement of one consistently perturbed linearisation (the
//      FP32 rounding of a Jacobian perturbs the weakest mode of S by ~eps*sqrt(cond), rounding
//      S itself by eps*cond).  The gradient g = -J^T w r does not carry the Jacobians' rounding
//      (FP64 or float-float, see linearize_obs / linearize_obs_ff): the rounded Jacobians shape
//      the step, never the fixed point;
//   K. per track and calibration group, K = sum over the group's observations of J_intr^T Y;
//   D. every output element of the chunk is owned by one thread, which gathers its terms in a
//      fixed order into compensated accumulators and writes the chunk partial once (which
//      thread owns which row is a host-built schedule that balances the warps' loads):
//        pose block (a, b):  sum_o J^T M J (own terms)  -  sum_(o != o') G_o G_o'^T
//        border (c, g):      sum_(o in c, g) w J_pose^T J_intr  -  sum_(o in c) G_o K_(t(o), g)^T
//        intrinsic (g, g'):  sum_(o in g) w J_intr^T J_intr  -  sum_t K_(t,g) K_(t,g')^T
//        rhs:                sum_o g_o - J^T Y q  (and the direct gradient sum_o g_o)
//      (the own term J^T M J plus the observation's own G G^T is w J^T J).  No atomics; the
//      result is deterministic.
// On the FP32 path all products and sums of D run in float-float arithmetic (exact FMA product
// residuals, two-sum accumulation): ~44 significant bits on the FP32 pipe, enough for reduced
// matrices of condition ~1e9, where FP32 products alone leave the weakest modes indefinite.
#include <cuda_runtime.h>

#include <type_traits>

#include "pb_device.cuh"
#include "pb_kernels.h"

namespace pb {

namespace {

template <typename T>
__device__ __forceinline__ T* carve(char*& ptr, size_t count) {
    T* out = reinterpret_cast<T*>(ptr);
    ptr += (count * sizeof(T) + 15) & ~static_cast<size_t>(15);
    return out;
}

constexpr int kOk = 1, kElim = 2;
__device__ __forceinline__ int info_group(int info) { return ((info >> 2) & 7) - 1; }
// per-observation track record: first observation (8 bits) | chunk track slot (8) | length (16)
__device__ __forceinline__ int trk_slot(int v) { return (v >> 8) & 0xFF; }

}  // namespace

template <typename T>
__global__ void __launch_bounds__(256, 2) k_assemble(Shape S, DevPtrs D, AsmOutT<T> O, double damping) {
    using P = typename Acc<T>::part_type;
    using Val = ValueOf<T>;
    using VT = typename Val::type;
    extern __shared__ __align__(16) char smem[];
    const int chunk = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int MO = S.max_obs, MT = S.max_tracks;
    const int ng = S.ng, ni = S.ni, nb = S.nb, nA = 6 + ni;
    // per-observation records are padded to an odd number of 4- or 8-byte words, so that the
    // lanes of a warp reading the same field of consecutive observations hit distinct banks
    const int sA = chunk_stride(2 * nA), sG = chunk_stride(18), sY = chunk_stride(6), sM = chunk_stride(6),
              sD = chunk_stride(nA);
    char* ptr = smem;
    double* s_V = carve<double>(ptr, static_cast<size_t>(MO) * 9);  // point normal terms, then the track factor
    T* s_A = carve<T>(ptr, static_cast<size_t>(MO) * sA);
    VT* s_G = carve<VT>(ptr, static_cast<size_t>(MO) * sG);
    VT* s_Y = carve<VT>(ptr, static_cast<size_t>(MO) * sY);
    VT* s_M = carve<VT>(ptr, static_cast<size_t>(MO) * sM);
    VT* s_D = carve<VT>(ptr, static_cast<size_t>(MO) * sD);
    int* s_info = carve<int>(ptr, MO);
    int* s_trk = carve<int>(ptr, MO);
    const int sK = chunk_stride(nb * 3);  // per-track K record (odd: lanes over tracks hit distinct banks)
    VT* s_K = carve<VT>(ptr, static_cast<size_t>(MT) * sK);
    int* s_tfirst = carve<int>(ptr, MT + 1);
    int* s_tmask = carve<int>(ptr, MT);  // calibration groups present in each chunk track
    double* s_cpc = carve<double>(ptr, MT);  // control-point cost of each chunk track
    double* s_misc = carve<double>(ptr, 40);
    int* s_flags = reinterpret_cast<int*>(s_misc + 32);
    int* s_wcount = reinterpret_cast<int*>(s_misc + 34);
    int* s_next_entry = reinterpret_cast<int*>(s_misc + 38);  // next intrinsic entry to take

    const int obs0 = D.ch_obs_begin[chunk], nobs = D.ch_obs_begin[chunk + 1] - obs0;
    if (tid == 0) {
        s_flags[0] = 0;
        s_next_entry[0] = 0;
    }
    __syncthreads();

    // ---- A: linearise one observation per thread; FP64 point normal equations
    const bool active = tid < nobs;
    const int o = obs0 + tid;
    Lin<T> L;
    double grad[9 + kMaxNI];
    double cost = 0.0;
    double w64 = 0.0;  // normal weight (FP64 value of the float-float weight on the mixed path)
    T jpT[6];          // point Jacobian of the arithmetic type
    int first = 0, k = 0;
    bool elim = false, ok = false;
    constexpr bool kMixed = std::is_same<T, float>::value;
    if constexpr (kMixed) {
        if (active) {
            // mixed path: FP64 projection, float-float weight and gradient (no cost: the LM takes it
            // from the line search)
            const int cam = D.obs_cam[o];
            const int trk = D.obs_trk[o];
            const int tb0 = D.trk_obs_begin[trk];
            first = tb0 - obs0;
            k = D.trk_obs_begin[trk + 1] - tb0;
            elim = D.trk_block[trk] >= 0;
            const int grp = ng > 0 ? D.cam_group[cam] : -1;
            const bool tangent = cam == S.gauge_scale && S.gauge_anchor >= 0 && S.gauge_baseline > 0.0;
            DCam c;
            load_cam(D.cams_eff + static_cast<size_t>(cam) * kCamStride, c);
            const double* X = D.points + static_cast<size_t>(trk) * 3;
            Proj pr;
            LinFF F;
            ok = project64(c, X[0], X[1], X[2], pr) &&
                 linearize_obs_ff(pr, D.obs_u[o], D.obs_v[o], D.cams_ff + static_cast<size_t>(cam) * kCamFF,
                                  ffl(D.pscale_ff[trk]), ffl(D.obs_w_ff[o]), S.loss,
                                  ff{S.loss_scale_hi, S.loss_scale_lo}, tangent, !S.ref_param, D.gauge_basis, ni,
                                  S.int_cols, F);
            if (!ok) atomicOr(s_flags, 2);
            s_info[tid] = (ok ? kOk : 0) | (elim ? kElim : 0) | ((grp + 1) << 2);
            T* A = s_A + static_cast<size_t>(tid) * sA;
            for (int a = 0; a < 6; ++a) {
                A[a] = ok ? F.Jc[a] : T(0);
                A[nA + a] = ok ? F.Jc[6 + a] : T(0);
            }
            for (int a = 0; a < ni; ++a) {
                A[6 + a] = ok ? F.Ji[a] : T(0);
                A[nA + 6 + a] = ok ? F.Ji[kMaxNI + a] : T(0);
            }
            VT* Dg = s_D + static_cast<size_t>(tid) * sD;
            for (int a = 0; a < 6; ++a) Dg[a] = ok ? F.g[a] : Val::zero();
            for (int a = 0; a < ni; ++a) Dg[6 + a] = ok ? F.g[9 + a] : Val::zero();
            // the point block, its factor and the projector of phases B and C stay in FP64: the
            // reduced weight M = w I - Y Y^T cancels to a small fraction of w, and the weakest modes
            // of the reduced matrix need its FP64 rounding
            double* V = s_V + static_cast<size_t>(tid) * 9;
            w64 = static_cast<double>(F.w.hi) + static_cast<double>(F.w.lo);
            for (int i = 0; i < 6; ++i) jpT[i] = F.Jp[i];
            if (elim && ok) {
                // V_o = w Jp^T Jp from the rounded Jacobian and the point gradient
                const double w = w64;
                const double j0 = F.Jp[0], j1 = F.Jp[1], j2 = F.Jp[2], j3 = F.Jp[3], j4 = F.Jp[4], j5 = F.Jp[5];
                V[0] = w * (j0 * j0 + j3 * j3);
                V[1] = w * (j0 * j1 + j3 * j4);
                V[2] = w * (j0 * j2 + j3 * j5);
                V[3] = w * (j1 * j1 + j4 * j4);
                V[4] = w * (j1 * j2 + j4 * j5);
                V[5] = w * (j2 * j2 + j5 * j5);
                for (int i = 0; i < 3; ++i)
                    V[6 + i] = static_cast<double>(F.g[6 + i].hi) + static_cast<double>(F.g[6 + i].lo);
            } else {
                for (int i = 0; i < 9; ++i) V[i] = 0.0;
            }
        }
    } else {
        if (active) {
            const int cam = D.obs_cam[o];
            const int trk = D.obs_trk[o];
            const int tb0 = D.trk_obs_begin[trk];
            first = tb0 - obs0;
            k = D.trk_obs_begin[trk + 1] - tb0;
            elim = D.trk_block[trk] >= 0;
            const int grp = ng > 0 ? D.cam_group[cam] : -1;
            DCam c;
            load_cam(D.cams_eff + static_cast<size_t>(cam) * kCamStride, c);
            const double* X = D.points + static_cast<size_t>(trk) * 3;
            const bool tangent = cam == S.gauge_scale && S.gauge_anchor >= 0 && S.gauge_baseline > 0.0;
            ok = linearize_obs<T>(c, X[0], X[1], X[2], D.pscale[trk], D.obs_u[o], D.obs_v[o], D.obs_w[o], S.loss,
                                  S.loss_scale, tangent, !S.ref_param, D.gauge_basis, ni, S.int_cols, true, L, grad);
            if (!ok) {
                atomicOr(s_flags, 2);
            } else {
                cost = L.cost;
            }
            s_info[tid] = (ok ? kOk : 0) | (elim ? kElim : 0) | ((grp + 1) << 2);
            T* A = s_A + static_cast<size_t>(tid) * sA;
            for (int a = 0; a < 6; ++a) {
                A[a] = ok ? L.Jc[a] : T(0);
                A[nA + a] = ok ? L.Jc[6 + a] : T(0);
            }
            for (int a = 0; a < ni; ++a) {
                A[6 + a] = ok ? L.Ji[a] : T(0);
                A[nA + 6 + a] = ok ? L.Ji[kMaxNI + a] : T(0);
            }
            // the observation's gradient -J^T w r (FP64): pose and intrinsic columns
            VT* Dg = s_D + static_cast<size_t>(tid) * sD;
            for (int a = 0; a < 6; ++a) Dg[a] = ok ? Val::make(grad[a]) : Val::zero();
            for (int a = 0; a < ni; ++a) Dg[6 + a] = ok ? Val::make(grad[9 + a]) : Val::zero();
            double* V = s_V + static_cast<size_t>(tid) * 9;
            w64 = L.wd;
            for (int i = 0; i < 6; ++i) jpT[i] = L.Jp[i];
            if (elim && ok) {
                // V_o = w Jp^T Jp from the Jacobian and the point gradient, in FP64
                const double w = L.wd;
                const double j0 = L.Jp[0], j1 = L.Jp[1], j2 = L.Jp[2], j3 = L.Jp[3], j4 = L.Jp[4], j5 = L.Jp[5];
                V[0] = w * (j0 * j0 + j3 * j3);
                V[1] = w * (j0 * j1 + j3 * j4);
                V[2] = w * (j0 * j2 + j3 * j5);
                V[3] = w * (j1 * j1 + j4 * j4);
                V[4] = w * (j1 * j2 + j4 * j5);
                V[5] = w * (j2 * j2 + j5 * j5);
                V[6] = grad[6];
                V[7] = grad[7];
                V[8] = grad[8];
            } else {
                for (int i = 0; i < 9; ++i) V[i] = 0.0;
            }
        }
    }
    // chunk-local track slots: rank of each track's first observation among the chunk's
    // track starts (all lanes of every warp take part: blockDim is a multiple of 32)
    const bool start = active && tid == first;
    const unsigned ballot = __ballot_sync(0xffffffffu, start);
    if (lane == 0) s_wcount[wid] = __popc(ballot);
    // block cost (FP64, fixed order)
    const double cw = warp_sum(cost);
    if (lane == 0) s_misc[wid] = cw;
    __syncthreads();

    // ---- B: track slots; per track FP64 Cholesky V(1+lambda) = R R^T.  R^-1 and q = R^-1 g_p
    // replace the track's first record of s_V (only this thread reads them in this phase).
    int ntc = 0, slot = 0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
        if (w == wid) slot = ntc + __popc(ballot & ((1u << lane) - 1u));
        ntc += s_wcount[w];
    }
    if (ntc > MT) {
        // the host bounds the tracks of a chunk; a larger count would overrun s_K
        if (tid == 0) atomicOr(s_flags, 4);
        ntc = 0;
    }
    if (start) {
        s_trk[tid] = first | (slot << 8) | (k << 16);
        if (slot < MT) {
            s_tfirst[slot] = tid;
            int mask = 0;
            for (int j = first; j < first + k; ++j) {
                const int g = info_group(s_info[j]);
                if (g >= 0) mask |= 1 << g;
            }
            s_tmask[slot] = mask;
        }
    }
    if (tid == 0 && ntc <= MT) s_tfirst[ntc] = nobs;
    __syncthreads();
    // Per track, one thread: track slot t goes to lane t / 4 of warp t % 4 (warps 4-7 for slots
    // 128 and up), so that the FP64 work of the chunk's tracks runs on a few warps spread over
    // the four sub-partitions rather than on scattered lanes of every warp.
    const int tslot = (wid >> 2) * 128 + lane * 4 + (wid & 3);
    const bool tact = tslot < ntc;
    const int tfirst = tact ? s_tfirst[tslot] : 0;
    const int tk = tact ? s_tfirst[tslot + 1] - tfirst : 0;
    const int tobs = obs0 + tfirst;
    const bool telim = tact && (s_info[tfirst] & kElim);
    // control points of the track (linearizeTrack, BundleAdjustPlaMatrixReferenceSchur.cpp:331-346):
    // their cost always, their point terms when the point is eliminated
    double cpV[6] = {0, 0, 0, 0, 0, 0}, cpg[3] = {0, 0, 0};
    if (tact && S.ncp > 0) {
        const int trk = D.obs_trk[tobs];
        const double* X = D.points + static_cast<size_t>(trk) * 3;
        double cc_sum = 0.0;
        for (int q = D.trk_cp_begin[trk]; q < D.trk_cp_begin[trk + 1]; ++q) {
            const double* rec = D.cp_rec + static_cast<size_t>(q) * 12;
            double r[3], cc, cw;
            if (!cp_eval(rec, X[0], X[1], X[2], S.cp_huber, r, cc, cw)) continue;  // not finite: skipped
            cc_sum += cc;
            // accumulatePointOnlyConstraint (:241-260): V += w J^T J, g -= w J^T r, J = sqrt(weight) W
            int e = 0;
            for (int a = 0; a < 3; ++a) {
                for (int b = a; b < 3; ++b)
                    cpV[e++] += cw * (rec[a] * rec[b] + rec[3 + a] * rec[3 + b] + rec[6 + a] * rec[6 + b]);
                cpg[a] -= cw * (rec[a] * r[0] + rec[3 + a] * r[1] + rec[6 + a] * r[2]);
            }
        }
        s_cpc[tslot] = cc_sum;
    }
    if (telim) {
        double V[6] = {cpV[0], cpV[1], cpV[2], cpV[3], cpV[4], cpV[5]}, rhs[3] = {cpg[0], cpg[1], cpg[2]};
        for (int j = 0; j < tk; ++j) {
            const double* v = s_V + static_cast<size_t>(tfirst + j) * 9;
            for (int i = 0; i < 6; ++i) V[i] += v[i];
            for (int i = 0; i < 3; ++i) rhs[i] += v[6 + i];
        }
        V[0] *= 1.0 + damping;
        V[3] *= 1.0 + damping;
        V[5] *= 1.0 + damping;
        // tryInverse3x3 singularity rule: |det| <= 1e-15
        const double det = V[0] * (V[3] * V[5] - V[4] * V[4]) - V[1] * (V[1] * V[5] - V[4] * V[2]) +
                           V[2] * (V[1] * V[4] - V[3] * V[2]);
        double Ri[6] = {0, 0, 0, 0, 0, 0}, q[3] = {0, 0, 0};
        bool singular = !(fabs(det) > 1e-15) || !isfinite(det);
        if (!singular) {
            // Cholesky through reciprocal square roots (no FP64 division on the critical path)
            const double i00 = rsqrt(V[0]);
            const double R10 = V[1] * i00, R20 = V[2] * i00;
            const double a11 = V[3] - R10 * R10;
            const double i11 = rsqrt(a11);
            const double R21 = (V[4] - R20 * R10) * i11;
            const double a22 = V[5] - R20 * R20 - R21 * R21;
            const double i22 = rsqrt(a22);
            if (!(V[0] > 0.0) || !(a11 > 0.0) || !(a22 > 0.0) || !isfinite(i22)) {
                singular = true;
            } else {
                const double i10 = -R10 * i00 * i11;
                const double i21 = -R21 * i11 * i22;
                const double i20 = -(R20 * i00 + R21 * i10) * i22;
                Ri[0] = i00; Ri[1] = i10; Ri[2] = i11; Ri[3] = i20; Ri[4] = i21; Ri[5] = i22;
                q[0] = i00 * rhs[0];
                q[1] = i10 * rhs[0] + i11 * rhs[1];
                q[2] = i20 * rhs[0] + i21 * rhs[1] + i22 * rhs[2];
            }
        }
        if (singular) atomicOr(s_flags, 1);
        double* st = s_V + static_cast<size_t>(tfirst) * 9;
        double* gt = O.trk_data + static_cast<size_t>(D.obs_trk[tobs]) * kTrackRec;
        for (int i = 0; i < 6; ++i) { st[i] = Ri[i]; gt[i] = Ri[i]; }
        for (int i = 0; i < 3; ++i) {
            st[6 + i] = q[i];
            gt[6 + i] = q[i];
            gt[9 + i] = rhs[i];
        }
    }
    __syncthreads();

    // ---- C: per observation, in FP64: Y = w Jp R^-T, M = w I - Y Y^T and Y q; then
    // G = J_pose^T Y (values: float-float on the FP32 path; zero for tracks not eliminated)
    if (active) {
        if (!start) s_trk[tid] = s_trk[first];
        VT* G = s_G + static_cast<size_t>(tid) * sG;
        VT* Ys = s_Y + static_cast<size_t>(tid) * sY;
        VT* Mo = s_M + static_cast<size_t>(tid) * sM;
        if (ok) {
            VT y[6];
            {
                // FP64 from the rounded Jacobian and the weight of phase A
                const double w = w64;
                double Y[2][3] = {{0, 0, 0}, {0, 0, 0}}, q[3] = {0, 0, 0};
                if (elim) {
                    const double* st = s_V + static_cast<size_t>(first) * 9;
                    const double i00 = st[0], i10 = st[1], i11 = st[2], i20 = st[3], i21 = st[4], i22 = st[5];
                    q[0] = st[6]; q[1] = st[7]; q[2] = st[8];
                    for (int pa = 0; pa < 2; ++pa) {
                        const double p0 = jpT[pa * 3], p1 = jpT[pa * 3 + 1], p2 = jpT[pa * 3 + 2];
                        Y[pa][0] = w * (i00 * p0);
                        Y[pa][1] = w * (i10 * p0 + i11 * p1);
                        Y[pa][2] = w * (i20 * p0 + i21 * p1 + i22 * p2);
                    }
                }
                Mo[0] = Val::make(w - (Y[0][0] * Y[0][0] + Y[0][1] * Y[0][1] + Y[0][2] * Y[0][2]));
                Mo[1] = Val::make(-(Y[0][0] * Y[1][0] + Y[0][1] * Y[1][1] + Y[0][2] * Y[1][2]));
                Mo[2] = Val::make(w - (Y[1][0] * Y[1][0] + Y[1][1] * Y[1][1] + Y[1][2] * Y[1][2]));
                Mo[3] = Val::make(Y[0][0] * q[0] + Y[0][1] * q[1] + Y[0][2] * q[2]);
                Mo[4] = Val::make(Y[1][0] * q[0] + Y[1][1] * q[1] + Y[1][2] * q[2]);
                Mo[5] = Val::make(w);
                for (int i = 0; i < 6; ++i) y[i] = Val::make(Y[i / 3][i % 3]);
            }
            for (int i = 0; i < 6; ++i) Ys[i] = y[i];
            const T* A = s_A + static_cast<size_t>(tid) * sA;
            // back-substitution record of the observation: A rows, then Y
            T* rec = O.obs_rec + static_cast<size_t>(o) * (2 * nA + 6);
            for (int i = 0; i < 2 * nA; ++i) rec[i] = A[i];
            for (int i = 0; i < 6; ++i) {
                if constexpr (kMixed) rec[2 * nA + i] = y[i].hi;  // RN of the FP64 value
                else rec[2 * nA + i] = y[i];
            }
            for (int a = 0; a < 6; ++a) {
                const T ja0 = A[a], ja1 = A[nA + a];
                G[a * 3 + 0] = ja0 * y[0] + ja1 * y[3];
                G[a * 3 + 1] = ja0 * y[1] + ja1 * y[4];
                G[a * 3 + 2] = ja0 * y[2] + ja1 * y[5];
            }
        } else {
            T* rec = O.obs_rec + static_cast<size_t>(o) * (2 * nA + 6);
            for (int i = 0; i < 2 * nA + 6; ++i) rec[i] = T(0);
            for (int i = 0; i < 6; ++i) Mo[i] = Val::zero();
            for (int i = 0; i < 6; ++i) Ys[i] = Val::zero();
            for (int i = 0; i < 18; ++i) G[i] = Val::zero();
        }
    }
    __syncthreads();
    // ---- K: per track and group, K[(g, c), k] = sum_(o in track, group g) (J_intr^T Y)[c, k]
    if (nb > 0) {
        const int per = nb * 3;
        for (int it = tid; it < ntc * per; it += blockDim.x) {
            const int t = it / per, r = it - t * per;
            const int gc = r / 3, kk = r - gc * 3;
            const int g = gc / ni, c = gc - g * ni;
            VT acc = Val::zero();
            for (int ob = s_tfirst[t]; ob < s_tfirst[t + 1]; ++ob) {
                if (info_group(s_info[ob]) != g) continue;
                const T* A = s_A + static_cast<size_t>(ob) * sA;
                const VT* Y = s_Y + static_cast<size_t>(ob) * sY;
                acc = acc + (A[6 + c] * Y[kk] + A[nA + 6 + c] * Y[3 + kk]);
            }
            s_K[static_cast<size_t>(t) * sK + r] = acc;
        }
        __syncthreads();
    }

    // ---- D: owner gathers over [pose block rows | camera rows | intrinsic entries]
    const int pair0 = D.ch_pair_begin[chunk], npairs = D.ch_pair_begin[chunk + 1] - pair0;
    const int cam0 = D.ch_cam_begin[chunk], ncams = D.ch_cam_begin[chunk + 1] - cam0;
    const int camrec = 12 + ng * 6 * ni;
    const int crow = 2 + ng * ni;  // rows of a camera record: rhs, direct rhs, border (g, c)
    const int chrec = nb * nb + 2 * nb;
    const int w_pair = npairs * 6, w_cam = ncams * crow;
    // host-built schedule (schedule_owner_tasks, pb_host.cpp): this warp's rounds of 32 tasks,
    // dealt to the warps by longest processing time
    const int task_end = D.warp_task_begin[chunk * kAssembleWarps + wid + 1];
    for (int pos = D.warp_task_begin[chunk * kAssembleWarps + wid] + lane; pos < task_end; pos += 32) {
        const int wk = D.task_list[pos];
        if (wk == kNoTask) continue;
        if (wk < w_pair) {
            // row x of the pose block of chunk pair slot s
            const int s = wk / 6, x = wk - s * 6;
            const int pk = D.ch_pairs[pair0 + s];
            const bool diag = (pk & 0xFFFF) == (pk >> 16);
            Acc<T> acc[6];
            const int i1 = D.slot_item_begin[pair0 + s + 1];
            for (int it = D.slot_item_begin[pair0 + s]; it < i1; ++it) {
                const unsigned item = D.slot_items[it];
                const int oa = item & 0xFF, ob = item >> 8;
                if (oa == ob) {
                    // own term: row x of J^T M J
                    const T* A = s_A + static_cast<size_t>(oa) * sA;
                    const VT* M = s_M + static_cast<size_t>(oa) * sM;
                    const T ax0 = A[x], ax1 = A[nA + x];
                    const VT u0 = ax0 * M[0] + ax1 * M[1];
                    const VT u1 = ax0 * M[1] + ax1 * M[2];
#pragma unroll
                    for (int y = 0; y < 6; ++y) {
                        acc_fma(acc[y], A[y], u0);
                        acc_fma(acc[y], A[nA + y], u1);
                    }
                } else {
                    const VT* Ga = s_G + static_cast<size_t>(oa) * sG + 3 * x;
                    const VT* Gb = s_G + static_cast<size_t>(ob) * sG;
                    const VT g0 = -Ga[0], g1 = -Ga[1], g2 = -Ga[2];
#pragma unroll
                    for (int y = 0; y < 6; ++y) {
                        acc_fma(acc[y], g0, Gb[3 * y]);
                        acc_fma(acc[y], g1, Gb[3 * y + 1]);
                        acc_fma(acc[y], g2, Gb[3 * y + 2]);
                    }
                }
            }
            P* out = O.part_pair + static_cast<size_t>(pair0 + s) * 36;
#pragma unroll
            for (int y = 0; y < 6; ++y) {
                if (!diag) {
                    out[x * 6 + y] = acc[y].part();
                } else if (y >= x) {
                    out[x * 6 + y] = acc[y].part();
                    out[y * 6 + x] = acc[y].part();
                }
            }
        } else if (wk < w_pair + w_cam) {
            const int r = wk - w_pair;
            const int l = r / crow, row = r - l * crow;
            const int b0 = D.lcam_obs_begin[cam0 + l], b1 = D.lcam_obs_begin[cam0 + l + 1];
            P* out = O.part_cam + static_cast<size_t>(cam0 + l) * camrec;
            Acc<T> acc[6];
            if (row < 2) {
                // gradient rows: the reduced gradient -J_pose^T (w r + Y q) and the direct
                // gradient -J_pose^T w r (the point term with the rounded Jacobian)
                for (int it = b0; it < b1; ++it) {
                    const int ob = D.lcam_obs[it];
                    const VT* Dg = s_D + static_cast<size_t>(ob) * sD;
#pragma unroll
                    for (int a = 0; a < 6; ++a) acc[a].add(Dg[a]);
                    if (row == 0) {
                        const T* A = s_A + static_cast<size_t>(ob) * sA;
                        const VT* M = s_M + static_cast<size_t>(ob) * sM;
                        const VT m0 = -M[3], m1 = -M[4];
#pragma unroll
                        for (int a = 0; a < 6; ++a) {
                            acc_fma(acc[a], A[a], m0);
                            acc_fma(acc[a], A[nA + a], m1);
                        }
                    }
                }
#pragma unroll
                for (int a = 0; a < 6; ++a) out[row * 6 + a] = acc[a].part();
            } else {
                // border column (g, c2) of the camera's pose rows
                const int gc = row - 2, g = gc / ni, c2 = gc - g * ni;
                for (int it = b0; it < b1; ++it) {
                    const int ob = D.lcam_obs[it];
                    const int info = s_info[ob];
                    const T* A = s_A + static_cast<size_t>(ob) * sA;
                    if (info_group(info) == g) {
                        const VT w = s_M[static_cast<size_t>(ob) * sM + 5];
                        const VT u0 = A[6 + c2] * w, u1 = A[nA + 6 + c2] * w;
#pragma unroll
                        for (int a = 0; a < 6; ++a) {
                            acc_fma(acc[a], A[a], u0);
                            acc_fma(acc[a], A[nA + a], u1);
                        }
                    }
                    const int ts = trk_slot(s_trk[ob]);
                    if ((info & kElim) && ts < ntc && ((s_tmask[ts] >> g) & 1)) {
                        const VT* Kt = s_K + static_cast<size_t>(ts) * sK + gc * 3;
                        const VT k0 = -Kt[0], k1 = -Kt[1], k2 = -Kt[2];
                        const VT* Go = s_G + static_cast<size_t>(ob) * sG;
#pragma unroll
                        for (int a = 0; a < 6; ++a) {
                            acc_fma(acc[a], Go[3 * a], k0);
                            acc_fma(acc[a], Go[3 * a + 1], k1);
                            acc_fma(acc[a], Go[3 * a + 2], k2);
                        }
                    }
                }
#pragma unroll
                for (int a = 0; a < 6; ++a) out[12 + (g * 6 + a) * ni + c2] = acc[a].part();
            }
        }
    }
    // Intrinsic block entries (i, j), i <= j, and intrinsic gradient entries: one warp per entry,
    // its lanes striding over the chunk's observations and tracks, then a fixed shuffle tree (the
    // entries sum over every observation of the chunk, so a thread per entry would be the
    // chunk's critical path).  Warps that finish their rows above start here at once.
    {
        P* out = O.part_chunk + static_cast<size_t>(chunk) * chrec;
        // a warp takes the next entry when it is free (an entry is summed the same way by any
        // warp, so the order of taking changes no result)
        for (;;) {
            int e = 0;
            if (lane == 0) e = atomicAdd(s_next_entry, 1);
            e = __shfl_sync(0xffffffffu, e, 0);
            if (e >= chrec) break;
            Acc<T> acc;
            if (e < nb * nb) {
                const int i = e / nb, j = e - i * nb;
                if (i > j) continue;
                const int g1 = i / ni, c1 = i - g1 * ni, g2 = j / ni, c2 = j - g2 * ni;
                if (g1 == g2) {
                    for (int ob = lane; ob < nobs; ob += 32) {
                        if (info_group(s_info[ob]) != g1) continue;
                        const T* A = s_A + static_cast<size_t>(ob) * sA;
                        const VT w = s_M[static_cast<size_t>(ob) * sM + 5];
                        acc_fma(acc, w, two_prod(A[6 + c1], A[6 + c2]));
                        acc_fma(acc, w, two_prod(A[nA + 6 + c1], A[nA + 6 + c2]));
                    }
                }
                const int need = (1 << g1) | (1 << g2);
                for (int t = lane; t < ntc; t += 32) {
                    if ((s_tmask[t] & need) != need) continue;
                    const VT* K1 = s_K + static_cast<size_t>(t) * sK + i * 3;
                    const VT* K2 = s_K + static_cast<size_t>(t) * sK + j * 3;
                    acc_fma(acc, -K1[0], K2[0]);
                    acc_fma(acc, -K1[1], K2[1]);
                    acc_fma(acc, -K1[2], K2[2]);
                }
                warp_merge(acc);
                if (lane == 0) {
                    out[e] = acc.part();
                    if (i != j) out[j * nb + i] = acc.part();
                }
            } else {
                const int idx = e - nb * nb;
                const bool reduced = idx < nb;
                const int col = reduced ? idx : idx - nb;
                const int g = col / ni, c = col - g * ni;
                for (int ob = lane; ob < nobs; ob += 32) {
                    if (info_group(s_info[ob]) != g) continue;
                    acc.add(s_D[static_cast<size_t>(ob) * sD + 6 + c]);
                    if (reduced) {
                        const T* A = s_A + static_cast<size_t>(ob) * sA;
                        const VT* M = s_M + static_cast<size_t>(ob) * sM;
                        acc_fma(acc, A[6 + c], -M[3]);
                        acc_fma(acc, A[nA + 6 + c], -M[4]);
                    }
                }
                warp_merge(acc);
                if (lane == 0) out[e] = acc.part();
            }
        }
    }
    if (tid == 0) {
        double c = 0.0;
        for (int w = 0; w < static_cast<int>((blockDim.x + 31) >> 5); ++w) c += s_misc[w];
        if (S.ncp > 0)
            for (int t = 0; t < ntc; ++t) c += s_cpc[t];
        O.part_cost[chunk] = c;
        O.part_flags[chunk] = s_flags[0];
    }
}

template <typename T>
static AsmOutT<T> typed_out(const AsmOut& o) {
    using P = typename Acc<T>::part_type;
    return {static_cast<P*>(o.part_pair_v), static_cast<P*>(o.part_cam_v), static_cast<P*>(o.part_chunk_v),
            o.part_cost, o.part_flags, static_cast<double*>(o.trk_data_v), static_cast<T*>(o.obs_rec_v)};
}

// 256 threads per chunk whatever its observation count (at most 256): threads beyond the chunk's
// observations idle in phases A-C and take their share of the gathers of phase D.
constexpr int kAssembleThreads = 256;
static_assert(kAssembleThreads == 32 * kAssembleWarps, "the owner-gather schedule is planned for 8 warps");

template <typename T>
void launch_assemble(const Shape& S, const DevPtrs& D, const AsmOut& O, double damping, size_t smem, cudaStream_t st) {
    if (S.nchunks == 0) return;
    k_assemble<T><<<S.nchunks, kAssembleThreads, smem, st>>>(S, D, typed_out<T>(O), damping);
}

void pb_set_assemble_smem_f32(size_t bytes) {
    cudaFuncSetAttribute(k_assemble<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}
void pb_set_assemble_smem_f64(size_t bytes) {
    cudaFuncSetAttribute(k_assemble<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

template void launch_assemble<float>(const Shape&, const DevPtrs&, const AsmOut&, double, size_t, cudaStream_t);
template void launch_assemble<double>(const Shape&, const DevPtrs&, const AsmOut&, double, size_t, cudaStream_t);

}  // namespace pb
